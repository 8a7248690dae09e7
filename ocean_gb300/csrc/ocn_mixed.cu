// ocn_mixed.cu -- mixed-precision long-range term of the BSE action
// (long_range.f90:873-963 restated for tensor cores), for a block of nv psi
// vectors that share H:
//
//   phi(k,x,v,a)  = sum_n u(n,k,x) q_v(n,k,a),     q = allow o psi_v     [tcgen05, split-BF16]
//   phi'(.,x,v,a) = FFT_fwd[ W(.,x) o FFT_bwd[phi(.,x,v,a)] ] / Nk            [FP32, shared memory]
//   part(n,k,v,a) = - sum_x conj(u(n,k,x)) phi'(k,x,v,a)                    [tcgen05, split-BF16]
//
// Split-BF16: every FP32 operand value is stored as hi = bf16(v), lo =
// bf16(v - hi); the MMAs accumulate (A_hi + A_lo)(B_hi + B_lo) in FP32 in tensor
// memory, which keeps ~16 significant bits of every product.
//
// Complex arithmetic is made real by stacking re/im along K (K = (c, n) for the
// band contraction, K = (c, x) for the x-mesh contraction) and by the output
// columns j = v*4Na + (split s)*2Na + (part re/im)*Na + alpha: D[:, j] +
// D[:, j + 2Na] is the full product.  MMA shape: M = 128 rows, N = 4 Na nvmax,
// K = 16 per instruction.  Every byte of u2 read from HBM serves all nv vectors.
//
// Operands live in HBM as bf16 tiles read by TMA:
//   UA_s [k][x][K1]  (K1 = 2 Nb)      A of the band -> x contraction, built once
//   UB_s [k][K2/64][n][64]            A of the x -> band contraction, built once, chunk-major
//                                     (each 128-band x 64 TMA box is one contiguous run)
//   B1   [k][j][K1]                   psi operand, rebuilt per action
//   B2   [k][K2][j]                   phi' operand, MN-major, written by the k-mesh transform
// with K2 = (x/64)*128 + c*64 + x%64 (both c halves of a 64-x block in consecutive
// 64-wide K chunks).  A operands and B1 are K-major with 128-byte swizzling; B2 is
// read in 16-column boxes with 32-byte swizzling.
// The GEMM kernel is persistent and warp-specialised: warp 0 issues TMA loads,
// warp 1 issues tcgen05.mma and owns the tensor-memory allocation, warps 2-5 drain
// the double-buffered accumulator.  Every mbarrier wait is bounded in time; on
// expiry the kernel records an error, drains what it issued, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>

#include "ocn_df.cuh"
#include "ocn_internal.h"
#include "ocn_kmesh_dft.cuh"

namespace ocn {

namespace {

constexpr int TC_MAX_STAGES = 4;
constexpr int TC_BM = 128;
constexpr int TC_BK = 64;  // bf16 elements per 128-byte swizzle row
constexpr int TC_THREADS = 192;
constexpr int TC_MAX_NCOL = 256;  // MMA N limit for M = 128
constexpr long long TC_WAIT_CYCLES = 2000000000LL;  // ~1 s at 2 GHz
constexpr size_t TC_SMEM_BUDGET = 220 * 1024;


struct TcParams {
  int mode;      // 1: band -> x (GEMM1), 2: x -> band (GEMM2)
  int ntiles;
  int nb, nk, nx, na;
  int ncol;      // MMA N = 4 Na nvmax
  int nv;        // vectors whose outputs are written
  int stages;    // shared-memory pipeline depth (<= TC_MAX_STAGES)
  int nch;       // K chunks of the full reduction
  int nxt;       // mode 1: x tiles per k
  int mt2, ks2, cps2;  // mode 2: M tiles, K splits, chunks per split
  int nvmax;     // partial-buffer vector stride
  uint32_t idesc;
  uint32_t tcols;
  float2* phi;   // mode 1 output [k][x][v*Na + a]
  float* part;   // mode 2 output [split][v][re|im][npsi] (binary32: the accumulator's own precision)
  size_t npsi;
  int* err;
  int bshared;   // B operand has one k slice shared by every k (multiplet back-projection)
  int koff;      // added to k for the A operand: spin s of a spin-polarised problem at s*Nk
  int spin;      // -1: write every alpha; 0/1: only alpha with alpha mod 2 == spin
  int estg;      // launch-wide: mode-1 outputs staged per warp in shared memory, stored coalesced
  int starve;    // launch-wide test hook: the producer issues no loads, so the MMA warp's
                 // first bounded wait runs out with nothing in flight (OCN_ERR_TIMEOUT path)
  int bmn;       // B is MN-major in SW32 boxes of 16 columns by 64 K rows (B2 of the x -> band contraction)
  int achunk;    // A is stored chunk-major, [k][K chunk][row][64] (UB): every A box is one contiguous run
  int* inc;      // launch-wide: non-null, block 0 adds 1 to it (the Haydock iteration counter; saves a launch)
};

// Tensor maps of a group launch (kernel parameter space, 384 bytes per problem).
constexpr int TC_GROUP_MAX = 64;
struct TcGroupMaps {
  CUtensorMap m[TC_GROUP_MAX][3];  // A hi, A lo, B
};

__device__ __forceinline__ uint32_t su32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the time limit passed or another role aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          long long limit) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0,
                                            int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// K-major operand tile with 128-byte swizzling: rows of 128 bytes, 8-row core
// groups 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// MN-major operand tile with 32-byte swizzling, as TMA writes boxes of 64 K-rows
// by 16 MN-elements (32 bytes): 8-row K groups 256 bytes apart (stride byte
// offset), consecutive 16-element MN atoms 2048 bytes apart (leading byte offset).
__device__ __forceinline__ uint64_t sw32_mn_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(2048 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)6 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct TileInfo {
  int k, row0, c0, c1, mt, sp;
};

__device__ __forceinline__ TileInfo decode(const TcParams& p, int t) {
  TileInfo ti;
  if (p.mode == 1) {
    ti.k = t / p.nxt;
    ti.row0 = (t % p.nxt) * TC_BM;
    ti.c0 = 0;
    ti.c1 = p.nch;
    ti.mt = 0;
    ti.sp = 0;
  } else {
    const int per_k = p.mt2 * p.ks2;
    ti.k = t / per_k;
    const int r = t % per_k;
    ti.mt = r / p.ks2;
    ti.sp = r % p.ks2;
    ti.row0 = ti.mt * TC_BM;
    ti.c0 = ti.sp * p.cps2;
    ti.c1 = min(p.nch, ti.c0 + p.cps2);
  }
  return ti;
}

// Operand source of one launch: one problem (three tensor maps and p), or a
// group of problems whose tile lists are concatenated (instance i owns tiles
// tile0[i] .. tile0[i+1]-1 and has its own tensor maps and parameters).  The
// per-tile work is the same either way.
struct TcSingle {
  const CUtensorMap *h, *l, *b;
  const TcParams* p;
  __device__ __forceinline__ int inst(int t, int* lt) const {
    *lt = t;
    return 0;
  }
  __device__ __forceinline__ const TcParams& par(int) const { return *p; }
  __device__ __forceinline__ const CUtensorMap* map(int, int w) const { return w == 0 ? h : (w == 1 ? l : b); }
};
struct TcGroup {
  const TcGroupMaps* maps;
  const TcParams* tab;
  const int* tile0;
  int n;
  __device__ __forceinline__ int inst(int t, int* lt) const {
    int lo = 0, hi = n - 1;  // the last instance whose first tile is <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile0[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    *lt = t - tile0[lo];
    return lo;
  }
  __device__ __forceinline__ const TcParams& par(int i) const { return tab[i]; }
  __device__ __forceinline__ const CUtensorMap* map(int i, int w) const { return &maps->m[i][w]; }
};

// p: launch-wide values (tile count, pipeline depth, shared-memory stage layout
// and accumulator stride for the largest N, tensor-memory columns, error flag).
template <class Src>
__device__ __forceinline__ void lr_tc_body(const TcParams& p, const Src& src) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  const uint32_t a_bytes = TC_BM * TC_BK * 2;
  const uint32_t b_bytes = (uint32_t)p.ncol * TC_BK * 2;
  const uint32_t stage_bytes = 2 * a_bytes + b_bytes;
  const int S = p.stages;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * stage_bytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * TC_MAX_STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const uint32_t full0 = su32(bars), empty0 = su32(bars + TC_MAX_STAGES);
  const uint32_t tfull0 = su32(bars + 2 * TC_MAX_STAGES), tempty0 = su32(bars + 2 * TC_MAX_STAGES + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (p.inc && blockIdx.x == 0 && threadIdx.x == 0) *p.inc += 1;  // nothing in this launch reads it
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, 128);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(p.tcols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------------ producer
      uint32_t stage = 0, phase = 0;
      int armed_phase[TC_MAX_STAGES];
      for (int s = 0; s < TC_MAX_STAGES; ++s) armed_phase[s] = -1;
      bool ok = true;
      for (int t = blockIdx.x; t < p.ntiles && ok && !p.starve; t += gridDim.x) {
        int lt;
        const int ii = src.inst(t, &lt);
        const TcParams& tp = src.par(ii);
        const TileInfo ti = decode(tp, lt);
        for (int c = ti.c0; c < ti.c1; ++c) {
          if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, TC_WAIT_CYCLES)) {
            ok = false;
            break;
          }
          const uint32_t sbase = su32(smem + stage * stage_bytes);
          mbar_expect_tx(full0 + 8 * stage, 2 * a_bytes + (uint32_t)tp.ncol * TC_BK * 2);
          if (tp.achunk) {  // (K in chunk, row, chunk, k)
            tma_load_4d(sbase, src.map(ii, 0), full0 + 8 * stage, 0, ti.row0, c, ti.k + tp.koff);
            tma_load_4d(sbase + a_bytes, src.map(ii, 1), full0 + 8 * stage, 0, ti.row0, c, ti.k + tp.koff);
          } else {
            tma_load_3d(sbase, src.map(ii, 0), full0 + 8 * stage, c * TC_BK, ti.row0, ti.k + tp.koff);
            tma_load_3d(sbase + a_bytes, src.map(ii, 1), full0 + 8 * stage, c * TC_BK, ti.row0, ti.k + tp.koff);
          }
          if (tp.bmn) {
            for (int j = 0; j < tp.ncol / 16; ++j)
              tma_load_3d(sbase + 2 * a_bytes + j * 2048, src.map(ii, 2), full0 + 8 * stage, 16 * j, c * TC_BK, ti.k);
          } else {
            tma_load_3d(sbase + 2 * a_bytes, src.map(ii, 2), full0 + 8 * stage, c * TC_BK, 0, tp.bshared ? 0 : ti.k);
          }
          armed_phase[stage] = (int)phase;
          if (++stage == (uint32_t)S) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      if (!ok) {
        *abort_flag = 1;
        atomicOr(p.err, 1);
      }
      // drain: never leave a TMA write in flight
      for (int s = 0; s < S; ++s)
        if (armed_phase[s] >= 0) {
          const long long t0 = clock64();
          while (!mbar_test(full0 + 8 * s, (uint32_t)armed_phase[s]) &&
                 clock64() - t0 < TC_WAIT_CYCLES) {
          }
        }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------------ MMA issuer
      uint32_t stage = 0, phase = 0, acc = 0, acc_phase = 0;
      int last_stage = -1;
      uint32_t last_phase = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
        int lt;
        const int ii = src.inst(t, &lt);
        const TcParams& tp = src.par(ii);
        const TileInfo ti = decode(tp, lt);
        if (!mbar_wait(tempty0 + 8 * acc, acc_phase ^ 1, abort_flag, TC_WAIT_CYCLES)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dt = tmem_base + acc * (uint32_t)p.ncol;
        for (int c = ti.c0; c < ti.c1; ++c) {
          if (!mbar_wait(full0 + 8 * stage, phase, abort_flag, TC_WAIT_CYCLES)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = su32(smem + stage * stage_bytes);
#pragma unroll
          for (int kk = 0; kk < TC_BK / 16; ++kk) {
            const uint64_t bd =
                tp.bmn ? sw32_mn_desc(sa + 2 * a_bytes + kk * 512) : sw128_desc(sa + 2 * a_bytes + kk * 32);
            umma_bf16(dt, sw128_desc(sa + kk * 32), bd, tp.idesc, (c > ti.c0 || kk > 0) ? 1u : 0u);
            umma_bf16(dt, sw128_desc(sa + a_bytes + kk * 32), bd, tp.idesc, 1u);
          }
          umma_commit(empty0 + 8 * stage);
          last_stage = (int)stage;
          last_phase = phase;
          if (++stage == (uint32_t)S) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        umma_commit(tfull0 + 8 * acc);
        acc ^= 1;
        if (acc == 0) acc_phase ^= 1;
      }
      if (!ok) {
        *abort_flag = 1;
        atomicOr(p.err, 2);
      }
      if (last_stage >= 0) {  // drain: every issued MMA finished reading shared memory
        const long long t0 = clock64();
        while (!mbar_test(empty0 + 8 * last_stage, last_phase) && clock64() - t0 < TC_WAIT_CYCLES) {
        }
      }
    }
  } else {
    // -------------------------------------------------------------- epilogue
    const int q = warp & 3;  // TMEM lane quadrant this warp may access
    const int row = q * 32 + lane;
    uint32_t acc = 0, acc_phase = 0;
    float v[48];  // one vector's 4 Na columns
    // mode-1 staging: this warp's 32 rows of (vector, alpha) values, row pitch wld
    const int wld = p.ncol / 4 + 1;
    float2* wst = reinterpret_cast<float2*>(smem + S * stage_bytes + 256) + (size_t)(warp - 2) * 32 * wld;
    for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
      int lt;
      const int ii = src.inst(t, &lt);
      const TcParams& tp = src.par(ii);
      const TileInfo ti = decode(tp, lt);
      const int na = tp.na, g4 = 4 * na;
      if (!mbar_wait(tfull0 + 8 * acc, acc_phase, abort_flag, TC_WAIT_CYCLES)) {
        *abort_flag = 1;
        atomicOr(p.err, 4);
        break;
      }
      tc_fence_after();
      const uint32_t ta = tmem_base + ((uint32_t)(q * 32) << 16) + acc * (uint32_t)p.ncol;
      for (int vv = 0; vv < tp.nv; ++vv) {
        for (int c16 = 0; c16 < g4; c16 += 16) tmem_ld16(ta + vv * g4 + c16, v + c16);
        tmem_ld_wait();
        if (tp.mode == 1) {
          const int x = ti.row0 + row;
          if (p.estg && tp.spin < 0) {
            float2* wr = wst + lane * wld + vv * na;
            for (int a = 0; a < na; ++a) wr[a] = make_float2(v[a] + v[2 * na + a], v[na + a] + v[3 * na + a]);
          } else if (x < tp.nx) {
            float2* o = tp.phi + ((size_t)ti.k * tp.nx + x) * (tp.nv * na) + vv * na;
            for (int a = 0; a < na; ++a)
              if (tp.spin < 0 || (a & 1) == tp.spin)
                o[a] = make_float2(v[a] + v[2 * na + a], v[na + a] + v[3 * na + a]);
          }
        } else {
          const int n = ti.row0 + row;
          if (n < tp.nb) {
            float* pr = tp.part + ((size_t)ti.sp * tp.nvmax + vv) * 2 * tp.npsi;
            float* pim = pr + tp.npsi;
            for (int a = 0; a < na; ++a) {
              if (tp.spin >= 0 && (a & 1) != tp.spin) continue;
              const size_t idx = (size_t)n + (size_t)tp.nb * ((size_t)ti.k + (size_t)tp.nk * a);
              pr[idx] = -(v[a] + v[2 * na + a]);
              pim[idx] = -(v[na + a] + v[3 * na + a]);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(tempty0 + 8 * acc);
      if (tp.mode == 1 && p.estg && tp.spin < 0) {
        // the warp's rows are one contiguous run of phi: consecutive lanes store
        // consecutive values
        __syncwarp();
        const int nt = tp.nv * na;
        const int r0 = ti.row0 + q * 32;
        const int rows = min(32, tp.nx - r0);
        if (rows > 0) {
          float2* dst = tp.phi + ((size_t)ti.k * tp.nx + r0) * nt;
          const int dr = 32 / nt, dc = 32 - dr * nt;  // (row, column) step of 32 elements
          int r = lane / nt, cc = lane - r * nt;
          for (int e = lane; e < rows * nt; e += 32) {
            dst[e] = wst[r * wld + cc];
            r += dr;
            cc += dc;
            if (cc >= nt) {
              cc -= nt;
              ++r;
            }
          }
        }
        __syncwarp();
      }
      acc ^= 1;
      if (acc == 0) acc_phase ^= 1;
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(p.tcols)
                 : "memory");
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_lr_tc(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
            const __grid_constant__ CUtensorMap tm_b, const __grid_constant__ TcParams p) {
  const TcSingle src{&tm_hi, &tm_lo, &tm_b, &p};
  lr_tc_body(p, src);
}

// All tiles of up to TC_GROUP_MAX problems in one persistent launch.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_lr_tc_group(const __grid_constant__ TcGroupMaps maps, const __grid_constant__ TcParams p,
                  const TcParams* __restrict__ tab, const int* __restrict__ tile0, int n) {
  const TcGroup src{&maps, tab, tile0, n};
  lr_tc_body(p, src);
}

// ---------------------------------------------------------- operand builders

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}
// two BF16 values as one 32-bit word, a at the lower address
__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// UA_s[k][x][K1]: K < Nb -> Re u(n=K), else Im u(n=K-Nb)   (from u [x][k][n])
__global__ void k_build_ua(const double2* __restrict__ u, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo, int nb, int nk, int nx, int p1) {
  const long long total = (long long)nk * nx * 2 * nb;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(i % (2 * nb));
    const long long r = i / (2 * nb);
    const int x = (int)(r % nx);
    const int k = (int)(r / nx);
    const int n = K < nb ? K : K - nb;
    const double2 z = u[((size_t)x * nk + k) * nb + n];
    const float v = (float)(K < nb ? z.x : z.y);
    __nv_bfloat16 h, l;
    split_bf16(v, h, l);
    const size_t o = ((size_t)k * nx + x) * p1 + K;
    hi[o] = h;
    lo[o] = l;
  }
}

// UB_s[k][j][n][K2 % 64], chunk j = K2 / 64 with K2 = (x/64)*128 + c*64 + x%64 -> Re u(n, x)
// (c = 0), Im u(n, x) (c = 1): chunk-major, so a 128-band x 64 box is contiguous.  The
// padding of a partial last 64-x block is never written (zero since allocation).
__global__ void k_build_ub(const double2* __restrict__ u, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo, int nb, int nk, int nx, int p2) {
  const long long total = (long long)nk * nb * 2 * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(i % (2 * nx));
    const long long r = i / (2 * nx);
    const int n = (int)(r % nb);
    const int k = (int)(r / nb);
    const int x = K < nx ? K : K - nx;
    const double2 z = u[((size_t)x * nk + k) * nb + n];
    const float v = (float)(K < nx ? z.x : z.y);
    __nv_bfloat16 h, l;
    split_bf16(v, h, l);
    const int K2 = ((x >> 6) << 7) + (K < nx ? 0 : 64) + (x & 63);
    const size_t o = (((size_t)k * (p2 >> 6) + (K2 >> 6)) * nb + n) * 64 + (K2 & 63);
    hi[o] = h;
    lo[o] = l;
  }
}

// B1[k][v*4Na + j][K1], j = s*2Na + part*Na + a, from q = allow o psi_v:
//   part 0 (Re phi): K=(0,n) -> qr, K=(1,n) -> -qi;  part 1 (Im phi): (0,n) -> qi, (1,n) -> qr
// Vector v of the block starts at pr + v*vstride (imaginary plane at +npsi).
__global__ void k_prep_b1(const double* __restrict__ pr, const double* __restrict__ pi, size_t vstride,
                          int nv, const double* __restrict__ allow, __nv_bfloat16* __restrict__ b1,
                          int nb, int nk, int na, int ncol, int p1) {
  const int total = nv * nk * 2 * nb;
  const int g4 = 4 * na;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int K = i % (2 * nb);
    const int k = (i / (2 * nb)) % nk;
    const int vv = i / (2 * nb * nk);
    const int c = K < nb ? 0 : 1;
    const int n = K - c * nb;
    const double* vr = pr + (size_t)vv * vstride;
    const double* vi = pi + (size_t)vv * vstride;
    __nv_bfloat16* base = b1 + (size_t)k * ncol * p1 + (size_t)vv * g4 * p1 + K;
    for (int a = 0; a < na; ++a) {
      const size_t idx = (size_t)n + (size_t)nb * ((size_t)k + (size_t)nk * a);
      const double m = allow[idx];
      const float qr = (float)(vr[idx] * m), qi = (float)(vi[idx] * m);
      const float v0 = c == 0 ? qr : -qi;
      const float v1 = c == 0 ? qi : qr;
      __nv_bfloat16 h0, l0, h1, l1;
      split_bf16(v0, h0, l0);
      split_bf16(v1, h1, l1);
      base[(size_t)(a)*p1] = h0;
      base[(size_t)(na + a) * p1] = h1;
      base[(size_t)(2 * na + a) * p1] = l0;
      base[(size_t)(3 * na + a) * p1] = l1;
    }
  }
}

// Multiplet amplitude operand MA[k][p][K1]: K < Nb -> Re mpc(p, n=K, k), else
// Im mpc(p, n=K-Nb, k) -- the layout of UA with the projector p in place of x,
// so amp(p, a) = sum_{k,n} mpc q (OCEAN_multiplet.f90:1730-1783) is the band->x
// contraction against the same psi operand B1, summed over k afterwards.
__global__ void k_build_ma(const double2* __restrict__ mpc, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo, int nb, int nk, int np, int p1) {
  const long long total = (long long)nk * np * 2 * nb;
  const size_t nbk = (size_t)nb * nk;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(i % (2 * nb));
    const long long r = i / (2 * nb);
    const int p = (int)(r % np);
    const int k = (int)(r / np);
    const int n = K < nb ? K : K - nb;
    const double2 z = mpc[(size_t)p * nbk + (size_t)k * nb + n];
    __nv_bfloat16 h, l;
    split_bf16((float)(K < nb ? z.x : z.y), h, l);
    const size_t o = ((size_t)k * np + p) * p1 + K;
    hi[o] = h;
    lo[o] = l;
  }
}

// Back-projection operand MB[k][n][K3]: K3 < Np -> Re mpc(p=K3, n, k), else
// Im mpc(p=K3-Np, n, k) -- the layout of UB with p in place of x, so that
// acc(n,k,a) += sum_p conj(mpc) hamp (OCEAN_multiplet.f90:1943-1998) is the
// x->band contraction against B3 built from hamp.
__global__ void k_build_mb(const double2* __restrict__ mpc, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo, int nb, int nk, int np, int p3) {
  const long long total = (long long)nk * nb * 2 * np;
  const size_t nbk = (size_t)nb * nk;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int K = (int)(i % (2 * np));
    const long long r = i / (2 * np);
    const int n = (int)(r % nb);
    const int k = (int)(r / nb);
    const int p = K < np ? K : K - np;
    const double2 z = mpc[(size_t)p * nbk + (size_t)k * nb + n];
    __nv_bfloat16 h, l;
    split_bf16((float)(K < np ? z.x : z.y), h, l);
    const size_t o = ((size_t)k * nb + n) * p3 + K;
    hi[o] = h;
    lo[o] = l;
  }
}

// amp[v][p][a] = sum_k amp_part[k][p][v*Na + a], summed in double-float: a CTA owns
// 32 consecutive (p, t) outputs (coalesced along t) and its AMP_KGROUPS warps
// split the k range (warp w takes k = w, w + AMP_KGROUPS, ...); warp 0 adds
// the group partials in order (deterministic).
constexpr int AMP_KGROUPS = 32;
__global__ void __launch_bounds__(32 * AMP_KGROUPS)
    k_amp_reduce_f32(const float2* __restrict__ part, double2* __restrict__ amp, int nk, int np, int na, int nv) {
  __shared__ float4 sh[AMP_KGROUPS][32];  // double-float (re h, re l, im h, im l)
  const int nt = na * nv;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  df sr{0.0f, 0.0f}, si{0.0f, 0.0f};  // exact sums of the binary32 terms to ~48 bits, on the FP32 pipe
  if (i < np * nt)
    for (int k = w; k < nk; k += AMP_KGROUPS) {
      const float2 f = part[(size_t)k * np * nt + i];
      sr = df_add(sr, f.x);
      si = df_add(si, f.y);
    }
  sh[w][lane] = make_float4(sr.h, sr.l, si.h, si.l);
  __syncthreads();
  if (w == 0 && i < np * nt) {
    df tr{0.0f, 0.0f}, ti{0.0f, 0.0f};
    for (int g = 0; g < AMP_KGROUPS; ++g) {
      const float4 q = sh[g][lane];
      tr = df_add(tr, df{q.x, q.y});
      ti = df_add(ti, df{q.z, q.w});
    }
    const int p = i / nt, t = i % nt;
    const int v = t / na, a = t % na;
    amp[((size_t)v * np + p) * na + a] = make_double2(df_value(tr), df_value(ti));
  }
}

// B3[v*4Na + j][K3] from h = -hamp[v][p][a] (the x->band epilogue negates):
//   part 0: K=(0,p) -> Re h, K=(1,p) -> Im h;  part 1: (0,p) -> Im h, (1,p) -> -Re h
__global__ void k_prep_b3(const double2* __restrict__ hamp, __nv_bfloat16* __restrict__ b3, int np, int na,
                          int nv, int p3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv * np * na) return;
  const int a = i % na, p = (i / na) % np, v = i / (na * np);
  const double2 hz = hamp[i];
  const float hr = (float)(-hz.x), hi_ = (float)(-hz.y);
  __nv_bfloat16* base = b3 + (size_t)v * 4 * na * p3;
  __nv_bfloat16 rh, rl, ih, il, nh, nl;
  split_bf16(hr, rh, rl);
  split_bf16(hi_, ih, il);
  split_bf16(-hr, nh, nl);
  base[(size_t)a * p3 + p] = rh;
  base[(size_t)a * p3 + np + p] = ih;
  base[(size_t)(2 * na + a) * p3 + p] = rl;
  base[(size_t)(2 * na + a) * p3 + np + p] = il;
  base[(size_t)(na + a) * p3 + p] = ih;
  base[(size_t)(na + a) * p3 + np + p] = nh;
  base[(size_t)(3 * na + a) * p3 + p] = il;
  base[(size_t)(3 * na + a) * p3 + np + p] = nl;
}

// Lanczos stage 2 and normalisation fused with the next action's psi operand
// (OCEAN_haydock.f90:862-889 then long_range.f90:897-906), on the double-float
// vectors of the mixed-precision loop, for chain v = blockIdx.y: from the
// combine's double-float partials, a + i ia = <h|psi> and b_i^2 = |h - a psi|^2 =
// |h|^2 - 2 a Re<h|psi> + a^2 |psi|^2 (formed in FP64 by one thread and broadcast,
// so h is read once); psi = (h - a psi) / b_i written in place of h, and B1 rows of
// vector v built from allow o psi.  One thread per (n, k) covers both K = n and
// K = Nb + n for every alpha.  Every CTA sums the partials in the same order.
__device__ __forceinline__ void norm_prep_body(const double* __restrict__ red1, int nblk, size_t rstride,
                            double* __restrict__ hbase, const double* __restrict__ pbase, size_t vstride,
                            size_t npsi, const float* __restrict__ allow, __nv_bfloat16* __restrict__ b1, int nb,
                            int nk, int na, int ncol, int p1, double* __restrict__ ra_base,
                            double* __restrict__ ia_base, double* __restrict__ rb_base, size_t cstride,
                            const int* __restrict__ itp, int bx, int by, int nbx) {
  __shared__ float2 sh[4][32];
  __shared__ float2 s_am, s_inv;
  const int vv = by;
  const float2* r1 = reinterpret_cast<const float2*>(red1 + (size_t)vv * rstride);  // <h|psi> pairs
  const float2* r2 = r1 + 2 * nblk;                                                // |h|^2, |psi|^2 pairs
  df q[4] = {df{0.0f, 0.0f}, df{0.0f, 0.0f}, df{0.0f, 0.0f}, df{0.0f, 0.0f}};
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    q[0] = df_add(q[0], df{r1[2 * i].x, r1[2 * i].y});
    q[1] = df_add(q[1], df{r1[2 * i + 1].x, r1[2 * i + 1].y});
    q[2] = df_add(q[2], df{r2[2 * i].x, r2[2 * i].y});
    q[3] = df_add(q[3], df{r2[2 * i + 1].x, r2[2 * i + 1].y});
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
    for (int o = 16; o > 0; o >>= 1)
      q[j] = df_add(q[j], df{__shfl_down_sync(0xffffffffu, q[j].h, o), __shfl_down_sync(0xffffffffu, q[j].l, o)});
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int j = 0; j < 4; ++j) sh[j][threadIdx.x >> 5] = make_float2(q[j].h, q[j].l);
  __syncthreads();
  df t[4] = {df{0.0f, 0.0f}, df{0.0f, 0.0f}, df{0.0f, 0.0f}, df{0.0f, 0.0f}};
  if (threadIdx.x < 32) {  // warp 0 adds the warp partials by a fixed shuffle tree
    const int nw = (int)(blockDim.x >> 5), l = threadIdx.x;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      t[j] = l < nw ? df{sh[j][l].x, sh[j][l].y} : df{0.0f, 0.0f};
      for (int o = 16; o > 0; o >>= 1)
        t[j] = df_add(t[j], df{__shfl_down_sync(0xffffffffu, t[j].h, o), __shfl_down_sync(0xffffffffu, t[j].l, o)});
    }
  }
  if (threadIdx.x == 0) {
    const double a = df_value(t[0]), hh = df_value(t[2]), pp = df_value(t[3]);
    const double b = sqrt(hh - 2.0 * a * a + a * a * pp);
    if (bx == 0) {
      const int it = *itp;
      ra_base[(size_t)vv * cstride + it - 1] = a;
      ia_base[(size_t)vv * cstride + it - 1] = df_value(t[1]);
      rb_base[(size_t)vv * cstride + it] = b;
    }
    const df am = df_neg(t[0]), inv = df_split(1.0 / b);
    s_am = make_float2(am.h, am.l);
    s_inv = make_float2(inv.h, inv.l);
  }
  __syncthreads();
  const df am{s_am.x, s_am.y}, inv{s_inv.x, s_inv.y};
  float2* hr = reinterpret_cast<float2*>(hbase + (size_t)vv * vstride);
  float2* hi = hr + npsi;
  const float2* pr = reinterpret_cast<const float2*>(pbase + (size_t)vv * vstride);
  const float2* pi = pr + npsi;
  const int g4 = 4 * na;
  const int total = nb * nk;
  for (int i = bx * blockDim.x + threadIdx.x; i < total; i += nbx * blockDim.x) {
    const int n = i % nb;
    const int k = i / nb;
    __nv_bfloat16* base = b1 + (size_t)k * ncol * p1 + (size_t)vv * g4 * p1;
    for (int a = 0; a < na; ++a) {
      const size_t idx = (size_t)i + (size_t)total * a;
      const df r = df_mul(df_add(df_ld(hr, idx), df_mul(am, df_ld(pr, idx))), inv);
      const df im = df_mul(df_add(df_ld(hi, idx), df_mul(am, df_ld(pi, idx))), inv);
      df_st(hr, idx, r);
      df_st(hi, idx, im);
      const float m = allow[idx];
      const float qr = df_to_float(r) * m, qi = df_to_float(im) * m;
      __nv_bfloat16 h0, l0, h1, l1, h2, l2;
      split_bf16(qr, h0, l0);
      split_bf16(qi, h1, l1);
      split_bf16(-qi, h2, l2);
      // K = n (c = 0): part 0 <- qr, part 1 <- qi;  K = Nb + n (c = 1): part 0 <- -qi, part 1 <- qr
      base[(size_t)(a)*p1 + n] = h0;
      base[(size_t)(na + a) * p1 + n] = h1;
      base[(size_t)(2 * na + a) * p1 + n] = l0;
      base[(size_t)(3 * na + a) * p1 + n] = l1;
      base[(size_t)(a)*p1 + nb + n] = h2;
      base[(size_t)(na + a) * p1 + nb + n] = h0;
      base[(size_t)(2 * na + a) * p1 + nb + n] = l2;
      base[(size_t)(3 * na + a) * p1 + nb + n] = l0;
    }
  }
}

__global__ void __launch_bounds__(LZ_DF_THREADS)
    k_norm_prep(const double* __restrict__ red1, int nblk, size_t rstride, double* __restrict__ hbase,
                const double* __restrict__ pbase, size_t vstride, size_t npsi, const float* __restrict__ allow,
                __nv_bfloat16* __restrict__ b1, int nb, int nk, int na, int ncol, int p1, double* __restrict__ ra_base,
                double* __restrict__ ia_base, double* __restrict__ rb_base, size_t cstride,
                const int* __restrict__ itp) {
  norm_prep_body(red1, nblk, rstride, hbase, pbase, vstride, npsi, allow, b1, nb, nk, na, ncol, p1, ra_base, ia_base,
                 rb_base, cstride, itp, blockIdx.x, blockIdx.y, gridDim.x);
}

struct NormGroupArgs {
  const double* red1;
  int nblk;
  size_t rstride;
  double* hbase;
  const double* pbase;
  size_t vstride, npsi;
  const float* allow;
  __nv_bfloat16* b1;
  int nb, nk, na, ncol, p1;
  double *ra_base, *ia_base, *rb_base;
  size_t cstride;
  const int* itp;
  int nv;
};
// grid (blocks per context, largest block of vectors, contexts)
__global__ void __launch_bounds__(LZ_DF_THREADS) k_norm_prep_group(const NormGroupArgs* __restrict__ tab) {
  const NormGroupArgs& a = tab[blockIdx.z];
  if ((int)blockIdx.y >= a.nv || (int)blockIdx.x >= a.nblk) return;
  norm_prep_body(a.red1, a.nblk, a.rstride, a.hbase, a.pbase, a.vstride, a.npsi, a.allow, a.b1, a.nb, a.nk, a.na,
                 a.ncol, a.p1, a.ra_base, a.ia_base, a.rb_base, a.cstride, a.itp, blockIdx.x, blockIdx.y, a.nblk);
}


// The last of n records whose first CTA is <= b (records ordered by cta0).
template <class A>
__device__ __forceinline__ int group_find(const A* __restrict__ tab, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tab[mid].cta0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// B2 rows of the x-point of this CTA, written straight from the transformed
// planes (no phi' round trip through HBM).  B2 is MN-major: B2[k][K2][col],
// K2 = (x/64)*128 + c*64 + x%64, col = v*4Na + s*2Na + part*Na + a, and
//   part 0 (Re out): c = 0 -> Re phi', c = 1 -> Im phi'
//   part 1 (Im out): c = 0 -> Im phi', c = 1 -> -Re phi'
// with s = 0 / 1 the high / low BF16 half.  The CTA holds transforms t0 .. t0+nt-1
// of its x-point (nt a multiple of Na, so whole vectors); get(t, k) = Nk phi'(k).
// One thread per (k, c, vector) writes the vector's 4 Na columns (8 Na bytes).
// One vector's 4 NA columns of row (k, c), transforms tb .. tb+NA-1: built in
// registers, stored as NA/2 16-byte words.
template <int NA, class Get>
__device__ __forceinline__ void b2_row(const Get& get, float norm, __nv_bfloat16* __restrict__ dst, int tb, int k,
                                       int c) {
  uint32_t pk[2 * NA];  // column j = s*2NA + part*NA + a in half j%2 of pk[j/2]
#pragma unroll
  for (int a = 0; a < NA; a += 2) {
    __nv_bfloat16 h[2][2], l[2][2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float2 f = get(tb + a + q, k);
      const float re = f.x * norm, im = f.y * norm;
      split_bf16(c == 0 ? re : im, h[0][q], l[0][q]);
      split_bf16(c == 0 ? im : -re, h[1][q], l[1][q]);
    }
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      pk[(part * NA + a) / 2] = pack_bf16(h[part][0], h[part][1]);
      pk[(2 * NA + part * NA + a) / 2] = pack_bf16(l[part][0], l[part][1]);
    }
  }
#pragma unroll
  for (int q = 0; q < NA / 2; ++q)
    reinterpret_cast<uint4*>(dst)[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
}

// Any Na (a multiple of 4): runs of 4 BF16 per (s, part, 4 alphas).
template <class Get>
__device__ __forceinline__ void b2_row_any(const Get& get, float norm, __nv_bfloat16* __restrict__ dst, int tb,
                                           int na, int k, int c) {
  for (int a0 = 0; a0 < na; a0 += 4) {
    __nv_bfloat16 h[2][4], l[2][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2 f = get(tb + a0 + q, k);
      const float re = f.x * norm, im = f.y * norm;
      split_bf16(c == 0 ? re : im, h[0][q], l[0][q]);
      split_bf16(c == 0 ? im : -re, h[1][q], l[1][q]);
    }
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      *reinterpret_cast<uint2*>(dst + part * na + a0) =
          make_uint2(pack_bf16(h[part][0], h[part][1]), pack_bf16(h[part][2], h[part][3]));
      *reinterpret_cast<uint2*>(dst + 2 * na + part * na + a0) =
          make_uint2(pack_bf16(l[part][0], l[part][1]), pack_bf16(l[part][2], l[part][3]));
    }
  }
}

// NTC: transforms per CTA when known at compile time (a multiple of Na), which
// bounds the Na the kernel instantiation can meet (and so its registers).
template <int NTC, class Get>
__device__ __forceinline__ void store_b2_rows(const Get& get, float norm, __nv_bfloat16* __restrict__ b2, int nk,
                                              int x, int na, int t0, int nt, int ncol, int k2ext) {
  const int nvl = nt / na, v0 = t0 / na;
  const int row_x = ((x >> 6) << 7) + (x & 63);
  const int items = nk * 2 * nvl;
  for (int e = threadIdx.x; e < items; e += blockDim.x) {
    const int vl = e % nvl;
    const int c = (e / nvl) & 1;
    const int k = e / (2 * nvl);
    __nv_bfloat16* dst = b2 + ((size_t)k * k2ext + row_x + 64 * c) * ncol + (size_t)(v0 + vl) * 4 * na;
    if (NTC == 4 || na == 4) b2_row<4>(get, norm, dst, vl * na, k, c);
    else if (na == 12) b2_row<12>(get, norm, dst, vl * na, k, c);
    else b2_row_any(get, norm, dst, vl * na, na, k, c);
  }
}

// FP32 k-mesh transform of one x-point per CTA (ocn_kmesh_dft.cuh), B2 rows out: generic meshes
__global__ void k_fft_b2(const float2* __restrict__ phi, const float* __restrict__ W, int nx,
                         const KmeshGeom<float> g, const float2* __restrict__ twg, __nv_bfloat16* __restrict__ b2,
                         int na, int ncol, int k2ext) {
  extern __shared__ float2 fsm[];
  float2* tw = fsm;
  float2* buf = fsm + 3 * OCN_MAX_KDIM;
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  kmesh_transform<float>(phi, W, nx, blockIdx.x, g, buf, tw);
  const auto get = [&](int t, int k) { return buf[t * g.slab + kpad(g, k)]; };
  store_b2_rows<0>(get, 1.0f / (float)g.nk, b2, g.nk, blockIdx.x, na, 0, g.na, ncol, k2ext);
}

// cubic meshes: nt transforms (a slice of the ld of the x-point) per CTA
// Cubic k-mesh transform of the nt transforms (a multiple of 4) of x-point x
// owned by this CTA, B2 rows out, in five phases over shared memory (four
// barriers):
//   A  per (k2, k3, group of 4 transforms): the N values along k1 of each, read
//      from phi as 32-byte rows (a k-point's 4 transforms are adjacent), backward
//      DFT along k1, into the padded planes;
//   B  backward DFT along k2;
//   C  backward DFT along k3, x W(x, k), forward DFT along k3 (one line in registers);
//   D  forward DFT along k2;
//   E  per (k2, k3, group of 4): forward DFT along k1 in registers, / Nk, and the
//      B2 columns of the 4 transforms for the N k-points of the line.
// The same separable transform as kmesh_cube_transform (backward = +i), with the
// W pass and the first / last passes fused.
template <int N>
__host__ __device__ constexpr size_t fft_b2_smem_elems(int nt) {
  return 3 * OCN_MAX_KDIM + (N * N * N + 1) / 2 + (size_t)nt * cube_slab<float2>(N);
}
inline size_t fft_b2_smem(int n, int nt) {
  switch (n) {
    case 2: return sizeof(float2) * fft_b2_smem_elems<2>(nt);
    case 3: return sizeof(float2) * fft_b2_smem_elems<3>(nt);
    case 4: return sizeof(float2) * fft_b2_smem_elems<4>(nt);
    case 5: return sizeof(float2) * fft_b2_smem_elems<5>(nt);
    case 6: return sizeof(float2) * fft_b2_smem_elems<6>(nt);
    default: return sizeof(float2) * fft_b2_smem_elems<8>(nt);
  }
}

template <int N, int NTC>
__device__ __forceinline__ void fft_b2_cube_body(const float2* __restrict__ phi, const float* __restrict__ W, int nx,
                                                 int x, int slice, int nt_rt, int ld, const float2* __restrict__ twg,
                                                 __nv_bfloat16* __restrict__ b2, int na, int ncol, int k2ext) {
  constexpr int N2 = N * N, NK = N * N * N, P3 = N + 1;
  constexpr int SLAB = cube_slab<float2>(N);
  const int nt = NTC ? NTC : nt_rt;
  extern __shared__ float2 fsm[];
  float2* tw = fsm;                                               // [axis][t]
  float* ws = reinterpret_cast<float*>(fsm + 3 * OCN_MAX_KDIM);  // W(x, k)
  float2* buf = fsm + 3 * OCN_MAX_KDIM + (NK + 1) / 2;
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  for (int i = threadIdx.x; i < NK; i += blockDim.x) ws[i] = W[(size_t)x * NK + i];
  __syncthreads();
  const int t0 = slice * nt;
  // line tasks (r = k2*N + k3, t) with t fastest: the 4 lanes of a group hold the
  // 4 transforms t = 4g .. 4g+3 of one (k2, k3) line
  const int tasks = N2 * nt;
  // A: load + backward DFT along k1
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int r = task / nt, t = task - r * nt;
    float2 v[N];
#pragma unroll
    for (int k1 = 0; k1 < N; ++k1) v[k1] = phi[((size_t)(k1 * N2 + r) * nx + x) * ld + t0 + t];
    line_dft<float2, float, N>(v, tw, 1.0f);
    float2* dst = buf + t * SLAB + (r / N) * P3 + r % N;
#pragma unroll
    for (int k1 = 0; k1 < N; ++k1) dst[k1 * N * P3] = v[k1];
  }
  __syncthreads();
  // B: backward along k2
  cube_pass<float, N, NTC>(buf, nt, 1, tw + OCN_MAX_KDIM, 1.0f);
  __syncthreads();
  // C: along k3: backward, x W, forward
  for (int l = threadIdx.x; l < nt * N2; l += blockDim.x) {
    const int t = l / N2, r = l - t * N2;  // r = k1*N + k2
    float2* p = buf + t * SLAB + r * P3;
    float2 v[N];
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j];
    line_dft<float2, float, N>(v, tw + 2 * OCN_MAX_KDIM, 1.0f);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float wv = ws[r * N + j];
      v[j].x *= wv;
      v[j].y *= wv;
    }
    line_dft<float2, float, N>(v, tw + 2 * OCN_MAX_KDIM, -1.0f);
#pragma unroll
    for (int j = 0; j < N; ++j) p[j] = v[j];
  }
  __syncthreads();
  // D: forward along k2
  cube_pass<float, N, NTC>(buf, nt, 1, tw + OCN_MAX_KDIM, -1.0f);
  __syncthreads();
  // E: forward along k1 and the B2 columns.  Lane q of a group of 4 writes word q
  // = (split s, part) = (q / 2, q % 2) of the group's 4 alphas: for Na = 4 the 4
  // lanes write one 32-byte row segment.  Every lane of the warp takes part in
  // the shuffles (tasks is a multiple of 4; idle lanes carry zeros).
  const float norm = 1.0f / (float)NK;
  const int row_x = ((x >> 6) << 7) + (x & 63);
  const int lane = threadIdx.x & 31, q = lane & 3, s = q >> 1, part = q & 1;
  for (int base = 0; base < tasks; base += blockDim.x) {
    const int task = base + threadIdx.x;
    const bool on = task < tasks;
    const int r = on ? task / nt : 0, t = on ? task - r * nt : 0;
    float2 v[N];
    if (on) {
      const float2* src = buf + t * SLAB + (r / N) * P3 + r % N;
#pragma unroll
      for (int k1 = 0; k1 < N; ++k1) v[k1] = src[k1 * N * P3];
      line_dft<float2, float, N>(v, tw, -1.0f);
    } else {
#pragma unroll
      for (int k1 = 0; k1 < N; ++k1) v[k1] = make_float2(0.0f, 0.0f);
    }
    const int tg = t0 + (t & ~3), vv = tg / na, a0 = tg - vv * na;
    __nv_bfloat16* col = b2 + (size_t)vv * 4 * na + s * 2 * na + part * na + a0;
#pragma unroll
    for (int k1 = 0; k1 < N; ++k1) {
      float2 f[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        f[j].x = __shfl_sync(0xffffffffu, v[k1].x, (lane & ~3) + j);
        f[j].y = __shfl_sync(0xffffffffu, v[k1].y, (lane & ~3) + j);
      }
      if (!on) continue;
      const size_t k = (size_t)k1 * N2 + r;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        __nv_bfloat16 e[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float re = f[j].x * norm, im = f[j].y * norm;
          const float val = part == 0 ? (c == 0 ? re : im) : (c == 0 ? im : -re);
          __nv_bfloat16 hv, lv;
          split_bf16(val, hv, lv);
          e[j] = s == 0 ? hv : lv;
        }
        *reinterpret_cast<uint2*>(col + (k * k2ext + row_x + 64 * c) * ncol) =
            make_uint2(pack_bf16(e[0], e[1]), pack_bf16(e[2], e[3]));
      }
    }
  }
}
template <int N, int NTC>
__global__ void k_fft_b2_cube(const float2* __restrict__ phi, const float* __restrict__ W, int nx, int nt, int ld,
                              const float2* __restrict__ twg, __nv_bfloat16* __restrict__ b2, int na, int ncol,
                              int k2ext) {
  fft_b2_cube_body<N, NTC>(phi, W, nx, blockIdx.x, blockIdx.y, nt, ld, twg, b2, na, ncol, k2ext);
}
typedef void (*CubeFnB2)(const float2*, const float*, int, int, int, const float2*, __nv_bfloat16*, int, int, int);

// The transforms of several contexts of one instantiation class (mesh, slice
// size) in one launch.
struct FftGroupArgs {
  const float2* phi;
  const float* W;
  int nx, nt, ld;  // x-points, transforms per CTA, transforms per x-point
  const float2* tw;
  __nv_bfloat16* b2;
  int na, ncol, k2ext;
  int cta0;        // first CTA of this context; its CTAs are (slice, x) = divmod(local, nx)
};
template <int N, int NTC>
__global__ void k_fft_b2_cube_group(const FftGroupArgs* __restrict__ tab, int n) {
  const FftGroupArgs& a = tab[group_find(tab, n, blockIdx.x)];
  const int local = blockIdx.x - a.cta0;
  fft_b2_cube_body<N, NTC>(a.phi, a.W, a.nx, local % a.nx, local / a.nx, a.nt, a.ld, a.tw, a.b2, a.na, a.ncol,
                           a.k2ext);
}
typedef void (*CubeFnB2Group)(const FftGroupArgs*, int);

__global__ void k_w_to_f32(const double* __restrict__ W, float* __restrict__ Wf, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    Wf[i] = (float)W[i];
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

}  // namespace

struct MixedLR {
  int p1 = 0, ncol = 0, nvmax = 1;
  int p2 = 0;  // K2 extent of UB rows and B2: 128 per 64-x block
  __nv_bfloat16 *ua_hi = nullptr, *ua_lo = nullptr, *ub_hi = nullptr, *ub_lo = nullptr;
  __nv_bfloat16 *b1 = nullptr, *b2 = nullptr;
  float2* phi = nullptr;
  float* Wf = nullptr;
  float2* twf = nullptr;  // FP32 twiddles exp(+2 pi i t / n_axis), [axis][t]
  int* d_err = nullptr;
  CUtensorMap tm_ua_hi, tm_ua_lo, tm_b1, tm_ub_hi, tm_ub_lo, tm_b2;
  TcParams g1{}, g2{};
  int grid1 = 1, grid2 = 1;
  size_t smem_bytes = 0;
  bool cube = false;        // cubic k-mesh: k_fft_b2_cube instantiations apply
  size_t stage_bytes = 0;   // shared memory of one pipeline stage
  int max_stages = 1;       // deepest pipeline that fits the shared-memory budget
  int cfg[7] = {0, 0, 0, 0, 0, 0, 0};  // stages, GEMM2 K splits (requested), grid caps of GEMM1 / GEMM2,
                                      // k-mesh transforms per CTA (0: all of an x-point), its threads (0: 128),
                                      // band->x output staging (1: when shared memory allows)
  size_t part_cap = 0;      // splits the partial-sum buffer holds
  // multiplet projector contractions (fg_combo) on the tensor cores
  bool mult_ready = false;
  int np = 0, p3 = 0;
  __nv_bfloat16 *ma_hi = nullptr, *ma_lo = nullptr;  // [k][p][p1]: amplitude contraction A
  __nv_bfloat16 *mb_hi = nullptr, *mb_lo = nullptr;  // [k][n][p3]: back-projection A
  __nv_bfloat16* b3 = nullptr;                        // [col][p3]: back-projection B (all k)
  float2* amp_part = nullptr;                         // [k][p][v*Na + a]
  double2 *amp = nullptr, *hamp = nullptr;            // [v][p][a]
  CUtensorMap tm_ma_hi, tm_ma_lo, tm_mb_hi, tm_mb_lo, tm_b3;
  TcParams gm1{}, gm2{};
  int gridm1 = 0, gridm2 = 0;
  bool ready = false;
  int* pending_inc = nullptr;  // set by a Haydock step: the next band -> x launch advances this counter
};

namespace {

// Shared memory of the band->x output staging: four epilogue warps, 32 rows of
// ncol/4 + 1 complex values each.
size_t estg_bytes(int ncol) { return (size_t)4 * 32 * (ncol / 4 + 1) * sizeof(float2); }

size_t device_smem_optin(const ocn_ctx* c) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device) != cudaSuccess) return 0;
  return (size_t)v;
}

int encode3d(ocn_ctx* c, EncodeTiledFn fn, CUtensorMap* m, void* base, uint64_t inner, uint64_t rows,
             uint64_t outer, uint64_t pitch_elems, uint32_t box_rows) {
  const cuuint64_t dims[3] = {inner, rows, outer};
  const cuuint64_t strides[2] = {pitch_elems * 2, pitch_elems * 2 * rows};
  const cuuint32_t box[3] = {(cuuint32_t)TC_BK, box_rows, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, OCN_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return OCN_OK;
}

// A stored chunk-major, [outer][chunk][row][64]: 64 x 128-row boxes with 128-byte
// swizzling, each one contiguous run of memory
int encode_a_chunked(ocn_ctx* c, EncodeTiledFn fn, CUtensorMap* m, void* base, uint64_t rows, uint64_t nchunk,
                     uint64_t outer) {
  const cuuint64_t dims[4] = {(cuuint64_t)TC_BK, rows, nchunk, outer};
  const cuuint64_t strides[3] = {(cuuint64_t)TC_BK * 2, (cuuint64_t)TC_BK * 2 * rows,
                                 (cuuint64_t)TC_BK * 2 * rows * nchunk};
  const cuuint32_t box[4] = {(cuuint32_t)TC_BK, (cuuint32_t)TC_BM, 1, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, OCN_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return OCN_OK;
}

// B2[k][K2][col] as 16-column by 64-row boxes with 32-byte swizzling (MN-major B)
int encode_b_mn(ocn_ctx* c, EncodeTiledFn fn, CUtensorMap* m, void* base, uint64_t ncol, uint64_t rows,
                uint64_t outer) {
  const cuuint64_t dims[3] = {ncol, rows, outer};
  const cuuint64_t strides[2] = {ncol * 2, ncol * 2 * rows};
  const cuuint32_t box[3] = {16, (cuuint32_t)TC_BK, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(c, OCN_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return OCN_OK;
}

template <typename T>
int alloc(ocn_ctx* c, T** p, size_t n) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (e != cudaSuccess) return set_err(c, OCN_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return OCN_OK;
}

}  // namespace

// Transforms per CTA of the cubic k-mesh step for ntot = Na * nv transforms:
// the configured count when it is a whole number of vectors (a multiple of Na
// dividing ntot: a CTA writes whole B2 column blocks), else all of them; reduced
// to one vector's Na when that would not fit in shared memory.
int cube_tc(const MixedLR* m, int kn, int na, int ntot) {
  const int q = m->cfg[4];
  int tc = (q > 0 && q % na == 0 && ntot % q == 0) ? q : ntot;
  if (fft_b2_smem(kn, tc) > 227u * 1024u) tc = na;
  return tc;
}

int mixed_init(ocn_ctx* c) {
  if (c->nspn != 1 && c->nspn != 2) return set_err(c, OCN_ERR_UNSUPPORTED, "nspn must be 1 or 2");
  const int nb = c->nb, nk = c->nk, nx = c->nx, na = c->na, nvmax = c->nvec, ns = c->nspn;
  const int ncol = 4 * na * nvmax;
  if (ncol > TC_MAX_NCOL)
    return set_err(c, OCN_ERR_ARG, "nvec too large: 4*nalpha*nvec must be <= 256");
  const bool cube = kmesh_cube_supported(c->dims.kmesh);
  const size_t fsm = cube ? fft_b2_smem(c->dims.kmesh[0], na)
                          : kmesh_smem(kmesh_geom<float>(c->dims.kmesh, na * nvmax));
  if (fsm > 227u * 1024u)
    return set_err(c, OCN_ERR_ARG, "nvec*nalpha*Nk too large for the shared-memory k-mesh transform");
  MixedLR* m = new (std::nothrow) MixedLR();
  if (!m) return set_err(c, OCN_ERR_ALLOC, "host allocation failed");
  c->mixed = m;
  m->nvmax = nvmax;
  m->ncol = ncol;
  m->p1 = (2 * nb + 7) / 8 * 8;
  const int nxc = (nx + TC_BK - 1) / TC_BK;  // 64-x blocks
  m->p2 = 2 * nxc * TC_BK;
  int rc;
  // u2 operands of both valence spins, spin-major: spin s at outer index s*Nk + k
  if ((rc = alloc(c, &m->ua_hi, (size_t)ns * nk * nx * m->p1)) ||
      (rc = alloc(c, &m->ua_lo, (size_t)ns * nk * nx * m->p1)) ||
      (rc = alloc(c, &m->ub_hi, (size_t)ns * nk * nb * m->p2)) ||
      (rc = alloc(c, &m->ub_lo, (size_t)ns * nk * nb * m->p2)) ||
      (rc = alloc(c, &m->b1, (size_t)nk * ncol * m->p1)) || (rc = alloc(c, &m->b2, (size_t)nk * ncol * m->p2)) ||
      (rc = alloc(c, &m->phi, (size_t)nk * nx * na * nvmax)) || (rc = alloc(c, &m->Wf, (size_t)nk * nx)) ||
      (rc = alloc(c, &m->d_err, 1)))
    return rc;
  OCN_CUDA(c, cudaMemset(m->d_err, 0, sizeof(int)));
  // operand rows of vectors outside the current block keep finite (zero) values
  OCN_CUDA(c, cudaMemset(m->b1, 0, (size_t)nk * ncol * m->p1 * 2));
  OCN_CUDA(c, cudaMemset(m->b2, 0, (size_t)nk * ncol * m->p2 * 2));
  // the padding of a partial last 64-x block stays zero
  OCN_CUDA(c, cudaMemset(m->ub_hi, 0, (size_t)ns * nk * nb * m->p2 * 2));
  OCN_CUDA(c, cudaMemset(m->ub_lo, 0, (size_t)ns * nk * nb * m->p2 * 2));

  void* fnp = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fnp, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || !fnp) return set_err(c, OCN_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  EncodeTiledFn fn = reinterpret_cast<EncodeTiledFn>(fnp);
  if ((rc = encode3d(c, fn, &m->tm_ua_hi, m->ua_hi, 2 * nb, nx, (uint64_t)ns * nk, m->p1, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_ua_lo, m->ua_lo, 2 * nb, nx, (uint64_t)ns * nk, m->p1, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_b1, m->b1, 2 * nb, ncol, nk, m->p1, ncol)) ||
      (rc = encode_a_chunked(c, fn, &m->tm_ub_hi, m->ub_hi, nb, m->p2 / TC_BK, (uint64_t)ns * nk)) ||
      (rc = encode_a_chunked(c, fn, &m->tm_ub_lo, m->ub_lo, nb, m->p2 / TC_BK, (uint64_t)ns * nk)) ||
      (rc = encode_b_mn(c, fn, &m->tm_b2, m->b2, ncol, m->p2, nk)))
    return rc;

  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ncol >> 3) << 17) |
                         ((uint32_t)(TC_BM >> 4) << 24);
  uint32_t tcols = 32;
  while ((int)tcols < 2 * ncol) tcols <<= 1;
  const size_t stage_bytes = 2 * (size_t)TC_BM * TC_BK * 2 + (size_t)ncol * TC_BK * 2;
  const int stages = (int)std::min<size_t>(TC_MAX_STAGES, (TC_SMEM_BUDGET - 1024 - 256) / stage_bytes);
  TcParams& g1 = m->g1;
  g1.mode = 1;
  g1.nb = nb; g1.nk = nk; g1.nx = nx; g1.na = na;
  g1.ncol = ncol;
  g1.nv = 1;
  g1.nvmax = nvmax;
  g1.stages = stages;
  g1.nch = (2 * nb + TC_BK - 1) / TC_BK;
  g1.nxt = (nx + TC_BM - 1) / TC_BM;
  g1.ntiles = nk * g1.nxt;
  g1.idesc = idesc;
  g1.tcols = tcols;
  g1.phi = m->phi;
  g1.err = m->d_err;
  g1.npsi = c->npsi;
  g1.bshared = 0;
  g1.koff = 0;
  g1.spin = -1;  // set per launch on spin-polarised problems
  TcParams& g2 = m->g2;
  g2 = g1;
  g2.mode = 2;
  g2.nch = 2 * nxc;
  g2.mt2 = (nb + TC_BM - 1) / TC_BM;
  g2.bmn = 1;
  g2.achunk = 1;
  g2.idesc = idesc | (1u << 16);  // B MN-major
  m->stage_bytes = stage_bytes;
  m->max_stages = stages;
  c->part_stride = (size_t)nvmax * 2 * c->npsi;
  // default tiling: K splits of GEMM2 so that about four tiles per SM exist,
  // full pipeline depth, one persistent CTA per SM at most
  int ks = (4 * c->sm_count + nk * g2.mt2 - 1) / (nk * g2.mt2);
  ks = std::max(1, std::min(ks, std::max(1, g2.nch / 4)));
  // pipeline depth: the deepest that leaves room for the band->x output staging (when that is >= 2)
  const int st_room = (int)((std::min<size_t>(TC_SMEM_BUDGET, device_smem_optin(c) - estg_bytes(ncol)) - 1024 - 256) /
                            stage_bytes);
  const int st_def = st_room >= 2 ? std::min(stages, st_room) : stages;
  // 256-thread transforms: measured best on 8^3; output staging: measured faster for blocks of vectors,
  // slightly slower for one vector
  const int cfg[7] = {st_def, ks, c->sm_count, c->sm_count, 0, 256, nvmax > 1 ? 1 : 0};
  if ((rc = mixed_configure(c, cfg))) return rc;
  if (int rc_ = allow_max_smem(c, k_lr_tc)) return rc_;
  if (int rc_ = allow_max_smem(c, k_fft_b2)) return rc_;
  if (cube) {
    // the three instantiations a call can select (nt = 4, 12, other)
    for (int nt : {4, 12, 1}) {
      CubeFnB2 f;
      OCN_CUBE_DISPATCH(k_fft_b2_cube, c->dims.kmesh[0], nt, f);
      if (int rc_ = allow_max_smem(c, f)) return rc_;
    }
    m->cube = true;
  }
  // FP32 twiddles, rounded from FP64 roots of unity
  float2 tw[3][OCN_MAX_KDIM];
  const double pi = 3.1415926535897932384626433832795;
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < OCN_MAX_KDIM; ++t) {
      const int n = c->dims.kmesh[a];
      tw[a][t] = t < n ? make_float2((float)cos(2.0 * pi * t / n), (float)sin(2.0 * pi * t / n))
                       : make_float2(0.f, 0.f);
    }
  if ((rc = alloc(c, &m->twf, (size_t)3 * OCN_MAX_KDIM))) return rc;
  OCN_CUDA(c, cudaMemcpy(m->twf, tw, sizeof(tw), cudaMemcpyHostToDevice));
  return OCN_OK;
}

// Tile configuration: cfg = {pipeline stages, K splits of GEMM2, persistent
// grid cap of GEMM1, of GEMM2, k-mesh transforms per CTA (0 = all of an
// x-point; a value that does not divide a block's count means all), threads of a
// k-mesh transform CTA (128, 256 or 512; 0 = 128), band->x output staging (0 or
// 1; applied when the pipeline leaves the shared memory)}.  Grows the
// partial-sum buffer when a configuration needs more splits.
int mixed_configure(ocn_ctx* c, const int cfg[7]) {
  MixedLR* m = c->mixed;
  if (!m) return set_err(c, OCN_ERR_STATE, "mixed-precision state missing");
  if (cfg[0] < 1 || cfg[0] > m->max_stages || cfg[1] < 1 || cfg[2] < 1 || cfg[3] < 1 || cfg[4] < 0 ||
      (cfg[5] != 0 && cfg[5] != 128 && cfg[5] != 256 && cfg[5] != 512) || cfg[6] < 0 || cfg[6] > 1)
    return set_err(c, OCN_ERR_ARG, "bad tile configuration");
  TcParams& g1 = m->g1;
  TcParams& g2 = m->g2;
  g1.stages = g2.stages = cfg[0];
  const int ks = std::max(1, std::min(cfg[1], g2.nch));
  g2.cps2 = (g2.nch + ks - 1) / ks;
  g2.ks2 = (g2.nch + g2.cps2 - 1) / g2.cps2;  // no empty split
  g2.ntiles = c->nk * g2.mt2 * g2.ks2;
  const size_t need = (size_t)g2.ks2 + (size_t)c->mult_parts;  // LR splits, then the multiplet's
  if (need > m->part_cap) {
    double* np = nullptr;
    int rc = alloc(c, &np, need * c->part_stride);
    if (rc) return rc;
    if (c->d_accpart) cudaFree(c->d_accpart);
    c->d_accpart = np;
    m->part_cap = need;
  }
  g2.part = reinterpret_cast<float*>(c->d_accpart);
  c->lr_xsplit = g2.ks2;
  m->gm2.part = reinterpret_cast<float*>(c->d_accpart) + (size_t)g2.ks2 * c->part_stride;
  m->smem_bytes = 1024 + (size_t)cfg[0] * m->stage_bytes + 256;
  {  // band->x outputs staged for coalesced stores when the pipeline leaves room
    const size_t eb = estg_bytes(m->ncol);
    const int on = (cfg[6] && m->smem_bytes + eb <= device_smem_optin(c)) ? 1 : 0;
    g1.estg = g2.estg = m->gm1.estg = m->gm2.estg = on;
    if (on) m->smem_bytes += eb;
  }
  m->grid1 = std::min(g1.ntiles, std::min(cfg[2], c->sm_count));
  m->grid2 = std::min(g2.ntiles, std::min(cfg[3], c->sm_count));
  m->gm1.stages = m->gm2.stages = cfg[0];
  m->gridm1 = std::min(m->gm1.ntiles, std::min(cfg[2], c->sm_count));
  m->gridm2 = std::min(m->gm2.ntiles, std::min(cfg[3], c->sm_count));
  for (int i = 0; i < 7; ++i) m->cfg[i] = cfg[i];
  return OCN_OK;
}

int mixed_config(const ocn_ctx* c, int cfg[7]) {
  if (!c->mixed) return OCN_ERR_STATE;
  for (int i = 0; i < 7; ++i) cfg[i] = c->mixed->cfg[i];
  return OCN_OK;
}

// Times the long-range term of an nv-vector block under candidate tile
// configurations (CUDA events on the context stream, reps launches each after
// one warm-up) and keeps the fastest.  Two rounds: pipeline depth 2..max x
// GEMM2 K splits {1, 2, 4, 8, current} x persistent grids of all SMs or half,
// then the k-mesh transforms per CTA {all, 4, 12} x their threads under the
// round-one winner, then the band->x output staging switched.
int mixed_autotune(ocn_ctx* c, int nv, int reps, double* best_ms, double* current_ms, int best_cfg[7]) {
  MixedLR* m = c->mixed;
  if (!m || !m->ready) return set_err(c, OCN_ERR_STATE, "mixed-precision operands not built");
  if (nv < 1 || nv > m->nvmax) return set_err(c, OCN_ERR_ARG, "block size exceeds nvec");
  reps = std::max(1, reps);
  const size_t n = c->npsi;
  double* v = nullptr;
  int rc = alloc(c, &v, 2 * n * nv);
  if (rc) return rc;
  for (int j = 0; j < nv && rc == OCN_OK; ++j) rc = vec_fill(c, v + 2 * j * n, 1.0, 0.5);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  typedef std::array<int, 7> Cfg;
  const Cfg def = {m->cfg[0], m->cfg[1], m->cfg[2], m->cfg[3], m->cfg[4], m->cfg[5], m->cfg[6]};
  double best = 1e300, dms = 0.0;
  Cfg bc = def;
  auto time_cfg = [&](const Cfg& a) -> int {
    int q;
    if ((q = mixed_configure(c, a.data()))) return q;
    if ((q = lr_apply_mixed(c, v, v + n, 2 * n, nv))) return q;  // warm-up
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && q == OCN_OK; ++r) q = lr_apply_mixed(c, v, v + n, 2 * n, nv);
    cudaEventRecord(e1, c->stream);
    cudaError_t ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) return cuda_fail(c, ce, "autotune");
    if (q || (q = mixed_check(c))) return q;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (a == def) dms = ms / reps;
    if (ms / reps < best) {
      best = ms / reps;
      bc = a;
    }
    return OCN_OK;
  };
  std::vector<Cfg> cand{def};  // the configuration in force, timed first
  for (int st = std::min(2, m->max_stages); st <= m->max_stages; ++st)
    for (int ks : {1, 2, 4, 8, def[1]})
      for (int gc : {c->sm_count, std::max(1, c->sm_count / 2)}) {
        const Cfg a = {st, ks, gc, gc, def[4], def[5], def[6]};
        if (std::find(cand.begin(), cand.end(), a) == cand.end()) cand.push_back(a);
      }
  for (size_t i = 0; i < cand.size() && rc == OCN_OK; ++i) rc = time_cfg(cand[i]);
  if (m->cube && rc == OCN_OK) {
    const Cfg r1 = bc;
    for (int tc : {0, 4, 12})
      for (int th : {128, 256, 512}) {
        Cfg a = r1;
        a[4] = tc;
        a[5] = th;
        const bool same = (tc == r1[4]) && (th == (r1[5] ? r1[5] : 128));
        if (!same && rc == OCN_OK) rc = time_cfg(a);
      }
  }
  if (rc == OCN_OK) {  // output staging on / off under the winner
    Cfg a = bc;
    a[6] = 1 - a[6];
    rc = time_cfg(a);
  }
  const int rf = mixed_configure(c, rc ? def.data() : bc.data());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(v);
  if (rc) return rc;
  if (rf) return rf;
  if (best_ms) *best_ms = best;
  if (current_ms) *current_ms = dms;
  if (best_cfg)
    for (int i = 0; i < 7; ++i) best_cfg[i] = bc[i];
  return OCN_OK;
}

// Split-BF16 operands and tiling of the multiplet projector contractions, from
// the projector coefficients of ocn_set_mult (c->mult.mpc [s][p][k*Nb + n]; the
// operands of both spins are stored spin-major, spin s at outer index s*Nk + k).
int mixed_set_mult(ocn_ctx* c) {
  MixedLR* m = c->mixed;
  if (!m) return OCN_OK;
  MultDev& d = c->mult;
  void* old[] = {m->ma_hi, m->ma_lo, m->mb_hi, m->mb_lo, m->b3, m->amp_part, m->amp, m->hamp};
  for (void* q : old)
    if (q) cudaFree(q);
  m->ma_hi = m->ma_lo = m->mb_hi = m->mb_lo = m->b3 = nullptr;
  m->amp_part = nullptr;
  m->amp = m->hamp = nullptr;
  m->mult_ready = false;
  c->mult_parts = 0;
  const int np = d.np, nb = c->nb, nk = c->nk, na = c->na, nvmax = m->nvmax;
  if (np < 1) return OCN_OK;
  m->np = np;
  m->p3 = (2 * np + 7) / 8 * 8;
  int rc;
  const int ns = c->nspn;
  if ((rc = alloc(c, &m->ma_hi, (size_t)ns * nk * np * m->p1)) ||
      (rc = alloc(c, &m->ma_lo, (size_t)ns * nk * np * m->p1)) ||
      (rc = alloc(c, &m->mb_hi, (size_t)ns * nk * nb * m->p3)) ||
      (rc = alloc(c, &m->mb_lo, (size_t)ns * nk * nb * m->p3)) ||
      (rc = alloc(c, &m->b3, (size_t)m->ncol * m->p3)) ||
      (rc = alloc(c, &m->amp_part, (size_t)nk * np * na * nvmax)) ||
      (rc = alloc(c, &m->amp, (size_t)nvmax * np * na)) || (rc = alloc(c, &m->hamp, (size_t)nvmax * np * na)))
    return rc;
  OCN_CUDA(c, cudaMemsetAsync(m->b3, 0, (size_t)m->ncol * m->p3 * 2, c->stream));
  const int grid = 8 * c->sm_count;
  for (int s = 0; s < ns; ++s) {
    const double2* ms = d.mpc + (size_t)s * np * nb * nk;
    const size_t oa = (size_t)s * nk * np * m->p1, ob = (size_t)s * nk * nb * m->p3;
    k_build_ma<<<grid, 256, 0, c->stream>>>(ms, m->ma_hi + oa, m->ma_lo + oa, nb, nk, np, m->p1);
    k_build_mb<<<grid, 256, 0, c->stream>>>(ms, m->mb_hi + ob, m->mb_lo + ob, nb, nk, np, m->p3);
    c->launches += 2;
  }
  OCN_CUDA(c, cudaGetLastError());
  void* fnp = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fnp, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || !fnp) return set_err(c, OCN_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  EncodeTiledFn fn = reinterpret_cast<EncodeTiledFn>(fnp);
  if ((rc = encode3d(c, fn, &m->tm_ma_hi, m->ma_hi, 2 * nb, np, (uint64_t)ns * nk, m->p1, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_ma_lo, m->ma_lo, 2 * nb, np, (uint64_t)ns * nk, m->p1, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_mb_hi, m->mb_hi, 2 * np, nb, (uint64_t)ns * nk, m->p3, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_mb_lo, m->mb_lo, 2 * np, nb, (uint64_t)ns * nk, m->p3, TC_BM)) ||
      (rc = encode3d(c, fn, &m->tm_b3, m->b3, 2 * np, m->ncol, 1, m->p3, m->ncol)))
    return rc;
  TcParams& a = m->gm1;  // amplitudes: band->x form with Np rows per k
  a = m->g1;
  a.nx = np;
  a.nxt = (np + TC_BM - 1) / TC_BM;
  a.ntiles = nk * a.nxt;
  a.phi = m->amp_part;
  a.bshared = 0;
  TcParams& b = m->gm2;  // back-projection: x->band form over 2 Np, B shared by every k
  b = m->g2;
  b.nx = np;
  b.nch = (2 * np + TC_BK - 1) / TC_BK;
  b.cps2 = b.nch;
  b.ks2 = 1;
  b.ntiles = nk * b.mt2;
  b.bshared = 1;
  b.bmn = 0;  // B3 is K-major
  b.achunk = 0;
  b.idesc = m->g1.idesc;
  c->mult_parts = 1;
  if ((rc = mixed_configure(c, m->cfg))) return rc;  // partial-sum room, multiplet grids
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  m->mult_ready = true;
  return OCN_OK;
}

// Multiplet term of nv vectors (OCEAN_fg_combo, OCEAN_multiplet.f90:1617-2005):
// amplitudes on the tensor cores, the direct / exchange matrices in FP64
// (k_mult_hamp), the back-projection on the tensor cores into the multiplet
// slice of d_accpart.  b1_ready: the psi operand B1 already holds these vectors.
int mult_apply_mixed(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv, bool b1_ready) {
  MixedLR* m = c->mixed;
  if (!m || !m->mult_ready) return set_err(c, OCN_ERR_STATE, "mixed-precision multiplet operands not built");
  if (nv < 1 || nv > m->nvmax) return set_err(c, OCN_ERR_ARG, "block size exceeds nvec");
  int rc;
  if (!b1_ready && (rc = mixed_prep_b1(c, d_pr, d_pi, vstride, nv))) return rc;
  TimedScope ts(c, T_MULT);
  const int np = m->np, na = c->na;
  TcParams a = m->gm1, b = m->gm2;
  a.nv = nv;
  b.nv = nv;
  const int ns = c->nspn;  // spin-polarised: per spin, each launch writes its own alphas
  for (int s = 0; s < ns; ++s) {
    a.koff = s * c->nk;
    a.spin = ns == 2 ? s : -1;
    a.inc = m->pending_inc;
    m->pending_inc = nullptr;
    k_lr_tc<<<m->gridm1, TC_THREADS, m->smem_bytes, c->stream>>>(m->tm_ma_hi, m->tm_ma_lo, m->tm_b1, a);
    ++c->launches;
  }
  k_amp_reduce_f32<<<(np * na * nv + 31) / 32, 32 * AMP_KGROUPS, 0, c->stream>>>(m->amp_part, m->amp, c->nk,
                                                                                 np, na, nv);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  for (int v = 0; v < nv; ++v)
    if ((rc = mult_hamp(c, m->amp + (size_t)v * np * na, m->hamp + (size_t)v * np * na))) return rc;
  k_prep_b3<<<(nv * np * na + 127) / 128, 128, 0, c->stream>>>(m->hamp, m->b3, np, na, nv, m->p3);
  ++c->launches;
  for (int s = 0; s < ns; ++s) {
    b.koff = s * c->nk;
    b.spin = ns == 2 ? s : -1;
    k_lr_tc<<<m->gridm2, TC_THREADS, m->smem_bytes, c->stream>>>(m->tm_mb_hi, m->tm_mb_lo, m->tm_b3, b);
    ++c->launches;
  }
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int mixed_free(ocn_ctx* c) {
  MixedLR* m = c->mixed;
  if (!m) return OCN_OK;
  void* bufs[] = {m->ua_hi, m->ua_lo, m->ub_hi, m->ub_lo, m->b1,     m->b2,       m->phi,  m->Wf,
                  m->d_err, m->twf,   m->ma_hi, m->ma_lo, m->mb_hi, m->mb_lo, m->b3, m->amp_part,
                  m->amp,   m->hamp};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete m;
  c->mixed = nullptr;
  return OCN_OK;
}

int mixed_set_bloch(ocn_ctx* c) {
  MixedLR* m = c->mixed;
  if (!m) return set_err(c, OCN_ERR_STATE, "mixed state missing");
  const int nb = c->nb, nk = c->nk, nx = c->nx;
  const int grid = 8 * c->sm_count;
  for (int s = 0; s < c->nspn; ++s) {  // u [s][x][k][n] -> spin-major operands
    const size_t us = (size_t)s * nx * nk * nb;
    const size_t oa = (size_t)s * nk * nx * m->p1, ob = (size_t)s * nk * nb * m->p2;
    k_build_ua<<<grid, 256, 0, c->stream>>>(c->d_u + us, m->ua_hi + oa, m->ua_lo + oa, nb, nk, nx, m->p1);
    OCN_CUDA(c, cudaGetLastError());
    k_build_ub<<<grid, 256, 0, c->stream>>>(c->d_u + us, m->ub_hi + ob, m->ub_lo + ob, nb, nk, nx, m->p2);
    OCN_CUDA(c, cudaGetLastError());
    c->launches += 2;
  }
  k_w_to_f32<<<grid, 256, 0, c->stream>>>(c->d_W, m->Wf, (size_t)nk * nx);
  OCN_CUDA(c, cudaGetLastError());
  c->launches += 1;
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  m->ready = true;
  return OCN_OK;
}

// The iteration counter of a Haydock step, advanced by the step's first
// tensor-core launch (band -> x or the multiplet amplitudes) instead of a launch
// of its own; mixed_take_advance reports (and clears) a request no launch took.
void mixed_defer_advance(ocn_ctx* c, int* itp) {
  if (c->mixed) c->mixed->pending_inc = itp;
}
bool mixed_take_advance(ocn_ctx* c) {
  if (!c->mixed || !c->mixed->pending_inc) return false;
  c->mixed->pending_inc = nullptr;
  return true;
}

int mixed_set_starve(ocn_ctx* c, int on) {
  MixedLR* m = c->mixed;
  if (!m || !m->ready) return set_err(c, OCN_ERR_STATE, "mixed-precision operands not built");
  m->g1.starve = m->g2.starve = on ? 1 : 0;
  return OCN_OK;
}

int mixed_check(ocn_ctx* c) {
  MixedLR* m = c->mixed;
  if (!m) return OCN_OK;
  int h = 0;
  OCN_CUDA(c, cudaMemcpy(&h, m->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    cudaMemset(m->d_err, 0, sizeof(int));
    return set_err(c, OCN_ERR_TIMEOUT, "tensor-core pipeline wait timed out (code " + std::to_string(h) + ")");
  }
  return OCN_OK;
}

int mixed_norm_prep(ocn_ctx* c, int nv, const double* psi, double* h, double* ra, double* ia, double* rb,
                    size_t cstride, const int* itp) {
  MixedLR* m = c->mixed;  // timed as part of the enclosing Lanczos step
  const int nblk = c->red_blocks;
  dim3 grid(nblk, nv);
  k_norm_prep<<<grid, LZ_DF_THREADS, 0, c->stream>>>(c->d_red, nblk, (size_t)4 * nblk, h, psi, 2 * c->npsi, c->npsi,
                                                      c->d_allow_f, m->b1, c->nb, c->nk, c->na, m->ncol, m->p1, ra,
                                                      ia, rb, cstride, itp);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int mixed_prep_b1(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv) {
  MixedLR* m = c->mixed;
  TimedScope ts(c, T_LR_PREP);
  const int total = nv * c->nk * 2 * c->nb;
  k_prep_b1<<<std::min((total + 255) / 256, 8 * c->sm_count), 256, 0, c->stream>>>(
      d_pr, d_pi, vstride, nv, c->d_allow, m->b1, c->nb, c->nk, c->na, m->ncol, m->p1);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int lr_apply_mixed(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv,
                   bool b1_ready) {
  MixedLR* m = c->mixed;
  if (!m || !m->ready) return set_err(c, OCN_ERR_STATE, "mixed-precision operands not built");
  if (nv < 1 || nv > m->nvmax) return set_err(c, OCN_ERR_ARG, "block size exceeds nvec");
  const int nk = c->nk, nx = c->nx, na = c->na;
  int rc;
  if (!b1_ready && (rc = mixed_prep_b1(c, d_pr, d_pi, vstride, nv))) return rc;
  TcParams g1 = m->g1, g2 = m->g2;
  g1.nv = nv;
  g2.nv = nv;
  const int ns = c->nspn;  // spin-polarised: one launch per valence spin, each writes its own alphas
  {
    TimedScope ts(c, T_LR_GEMM1);
    for (int s = 0; s < ns; ++s) {
      g1.koff = s * nk;
      g1.spin = ns == 2 ? s : -1;
      g1.inc = m->pending_inc;  // the first launch of a Haydock step advances its iteration counter
      m->pending_inc = nullptr;
      k_lr_tc<<<m->grid1, TC_THREADS, m->smem_bytes, c->stream>>>(m->tm_ua_hi, m->tm_ua_lo, m->tm_b1, g1);
      ++c->launches;
      OCN_CUDA(c, cudaGetLastError());
    }
  }
  {
    TimedScope ts(c, T_LR_FFT);  // the k-mesh transform writes the x -> band operand B2 directly
    if (m->cube) {
      // transforms per CTA: all of the x-point, or a slice (tile parameter 5)
      const int ntot = na * nv;
      const int tc = cube_tc(m, c->dims.kmesh[0], na, ntot);
      CubeFnB2 f;
      OCN_CUBE_DISPATCH(k_fft_b2_cube, c->dims.kmesh[0], tc, f);
      const int th = m->cfg[5] ? m->cfg[5] : 128;
      f<<<dim3(nx, ntot / tc), th, fft_b2_smem(c->dims.kmesh[0], tc), c->stream>>>(
          m->phi, m->Wf, nx, tc, ntot, m->twf, m->b2, na, m->ncol, m->p2);
    } else {
      const KmeshGeom<float> g = kmesh_geom<float>(c->dims.kmesh, na * nv);
      k_fft_b2<<<nx, 256, kmesh_smem(g), c->stream>>>(m->phi, m->Wf, nx, g, m->twf, m->b2, na, m->ncol, m->p2);
    }
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  {
    TimedScope ts(c, T_LR_GEMM2);
    for (int s = 0; s < ns; ++s) {
      g2.koff = s * nk;
      g2.spin = ns == 2 ? s : -1;
      k_lr_tc<<<m->grid2, TC_THREADS, m->smem_bytes, c->stream>>>(m->tm_ub_hi, m->tm_ub_lo, m->tm_b2, g2);
      ++c->launches;
      OCN_CUDA(c, cudaGetLastError());
    }
  }
  return OCN_OK;
}

// ------------------------------------------------- grouped long-range term

struct LrGroup {
  struct TcLaunch {
    TcGroupMaps maps;
    TcParams p{};
    TcParams* d_tab = nullptr;
    int* d_tile0 = nullptr;
    int ninst = 0, grid = 0;
    size_t smem = 0;
  };
  std::vector<TcLaunch> g1, g2;
  // k-mesh transforms with B2 out, one launch per instantiation class
  struct FftClass {
    CubeFnB2Group f = nullptr;
    int kn = 0, tc = 0, th = 0, nctas = 0;
    size_t smem = 0;
    std::vector<FftGroupArgs> h;
    FftGroupArgs* d = nullptr;
  };
  std::vector<FftClass> fft;
  NormGroupArgs* d_norm[3] = {nullptr, nullptr, nullptr};
  int n = 0, nvmax = 1, nblk = 0;
};

std::string batch_group_refusal(const ocn_ctx* c) {
  if (c->dims.precision != OCN_PREC_MIXED || !c->mixed || !c->mixed->ready) return "not mixed precision";
  if (c->nspn != 1) return "spin-polarised";
  if (!c->mixed->cube) return "k-mesh without a cubic transform";
  if (!(c->sys.long_range && c->sys.nhflag[0] == 1)) return "long-range term off";
  if (c->sys.mult && c->sys.nhflag[4] == 1 && c->have_mult) return "multiplet term on";
  if (c->timing.on) return "timing on";
  return "";
}

void lr_group_destroy(LrGroup* g) {
  if (!g) return;
  for (auto* v : {&g->g1, &g->g2})
    for (auto& L : *v) {
      if (L.d_tab) cudaFree(L.d_tab);
      if (L.d_tile0) cudaFree(L.d_tile0);
    }
  for (auto& f : g->fft)
    if (f.d) cudaFree(f.d);
  for (int r = 0; r < 3; ++r)
    if (g->d_norm[r]) cudaFree(g->d_norm[r]);
  delete g;
}

namespace {

template <typename T>
int upload(ocn_ctx* c, T** d, const std::vector<T>& h) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(d), h.size() * sizeof(T));
  if (e == cudaSuccess) e = cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? OCN_OK : cuda_fail(c, e, "batched launch tables");
}

}  // namespace

// Launch plan of the long-range term and the normalisation of every member:
// the two contractions as persistent launches over the concatenated tile
// lists (TC_GROUP_MAX members each), the k-mesh transforms as one launch per
// (mesh, transforms per CTA, threads) class, the operand builders as one
// launch.  Every member keeps its own tiling, so its results are those of its
// own launches.
int lr_group_create(const std::vector<BatchMember>& mem, LrGroup** out) {
  *out = nullptr;
  if (mem.empty()) return OCN_ERR_ARG;
  ocn_ctx* c0 = mem[0].c;
  LrGroup* g = new (std::nothrow) LrGroup();
  if (!g) return set_err(c0, OCN_ERR_ALLOC, "host allocation failed");
  g->n = (int)mem.size();
  int ncol_max = 0;
  for (const BatchMember& b : mem) {
    ncol_max = std::max(ncol_max, b.c->mixed->ncol);
    g->nvmax = std::max(g->nvmax, b.nv);
    g->nblk = std::max(g->nblk, b.c->red_blocks);
  }
  const size_t a_bytes = (size_t)TC_BM * TC_BK * 2;
  const size_t stage_bytes = 2 * a_bytes + (size_t)ncol_max * TC_BK * 2;
  // deepest pipeline that still leaves room for the output staging
  const size_t room = std::min<size_t>(TC_SMEM_BUDGET, device_smem_optin(c0) - estg_bytes(ncol_max));
  int S = (int)std::min<size_t>(TC_MAX_STAGES, (room - 1024 - 256) / stage_bytes);
  if (S < 2) S = (int)std::min<size_t>(TC_MAX_STAGES, (TC_SMEM_BUDGET - 1024 - 256) / stage_bytes);
  uint32_t tcols = 32;
  while ((int)tcols < 2 * ncol_max) tcols <<= 1;
  int rc = OCN_OK;
  if ((rc = allow_max_smem(c0, k_lr_tc_group))) {
    lr_group_destroy(g);
    return rc;
  }
  for (int mode = 1; mode <= 2 && rc == OCN_OK; ++mode) {
    std::vector<LrGroup::TcLaunch>& dst = mode == 1 ? g->g1 : g->g2;
    for (size_t c0i = 0; c0i < mem.size() && rc == OCN_OK; c0i += TC_GROUP_MAX) {
      dst.emplace_back();
      LrGroup::TcLaunch& L = dst.back();
      std::vector<TcParams> tab;
      std::vector<int> tile0;
      int total = 0;
      const size_t end = std::min(mem.size(), c0i + TC_GROUP_MAX);
      for (size_t i = c0i; i < end; ++i) {
        const MixedLR* m = mem[i].c->mixed;
        TcParams q = mode == 1 ? m->g1 : m->g2;
        q.nv = mem[i].nv;
        q.koff = 0;
        q.spin = -1;
        tile0.push_back(total);
        total += q.ntiles;
        tab.push_back(q);
        const int j = (int)(i - c0i);
        L.maps.m[j][0] = mode == 1 ? m->tm_ua_hi : m->tm_ub_hi;
        L.maps.m[j][1] = mode == 1 ? m->tm_ua_lo : m->tm_ub_lo;
        L.maps.m[j][2] = mode == 1 ? m->tm_b1 : m->tm_b2;
      }
      tile0.push_back(total);
      L.ninst = (int)tab.size();
      L.p = tab[0];
      L.p.ntiles = total;
      L.p.ncol = ncol_max;
      L.p.stages = S;
      L.p.tcols = tcols;
      L.p.err = mem[c0i].c->mixed->d_err;
      L.grid = std::min(total, c0->sm_count);
      L.smem = 1024 + (size_t)S * stage_bytes + 256;
      bool want = false;
      for (size_t i = c0i; i < end; ++i) want = want || mem[i].c->mixed->cfg[6] != 0;
      L.p.estg = (want && L.smem + estg_bytes(ncol_max) <= device_smem_optin(c0)) ? 1 : 0;
      if (L.p.estg) L.smem += estg_bytes(ncol_max);
      if ((rc = upload(c0, &L.d_tab, tab)) == OCN_OK) rc = upload(c0, &L.d_tile0, tile0);
    }
  }
  // k-mesh transforms with the B2 rows out: one launch for every context
  for (size_t i = 0; i < mem.size() && rc == OCN_OK; ++i) {
    ocn_ctx* c = mem[i].c;
    const MixedLR* m = c->mixed;
    const int ntot = c->na * mem[i].nv;
    const int kn = c->dims.kmesh[0];
    const int tc = cube_tc(m, kn, c->na, ntot);
    const int th = m->cfg[5] ? m->cfg[5] : 128;
    LrGroup::FftClass* cls = nullptr;
    for (auto& f : g->fft)
      if (f.kn == kn && f.tc == tc && f.th == th) cls = &f;
    if (!cls) {
      g->fft.emplace_back();
      cls = &g->fft.back();
      cls->kn = kn;
      cls->tc = tc;
      cls->th = th;
      cls->smem = fft_b2_smem(kn, tc);
      OCN_CUBE_DISPATCH(k_fft_b2_cube_group, kn, tc, cls->f);
      if (!cls->f) rc = set_err(c0, OCN_ERR_UNSUPPORTED, "no cubic transform for this k-mesh");
      else rc = allow_max_smem(c0, cls->f);
    }
    cls->h.push_back(FftGroupArgs{m->phi, m->Wf, c->nx, tc, ntot, m->twf, m->b2, c->na, m->ncol, m->p2, cls->nctas});
    cls->nctas += c->nx * (ntot / tc);
  }
  for (auto& f : g->fft)
    if (rc == OCN_OK) rc = upload(c0, &f.d, f.h);
  // Lanczos stage 2 + normalisation + next psi operand, per buffer rotation
  for (int r = 0; r < 3 && rc == OCN_OK; ++r) {
    std::vector<NormGroupArgs> nt;
    for (const BatchMember& b : mem) {
      const ocn_ctx* c = b.c;
      const MixedLR* m = c->mixed;
      NormGroupArgs a;
      a.red1 = c->d_red;
      a.nblk = c->red_blocks;
      a.rstride = (size_t)4 * c->red_blocks;
      a.hbase = b.buf[(r + 2) % 3];
      a.pbase = b.buf[(r + 1) % 3];
      a.vstride = 2 * c->npsi;
      a.npsi = c->npsi;
      a.allow = c->d_allow_f;
      a.b1 = m->b1;
      a.nb = c->nb;
      a.nk = c->nk;
      a.na = c->na;
      a.ncol = m->ncol;
      a.p1 = m->p1;
      a.ra_base = b.ra;
      a.ia_base = b.ia;
      a.rb_base = b.rb;
      a.cstride = b.cstride;
      a.itp = c->d_iter;
      a.nv = b.nv;
      nt.push_back(a);
    }
    rc = upload(c0, &g->d_norm[r], nt);
  }
  if (rc != OCN_OK) {
    lr_group_destroy(g);
    return rc;
  }
  *out = g;
  return OCN_OK;
}

// Kernels one lr_group_apply + lr_group_norm launch.
int lr_group_launches(const LrGroup* g) { return (int)(g->g1.size() + g->g2.size() + g->fft.size()) + 1; }

int lr_group_apply(LrGroup* g, cudaStream_t s) {
  for (auto& L : g->g1)
    k_lr_tc_group<<<L.grid, TC_THREADS, L.smem, s>>>(L.maps, L.p, L.d_tab, L.d_tile0, L.ninst);
  for (auto& f : g->fft) f.f<<<f.nctas, f.th, f.smem, s>>>(f.d, (int)f.h.size());
  for (auto& L : g->g2)
    k_lr_tc_group<<<L.grid, TC_THREADS, L.smem, s>>>(L.maps, L.p, L.d_tab, L.d_tile0, L.ninst);
  return cudaGetLastError() == cudaSuccess ? OCN_OK : OCN_ERR_CUDA;
}

int lr_group_norm(LrGroup* g, int rot, cudaStream_t s) {
  k_norm_prep_group<<<dim3(g->nblk, g->nvmax, g->n), LZ_DF_THREADS, 0, s>>>(g->d_norm[rot]);
  return cudaGetLastError() == cudaSuccess ? OCN_OK : OCN_ERR_CUDA;
}

}  // namespace ocn
