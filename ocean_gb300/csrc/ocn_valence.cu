// ocn_valence.cu -- the valence BSE action and its Haydock recursion on one GPU.
//
//   H psi = E o psi + allow o [ 2 X(allow o psi) - D(allow o psi) ]
//
// X: exchange ("bubble", OCEAN2/OCEAN_bubble.f90:420-796); D: screened direct
// ("ladder", OCEAN2/OCEAN_ladder.f90:155-1004); order of OCEAN_xact's valence
// branch (OCEAN2/OCEAN_action.f90:521-600).  valence_ham_spin 1 or 2 (psi in 1
// or 4 spin blocks), one or two DFT spins, resonant pairs (nbw = 1).
//
// Both terms start from A(x,v,k) = sum_c con(x,c,k) psi(c,v,k) and end with
// out(c,v,k) = sum_x conj(con(x,c,k)) M(x,v,k), so one kernel builds A (and the
// exchange partials l_k(x) = sum_v conj(val) A), one projects
// M = 2 s(x) val - B back onto the pairs, and in between
//   exchange: l(x) = sum_k l_k(x); s = FFT_fwd[bubble o FFT_bwd[l]] on the x-mesh
//   direct:   per x (one CTA) and a range of y: T(y,k) = sum_v A(x,v,k)
//             conj(val(y,v,k)), FFT_fwd over k, times ladder(k,x,y), FFT_bwd,
//             and B(x,v,k) += sum_y T(y,k) val(y,v,k) -- T never leaves shared
//             memory (the reference stores all Nx*Ny*Nk of it).
// The direct term is the O(Nx^2 Nk) part: FP64 in OCN_PREC_FP64, FP32 (A, val,
// ladder, transforms, B) in OCN_PREC_MIXED; everything else is FP64.
//
// Device layouts: psi/E/allow (Nc,Nv,Nk) planes as in the reference;
// con [k][c][x] and val [k][v][x] interleaved complex (the reference's (x,c,k)
// order); valT [y][v][k] and the ladder [y][x][k] (the reference's
// ladder(k,x,y)) with k fastest for the transforms.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "ocn_internal.h"
#include "ocn_kmesh_dft.cuh"

namespace {

using ocn::C2;
using ocn::KmeshGeom;

constexpr int VAL_MAX_NV = 32;
constexpr int VAL_CC = 16;        // conduction bands staged per pass of kv_amat
constexpr int VAL_THREADS = 256;
constexpr int VAL_FIN_WARPS = VAL_THREADS / 32;

std::string g_val_create_err;

}  // namespace

struct ocn_val_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  size_t smem_optin = 0;
  ocn_val_dims dims{};
  int nc = 0, nv = 0, nk = 0, nx = 0;
  int nspn = 1, vspin = 1;  // DFT spins of the states; valence_ham_spin (vspin^2 psi blocks)
  size_t npsi = 0;          // all blocks
  size_t nb1 = 0;           // one block: Nc Nv Nk
  int mixed = 0;
  bool have_e = false, have_allow = false, have_states = false, have_bubble = false, have_ladder = false;
  bool ei_nonzero = false;
  double* d_er = nullptr;
  double* d_ei = nullptr;
  double* d_allow = nullptr;
  double2* d_con = nullptr;   // [k][c][x]
  double2* d_val = nullptr;   // [k][v][x]
  float2* d_con32 = nullptr;  // FP32 copies (mixed precision)
  float2* d_val32 = nullptr;
  void* d_valT = nullptr;     // [y][v][k], double2 or float2
  void* d_lad = nullptr;      // [y][x][k], double or float
  double* d_bub = nullptr;    // [x]
  double* d_fxc = nullptr;    // [x] ALDA kernel; set: the f_xc term is on (OCEAN_fxc_act)
  bool have_fxc = false;
  double2* d_twk = nullptr;   // exp(+2 pi i t / n_axis) for the k-mesh, [axis][t]
  float2* d_twk32 = nullptr;
  double2* d_twx = nullptr;   // same for the x-mesh
  double2* d_lp = nullptr;    // exchange partials [k][x]
  double2* d_s = nullptr;     // s(x)
  void* d_A = nullptr;        // [x][v][k] in the direct term's precision
  void* d_Bp = nullptr;       // [ys][k][v][x] in the direct term's precision
  double* d_vec = nullptr;    // 4 vectors of 2*npsi: in/psi, out/h, old, spare
  double* d_red = nullptr;
  double* d_coef = nullptr;
  int coef_cap = 0;
  int red_blocks = 1;
  int ytile = 1, ysplit = 1, yper = 1;
  int xper = 1;  // x-points per CTA of the cubic direct-term kernel
  size_t lad_smem = 0;
  long long launches = 0;
  std::string err;
};

namespace {

int vset_err(ocn_val_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_val_create_err = msg;
  return code;
}

int vcuda(ocn_val_ctx* c, cudaError_t e, const char* what) {
  return vset_err(c, OCN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VCUDA(c, call)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return vcuda(c, _e, #call);   \
  } while (0)

template <typename T>
int valloc(ocn_val_ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return OCN_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) return vset_err(c, OCN_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return OCN_OK;
}

// ------------------------------------------------------------------ kernels

// A(x,v,k) = sum_c con(x,c,k) (allow o psi)(c,v,k) (OCEAN_bubble.f90:521-530,
// OCEAN_ladder.f90:317-326) and the exchange partial
// l_k(x) = sum_v conj(val(x,v,k)) A(x,v,k) (OCEAN_bubble.f90:568-580), summed
// over the block's 8 k-points (in k order) into lp[k / 8][x].
// Block: 32 x-points by 8 k-points; lanes along x read con rows coalesced.
// R: arithmetic and state precision (FP32 copies of con/val in mixed mode).
template <typename R, int MAXV>
__global__ void __launch_bounds__(VAL_THREADS)
    kv_amat(const double* __restrict__ pr, const double* __restrict__ pi, const double* __restrict__ allow,
            const typename C2<R>::T* __restrict__ con, const typename C2<R>::T* __restrict__ val, int nc, int nv,
            int nk, int nx, double2* __restrict__ lp, typename C2<R>::T* __restrict__ A) {
  typedef typename C2<R>::T CT;
  extern __shared__ __align__(16) unsigned char amsm[];
  CT* qs = reinterpret_cast<CT*>(amsm);  // [kl][cl][v]
  __shared__ double2 lred[8][32];
  const int xl = threadIdx.x, kl = threadIdx.y;
  const int tid = kl * 32 + xl;
  const int x = blockIdx.x * 32 + xl, k0 = blockIdx.y * 8, k = k0 + kl;
  CT acc[MAXV];
#pragma unroll
  for (int v = 0; v < MAXV; ++v) {
    acc[v].x = (R)0;
    acc[v].y = (R)0;
  }
  for (int c0 = 0; c0 < nc; c0 += VAL_CC) {
    const int cn = min(VAL_CC, nc - c0);
    __syncthreads();
    for (int e = tid; e < 8 * VAL_CC * nv; e += VAL_THREADS) {
      const int kk = e / (VAL_CC * nv), r = e % (VAL_CC * nv);
      const int cl = r / nv, v = r % nv;
      CT q;
      q.x = (R)0;
      q.y = (R)0;
      if (k0 + kk < nk && cl < cn) {
        const size_t idx = (size_t)(c0 + cl) + (size_t)nc * (v + (size_t)nv * (k0 + kk));
        const double m = allow[idx];
        q.x = (R)(pr[idx] * m);
        q.y = (R)(pi[idx] * m);
      }
      qs[e] = q;
    }
    __syncthreads();
    if (x < nx && k < nk) {
      for (int cl = 0; cl < cn; ++cl) {
        const CT cv = con[((size_t)k * nc + c0 + cl) * nx + x];
        const CT* q = qs + (kl * VAL_CC + cl) * nv;
#pragma unroll
        for (int v = 0; v < MAXV; ++v)
          if (v < nv) {
            const CT qq = q[v];
            acc[v].x += cv.x * qq.x - cv.y * qq.y;
            acc[v].y += cv.y * qq.x + cv.x * qq.y;
          }
      }
    }
  }
  R lr = (R)0, li = (R)0;
  if (x < nx && k < nk) {
#pragma unroll
    for (int v = 0; v < MAXV; ++v)
      if (v < nv) {
        const CT vv = val[((size_t)k * nv + v) * nx + x];
        lr += vv.x * acc[v].x + vv.y * acc[v].y;
        li += vv.x * acc[v].y - vv.y * acc[v].x;
        A[((size_t)x * nv + v) * nk + k] = acc[v];
      }
  }
  lred[kl][xl] = make_double2((double)lr, (double)li);
  __syncthreads();
  if (kl == 0 && x < nx) {
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < 8; ++i) {
      sr += lred[i][xl].x;
      si += lred[i][xl].y;
    }
    lp[(size_t)blockIdx.y * nx + x] = make_double2(sr, si);
  }
}

// l(x) = sum_b lp[b][x] over the nkb k-blocks: 32 slices per x-point, each a
// strided sum in b order, then the slices in order.
__global__ void __launch_bounds__(1024) kv_bub_reduce(const double2* __restrict__ lp, int nkb, int nx,
                                                      double2* __restrict__ l) {
  __shared__ double2 part[32][33];
  const int xl = threadIdx.x, sl = threadIdx.y;
  const int x = blockIdx.x * 32 + xl;
  double sr = 0.0, si = 0.0;
  if (x < nx)
    for (int b = sl; b < nkb; b += 32) {
      const double2 t = lp[(size_t)b * nx + x];
      sr += t.x;
      si += t.y;
    }
  part[sl][xl] = make_double2(sr, si);
  __syncthreads();
  if (sl == 0 && x < nx) {
    double tr = 0.0, ti = 0.0;
    for (int i = 0; i < 32; ++i) {
      tr += part[i][xl].x;
      ti += part[i][xl].y;
    }
    l[x] = make_double2(tr, ti);
  }
}

// One pass along `ax` of a 3-D DFT over the whole mesh, one output element per
// thread (out of place): out(m) = sum_j in(j) w^(j m), w = exp(sgn 2 pi i / n_ax).
__device__ __forceinline__ void xmesh_pass(const double2* __restrict__ in, double2* __restrict__ out, const int n[3],
                                           int ax, const double2* __restrict__ tw, double sgn) {
  const int nx = n[0] * n[1] * n[2];
  const int st = ax == 2 ? 1 : (ax == 1 ? n[2] : n[1] * n[2]);
  const int na = n[ax];
  for (int o = threadIdx.x; o < nx; o += blockDim.x) {
    const int m = (o / st) % na;
    const double2* line = in + (o - m * st);
    double sr = 0.0, si = 0.0;
    int t = 0;
    for (int j = 0; j < na; ++j) {
      const double2 v = line[j * st];
      const double2 w = tw[t];
      const double wy = sgn * w.y;
      sr += v.x * w.x - v.y * wy;
      si += v.x * wy + v.y * w.x;
      t += m;
      if (t >= na) t -= na;
    }
    out[o] = make_double2(sr, si);
  }
}

// s = FFT_fwd[ bubble o FFT_bwd[ l ] ] on the x-mesh, neither normalised
// (OCEAN_bubble.f90:663-665; FFTW signs +1 backward, -1 forward,
// Modules/FFT_wrapper.f90:24-25).  One CTA of 1024 threads, ping-pong buffers.
// With fxc (the ALDA kernel, OCEAN_fxc_act, OCEAN_fxc.f90:250-253) the local
// term fxc(x) l(x) is added to s; without use_x only that term is formed.
__global__ void __launch_bounds__(1024) kv_bub_fft(double2* __restrict__ l, const double* __restrict__ bub,
                                                   const double* __restrict__ fxc, int use_x, const int3 mesh,
                                                   const double2* __restrict__ twg) {
  extern __shared__ double2 sm[];
  const int n[3] = {mesh.x, mesh.y, mesh.z};
  const int nx = n[0] * n[1] * n[2];
  double2* tw = sm;
  double2* b0 = sm + 3 * OCN_MAX_KDIM;
  double2* b1 = b0 + nx;
  if (!use_x) {  // the local term alone; each x read and written by one thread
    for (int x = threadIdx.x; x < nx; x += blockDim.x) {
      const double2 v = l[x];
      l[x] = make_double2(fxc[x] * v.x, fxc[x] * v.y);
    }
    return;
  }
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  for (int x = threadIdx.x; x < nx; x += blockDim.x) b0[x] = l[x];
  __syncthreads();
  xmesh_pass(b0, b1, n, 0, tw, 1.0);
  __syncthreads();
  xmesh_pass(b1, b0, n, 1, tw + OCN_MAX_KDIM, 1.0);
  __syncthreads();
  xmesh_pass(b0, b1, n, 2, tw + 2 * OCN_MAX_KDIM, 1.0);
  __syncthreads();
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    b1[x].x *= bub[x];
    b1[x].y *= bub[x];
  }
  __syncthreads();
  xmesh_pass(b1, b0, n, 0, tw, -1.0);
  __syncthreads();
  xmesh_pass(b0, b1, n, 1, tw + OCN_MAX_KDIM, -1.0);
  __syncthreads();
  xmesh_pass(b1, b0, n, 2, tw + 2 * OCN_MAX_KDIM, -1.0);
  __syncthreads();
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    double2 v = b0[x];
    if (fxc) {  // l[x] still holds this thread's input value
      const double2 u = l[x];
      v.x += fxc[x] * u.x;
      v.y += fxc[x] * u.y;
    }
    l[x] = v;
  }
}

// Direct term for the x-point of this CTA and the y-range blockIdx.y
// (OCEAN_ladder.f90:438-449 T, :596-624 transforms and ladder, :711-720 B).
// N > 0: cubic k-mesh N^3 (radix butterflies); N == 0: any mesh.
template <typename R, int N>
__global__ void __launch_bounds__(VAL_THREADS)
    kv_ladder(const typename C2<R>::T* __restrict__ A, const typename C2<R>::T* __restrict__ valT,
              const R* __restrict__ lad, typename C2<R>::T* __restrict__ Bp, int nv, int nk, int nx, int ytile,
              int yper, const KmeshGeom<R> g, int slab, const typename C2<R>::T* __restrict__ twg) {
  typedef typename C2<R>::T CT;
  extern __shared__ __align__(16) unsigned char vsm[];
  CT* tw = reinterpret_cast<CT*>(vsm);
  CT* As = tw + 3 * OCN_MAX_KDIM;
  CT* Bs = As + (size_t)nv * nk;
  CT* T = Bs + (size_t)nv * nk;
  const int x = blockIdx.x, ys = blockIdx.y;
  const int ybeg = ys * yper, yend = min(nx, ybeg + yper);
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  const CT* Ax = A + (size_t)x * nv * nk;
  for (int e = threadIdx.x; e < nv * nk; e += blockDim.x) {
    As[e] = Ax[e];
    CT z;
    z.x = (R)0;
    z.y = (R)0;
    Bs[e] = z;
  }
  auto kp = [&](int k) -> int {
    if constexpr (N > 0) return (k / N) * (N + 1) + k % N;
    else return ocn::kpad(g, k);
  };
  __syncthreads();
  for (int y0 = ybeg; y0 < yend; y0 += ytile) {
    const int ny = min(ytile, yend - y0);
    for (int e = threadIdx.x; e < ny * nk; e += blockDim.x) {
      const int yl = e / nk, k = e % nk;
      const CT* vt = valT + (size_t)(y0 + yl) * nv * nk + k;
      R sr = (R)0, si = (R)0;
      for (int v = 0; v < nv; ++v) {
        const CT a = As[v * nk + k], b = vt[(size_t)v * nk];
        sr += a.x * b.x + a.y * b.y;
        si += a.y * b.x - a.x * b.y;
      }
      CT t;
      t.x = sr;
      t.y = si;
      T[yl * slab + kp(k)] = t;
    }
    __syncthreads();
    KmeshGeom<R> gg = g;
    gg.na = ny;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      if constexpr (N > 0) ocn::cube_pass<R, N, 0>(T, ny, ax, tw + ax * OCN_MAX_KDIM, (R)-1);
      else ocn::dft_pass<R>(T, gg, ax, tw + ax * OCN_MAX_KDIM, (R)-1);
      __syncthreads();
    }
    for (int e = threadIdx.x; e < ny * nk; e += blockDim.x) {
      const int yl = e / nk, k = e % nk;
      const R w = lad[((size_t)(y0 + yl) * nx + x) * nk + k];
      CT& t = T[yl * slab + kp(k)];
      t.x *= w;
      t.y *= w;
    }
    __syncthreads();
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      if constexpr (N > 0) ocn::cube_pass<R, N, 0>(T, ny, ax, tw + ax * OCN_MAX_KDIM, (R)1);
      else ocn::dft_pass<R>(T, gg, ax, tw + ax * OCN_MAX_KDIM, (R)1);
      __syncthreads();
    }
    for (int e = threadIdx.x; e < nv * nk; e += blockDim.x) {
      const int v = e / nk, k = e % nk;
      CT acc = Bs[e];
      const CT* vt = valT + ((size_t)y0 * nv + v) * nk + k;
      for (int yl = 0; yl < ny; ++yl) {
        const CT t = T[yl * slab + kp(k)];
        const CT b = vt[(size_t)yl * nv * nk];
        acc.x += t.x * b.x - t.y * b.y;
        acc.y += t.y * b.x + t.x * b.y;
      }
      Bs[e] = acc;
    }
    __syncthreads();
  }
  const R inv = (R)1 / (R)nk;  // FFT_wrapper_single's backward normalisation
  for (int e = threadIdx.x; e < nv * nk; e += blockDim.x) {
    const int v = e / nk, k = e % nk;
    CT o = Bs[e];
    o.x *= inv;
    o.y *= inv;
    Bp[(((size_t)ys * nk + k) * nv + v) * nx + x] = o;
  }
}

// N consecutive complex values; FP32 lines of even length (16-byte aligned:
// every caller's offset is a multiple of N complex values) as 16-byte loads.
template <typename CT, int N>
__device__ __forceinline__ void load_line(const CT* __restrict__ p, CT (&v)[N]) {
  if constexpr (sizeof(CT) == 8 && N % 2 == 0) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
      const float4 t = __ldg(q + i);
      v[2 * i].x = t.x;
      v[2 * i].y = t.y;
      v[2 * i + 1].x = t.z;
      v[2 * i + 1].y = t.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j];
  }
}

// The direct term on a cubic k-mesh N^3 for X x-points per CTA (same
// arithmetic as kv_ladder, fewer shared-memory passes): the T build is fused
// with the forward transform along k3 (one val line serves all X x-points),
// the forward transform along k1, the ladder product and the backward
// transform along k1 share one pass in registers, and the backward transform
// along k3 is redone in registers by each thread of the B sum (FP32), whose
// (k1 k2 line, v) pairs stay in registers across the whole y-range.
// MAXC: (line, v) pairs per thread (N^2 nv <= MAXC * blockDim).
template <typename R, int N, int MAXC, int X>
__global__ void __launch_bounds__(VAL_THREADS, (sizeof(R) == 4 && X == 1) ? 4 : 2)
    kv_ladder_cube(const typename C2<R>::T* __restrict__ A, const typename C2<R>::T* __restrict__ valT,
                   const R* __restrict__ lad, typename C2<R>::T* __restrict__ Bp, int nv, int nx, int ytile, int yper,
                   const typename C2<R>::T* __restrict__ twg) {
  typedef typename C2<R>::T CT;
  constexpr int NK = N * N * N, NL = N * N, P3 = N + 1;
  constexpr int SLAB = ocn::cube_slab<CT>(N);
  // FP32: the last backward transform is redone by each of the nv threads of a
  // line in the B sum (saves a shared-memory pass); FP64 is FP64-pipe bound,
  // so there it stays one shared pass (85 ms against 104 ms per H psi)
  constexpr bool FUSE_K3 = sizeof(R) == 4;
  extern __shared__ __align__(16) unsigned char vsm[];
  CT* tw = reinterpret_cast<CT*>(vsm);
  CT* As = tw + 3 * OCN_MAX_KDIM;        // [xi][(v N + k3) NL + line]
  CT* T = As + (size_t)X * nv * NK;      // slab (yl X + xi)
  const int x0 = blockIdx.x * X, ys = blockIdx.y;
  const int ybeg = ys * yper, yend = min(nx, ybeg + yper);
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  // the lanes of the T build (consecutive k1 k2 lines) read consecutive words;
  // an x-point past the mesh (odd Nx) is staged as zeros and never stored
  for (int e = threadIdx.x; e < X * nv * NK; e += blockDim.x) {
    const int xi = e / (nv * NK), r = e % (nv * NK);
    const int vv = r / NK, k = r % NK;
    CT a;
    a.x = (R)0;
    a.y = (R)0;
    if (x0 + xi < nx) a = A[(size_t)(x0 + xi) * nv * NK + r];
    As[xi * nv * NK + (vv * N + k % N) * NL + k / N] = a;
  }
  const int ncomb = NL * nv;
  CT acc[MAXC][X][N];
#pragma unroll
  for (int q = 0; q < MAXC; ++q)
#pragma unroll
    for (int xi = 0; xi < X; ++xi)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        acc[q][xi][j].x = (R)0;
        acc[q][xi][j].y = (R)0;
      }
  __syncthreads();
  for (int y0 = ybeg; y0 < yend; y0 += ytile) {
    const int ny = min(ytile, yend - y0);
    // T(x, y, k) for a k3 line, then the forward transform along k3
    for (int li = threadIdx.x; li < ny * NL; li += blockDim.x) {
      const int yl = li / NL, ln = li % NL;
      const CT* vt = valT + (size_t)(y0 + yl) * nv * NK + ln * N;
      CT v[X][N];
#pragma unroll
      for (int xi = 0; xi < X; ++xi)
#pragma unroll
        for (int j = 0; j < N; ++j) {
          v[xi][j].x = (R)0;
          v[xi][j].y = (R)0;
        }
      for (int vv = 0; vv < nv; ++vv) {
        CT bl[N];
        load_line<CT, N>(vt + (size_t)vv * NK, bl);
#pragma unroll
        for (int xi = 0; xi < X; ++xi) {
          const CT* as = As + xi * nv * NK + ln;
#pragma unroll
          for (int j = 0; j < N; ++j) {
            const CT a = as[(vv * N + j) * NL], b = bl[j];
            v[xi][j].x += a.x * b.x + a.y * b.y;
            v[xi][j].y += a.y * b.x - a.x * b.y;
          }
        }
      }
#pragma unroll
      for (int xi = 0; xi < X; ++xi) {
        ocn::line_dft<CT, R, N>(v[xi], tw + 2 * OCN_MAX_KDIM, (R)-1);
        CT* p = T + (yl * X + xi) * SLAB + ln * P3;
#pragma unroll
        for (int j = 0; j < N; ++j) p[j] = v[xi][j];
      }
    }
    __syncthreads();
    ocn::cube_pass<R, N, 0>(T, ny * X, 1, tw + OCN_MAX_KDIM, (R)-1);
    __syncthreads();
    // forward along k1, times ladder(k, x, y), backward along k1
    for (int li = threadIdx.x; li < ny * X * NL; li += blockDim.x) {
      const int sl = li / NL, r = li % NL;
      const int yl = sl / X, xi = sl % X;
      const int k2 = r / N, k3 = r % N;
      CT* p = T + sl * SLAB + k2 * P3 + k3;
      const int xx = min(x0 + xi, nx - 1);  // a padding x-point reads a valid row and is never stored
      const R* w = lad + ((size_t)(y0 + yl) * nx + xx) * NK + r;
      CT v[N];
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = p[j * N * P3];
      ocn::line_dft<CT, R, N>(v, tw, (R)-1);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const R ww = w[j * NL];
        v[j].x *= ww;
        v[j].y *= ww;
      }
      ocn::line_dft<CT, R, N>(v, tw, (R)1);
#pragma unroll
      for (int j = 0; j < N; ++j) p[j * N * P3] = v[j];
    }
    __syncthreads();
    ocn::cube_pass<R, N, 0>(T, ny * X, 1, tw + OCN_MAX_KDIM, (R)1);
    __syncthreads();
    if constexpr (!FUSE_K3) {
      ocn::cube_pass<R, N, 0>(T, ny * X, 2, tw + 2 * OCN_MAX_KDIM, (R)1);
      __syncthreads();
    }
    // backward along k3 (in registers when fused), then B(x, v, k) += T(x, y, k) val(y, v, k)
#pragma unroll
    for (int q = 0; q < MAXC; ++q) {
      const int cb = threadIdx.x + q * VAL_THREADS;
      if (cb < ncomb) {
        const int ln = cb / nv, vv = cb % nv;
        for (int yl = 0; yl < ny; ++yl) {
          CT bl[N];
          load_line<CT, N>(valT + ((size_t)(y0 + yl) * nv + vv) * NK + ln * N, bl);
#pragma unroll
          for (int xi = 0; xi < X; ++xi) {
            const CT* p = T + (yl * X + xi) * SLAB + ln * P3;
            CT t[N];
#pragma unroll
            for (int j = 0; j < N; ++j) t[j] = p[j];
            if constexpr (FUSE_K3) ocn::line_dft<CT, R, N>(t, tw + 2 * OCN_MAX_KDIM, (R)1);
#pragma unroll
            for (int j = 0; j < N; ++j) {
              acc[q][xi][j].x += t[j].x * bl[j].x - t[j].y * bl[j].y;
              acc[q][xi][j].y += t[j].y * bl[j].x + t[j].x * bl[j].y;
            }
          }
        }
      }
    }
    __syncthreads();
  }
  const R inv = (R)1 / (R)NK;  // FFT_wrapper_single's backward normalisation
#pragma unroll
  for (int q = 0; q < MAXC; ++q) {
    const int cb = threadIdx.x + q * VAL_THREADS;
    if (cb < ncomb) {
      const int ln = cb / nv, vv = cb % nv;
#pragma unroll
      for (int xi = 0; xi < X; ++xi) {
        if (x0 + xi >= nx) continue;
#pragma unroll
        for (int j = 0; j < N; ++j) {
          CT o = acc[q][xi][j];
          o.x *= inv;
          o.y *= inv;
          Bp[(((size_t)ys * NK + ln * N + j) * nv + vv) * nx + x0 + xi] = o;
        }
      }
    }
  }
}

// out(c,v,k) = E o psi (conj E when backwards) + allow o sum_x conj(con(x,c,k))
// M(x,v,k), M = xpref s(x) val(x,v,k) - sum_ys B_ys(x,v,k) (OCEAN_bubble.f90:742-757
// with xpref = spin_prefac, OCEAN_ladder.f90:900-911 with -1, OCEAN_energies.f90:890-906).
// One CTA per k; a warp owns (c,v) outputs and its lanes run over x.
template <typename R>
__global__ void __launch_bounds__(VAL_THREADS)
    kv_final(const double* __restrict__ pr, const double* __restrict__ pi, const double* __restrict__ er,
             const double* __restrict__ ei, const double* __restrict__ allow, const typename C2<R>::T* __restrict__ con,
             const typename C2<R>::T* __restrict__ val, const double2* __restrict__ s,
             const typename C2<R>::T* __restrict__ Bp, int nysplit, int nc, int nv, int nk, int nx, int xchunk,
             int use_e, int use_x, int use_d, int backwards, double xpref, double* __restrict__ outr,
             double* __restrict__ outi) {
  typedef typename C2<R>::T CT;
  extern __shared__ double2 fsm[];
  double2* accs = fsm;                                   // [c + nc v]
  CT* M = reinterpret_cast<CT*>(fsm + (size_t)nc * nv);  // [v][xl]
  const int k = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nout = nc * nv;
  for (int o = threadIdx.x; o < nout; o += blockDim.x) accs[o] = make_double2(0.0, 0.0);
  if (use_x || use_d) {
    for (int x0 = 0; x0 < nx; x0 += xchunk) {
      const int xn = min(xchunk, nx - x0);
      __syncthreads();
      for (int e = threadIdx.x; e < nv * xn; e += blockDim.x) {
        const int v = e / xn, xl = e % xn, x = x0 + xl;
        R mr = (R)0, mi = (R)0;
        if (use_x) {
          const CT vv = val[((size_t)k * nv + v) * nx + x];
          const double2 sd = s[x];
          const R sx = (R)sd.x, sy = (R)sd.y;
          mr = (R)xpref * (sx * vv.x - sy * vv.y);
          mi = (R)xpref * (sy * vv.x + sx * vv.y);
        }
        if (use_d)
          for (int ys = 0; ys < nysplit; ++ys) {
            const CT b = Bp[(((size_t)ys * nk + k) * nv + v) * nx + x];
            mr -= b.x;
            mi -= b.y;
          }
        CT mm;
        mm.x = mr;
        mm.y = mi;
        M[(size_t)v * xchunk + xl] = mm;
      }
      __syncthreads();
      for (int o = warp; o < nout; o += VAL_FIN_WARPS) {
        const int c = o % nc, v = o / nc;
        const CT* cr = con + ((size_t)k * nc + c) * nx + x0;
        const CT* mv = M + (size_t)v * xchunk;
        R pr_ = (R)0, pi_ = (R)0;
        for (int xl = lane; xl < xn; xl += 32) {
          const CT cc = cr[xl], m = mv[xl];
          pr_ += cc.x * m.x + cc.y * m.y;
          pi_ += cc.x * m.y - cc.y * m.x;
        }
        double sr = (double)pr_, si = (double)pi_;
        for (int off = 16; off > 0; off >>= 1) {
          sr += __shfl_down_sync(0xffffffffu, sr, off);
          si += __shfl_down_sync(0xffffffffu, si, off);
        }
        if (lane == 0) {
          accs[o].x += sr;
          accs[o].y += si;
        }
      }
    }
  }
  __syncthreads();
  for (int o = threadIdx.x; o < nout; o += blockDim.x) {
    const int c = o % nc, v = o / nc;
    const size_t idx = (size_t)c + (size_t)nc * (v + (size_t)nv * k);
    double hr = 0.0, hi = 0.0;
    if (use_e) {
      const double a = er[idx], b = ei ? ei[idx] : 0.0, qr = pr[idx], qi = pi[idx];
      if (backwards) {
        hr = a * qr + b * qi;
        hi = a * qi - b * qr;
      } else {
        hr = a * qr - b * qi;
        hi = a * qi + b * qr;
      }
    }
    const double m = allow[idx];
    outr[idx] = hr + m * accs[o].x;
    outi[idx] = hi + m * accs[o].y;
  }
}

// planes (x, i, k) -> interleaved [k][i][x] (same order) and, for val, the
// transposed copy [x][i][k] used by the direct term.
__global__ void kv_interleave(const double* __restrict__ re, const double* __restrict__ im, size_t n,
                              double2* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = make_double2(re[i], im[i]);
}

template <typename R>
__global__ void kv_transpose_val(const double2* __restrict__ val, int nv, int nk, int nx,
                                 typename C2<R>::T* __restrict__ valT) {
  const size_t n = (size_t)nx * nv * nk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk);
    const size_t r = i / nk;
    const int v = (int)(r % nv);
    const int y = (int)(r / nv);
    const double2 t = val[((size_t)k * nv + v) * nx + y];
    typename C2<R>::T o;
    o.x = (R)t.x;
    o.y = (R)t.y;
    valT[i] = o;
  }
}

__global__ void kv_to_float(const double* __restrict__ in, size_t n, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// ------------------------------------------------------- Lanczos kernels
// ocean_hay_ab_twoterm (OCEAN_haydock.f90:824-938) in three stages; every block
// re-adds the block partials in the same fixed order.

__device__ __forceinline__ void kv_block_pair(double a, double b, double* red) {
  __shared__ double sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = a;
    sh[1][w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      s0 += sh[0][i];
      s1 += sh[1][i];
    }
    red[2 * blockIdx.x] = s0;
    red[2 * blockIdx.x + 1] = s1;
  }
}

__device__ __forceinline__ void kv_sum_pairs(const double* red, int nb, double* s0, double* s1) {
  __shared__ double sh[2][32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += red[2 * i];
    b += red[2 * i + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = a;
    sh[1][w] = b;
  }
  __syncthreads();
  double ta = 0.0, tb = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
    ta += sh[0][i];
    tb += sh[1][i];
  }
  *s0 = ta;
  *s1 = tb;
}

// h -= b_{i-1} old; partial <h|psi> = sum conj(h) psi (OCEAN_psi.f90:2029-2034)
__global__ void __launch_bounds__(VAL_THREADS)
    kv_lz1(double* __restrict__ h, const double* __restrict__ old, const double* __restrict__ psi, size_t n,
           const double* __restrict__ rb, int it, double* __restrict__ red) {
  const double bm = it > 0 ? -rb[it - 1] : 0.0;
  double dr = 0.0, di = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double hr = h[e] + bm * old[e], hi = h[n + e] + bm * old[n + e];
    h[e] = hr;
    h[n + e] = hi;
    const double qr = psi[e], qi = psi[n + e];
    dr += hr * qr + hi * qi;
    di += hr * qi - hi * qr;
  }
  kv_block_pair(dr, di, red);
}

// a_{i-1} = Re<h|psi>; h -= a psi; partial |h|^2
__global__ void __launch_bounds__(VAL_THREADS)
    kv_lz2(const double* __restrict__ red1, int nb, double* __restrict__ h, const double* __restrict__ psi,
           size_t n, double* __restrict__ ra, double* __restrict__ ia, int it, double* __restrict__ red2) {
  double a, ai;
  kv_sum_pairs(red1, nb, &a, &ai);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ra[it - 1] = a;
    ia[it - 1] = ai;
  }
  const double am = -a;
  double s = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double r = h[e] + am * psi[e], i = h[n + e] + am * psi[n + e];
    h[e] = r;
    h[n + e] = i;
    s += r * r + i * i;
  }
  __syncthreads();
  kv_block_pair(s, 0.0, red2);
}

// b_i = sqrt(sum); psi_new = h / b_i in place
__global__ void __launch_bounds__(VAL_THREADS)
    kv_lz3(const double* __restrict__ red2, int nb, double* __restrict__ h, size_t n, double* __restrict__ rb,
           int it) {
  double bb, dummy;
  kv_sum_pairs(red2, nb, &bb, &dummy);
  const double b = sqrt(bb);
  if (blockIdx.x == 0 && threadIdx.x == 0) rb[it] = b;
  const double inv = 1.0 / b;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < 2 * n; e += (size_t)gridDim.x * blockDim.x)
    h[e] *= inv;
}

// ---------------------------------------------------------------- host side

int grid_for(size_t n, int threads, int cap) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + threads - 1) / threads, (size_t)cap));
}

void twiddles(const int n3[3], double2 out[3][OCN_MAX_KDIM]) {
  const double pi = 3.1415926535897932384626433832795;
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < OCN_MAX_KDIM; ++t)
      out[a][t] = t < n3[a] ? make_double2(cos(2.0 * pi * t / n3[a]), sin(2.0 * pi * t / n3[a]))
                            : make_double2(0.0, 0.0);
}

bool cubic(const int m[3]) { return m[0] == m[1] && m[1] == m[2]; }
bool cube_kernel_n(int n) { return n == 2 || n == 3 || n == 4 || n == 5 || n == 6 || n == 8; }

template <typename R>
size_t ladder_slab(const ocn_val_ctx* c) {
  if (cubic(c->dims.kmesh) && cube_kernel_n(c->dims.kmesh[0]))
    return (size_t)ocn::cube_slab<typename C2<R>::T>(c->dims.kmesh[0]);
  return (size_t)c->dims.kmesh[0] * c->dims.kmesh[1] * (c->dims.kmesh[2] + 1);
}

// the fused cubic kernel applies when the mesh is a supported cube and each
// thread owns at most two (line, v) pairs
bool use_cube_kernel(const ocn_val_ctx* c) {
  const int n = c->dims.kmesh[0];
  return cubic(c->dims.kmesh) && cube_kernel_n(n) && n * n * c->nv <= 2 * VAL_THREADS;
}

template <typename R>
size_t ladder_smem(const ocn_val_ctx* c, int ytile) {
  if (use_cube_kernel(c))  // X x-points' A and ytile * X transforms; B sums live in registers
    return sizeof(typename C2<R>::T) * (3 * OCN_MAX_KDIM + (size_t)c->xper * c->nv * c->nk +
                                        (size_t)ytile * c->xper * ladder_slab<R>(c));
  return sizeof(typename C2<R>::T) *
         (3 * OCN_MAX_KDIM + 2 * (size_t)c->nv * c->nk + (size_t)ytile * ladder_slab<R>(c));
}

template <typename R>
using LadderFn = void (*)(const typename C2<R>::T*, const typename C2<R>::T*, const R*, typename C2<R>::T*, int,
                          int, int, int, int, const KmeshGeom<R>, int, const typename C2<R>::T*);

template <typename R>
using LadderCubeFn = void (*)(const typename C2<R>::T*, const typename C2<R>::T*, const R*, typename C2<R>::T*,
                              int, int, int, int, const typename C2<R>::T*);

template <typename R, int N>
LadderCubeFn<R> cube_fn2(const ocn_val_ctx* c) {
  const bool one = N * N * c->nv <= VAL_THREADS;
  if (c->xper == 2) return one ? kv_ladder_cube<R, N, 1, 2> : kv_ladder_cube<R, N, 2, 2>;
  return one ? kv_ladder_cube<R, N, 1, 1> : kv_ladder_cube<R, N, 2, 1>;
}

template <typename R>
LadderCubeFn<R> ladder_cube_fn(const ocn_val_ctx* c) {
  switch (c->dims.kmesh[0]) {
    case 2: return cube_fn2<R, 2>(c);
    case 3: return cube_fn2<R, 3>(c);
    case 4: return cube_fn2<R, 4>(c);
    case 5: return cube_fn2<R, 5>(c);
    case 6: return cube_fn2<R, 6>(c);
    case 8: return cube_fn2<R, 8>(c);
  }
  return nullptr;
}

template <typename R>
LadderFn<R> ladder_fn(const ocn_val_ctx* c) {
  if (cubic(c->dims.kmesh)) switch (c->dims.kmesh[0]) {
      case 2: return kv_ladder<R, 2>;
      case 3: return kv_ladder<R, 3>;
      case 4: return kv_ladder<R, 4>;
      case 5: return kv_ladder<R, 5>;
      case 6: return kv_ladder<R, 6>;
      case 8: return kv_ladder<R, 8>;
    }
  return kv_ladder<R, 0>;
}

// The dynamic shared-memory limit of a kernel is process-wide state of the
// device, shared by every context. It is raised once to the device's opt-in
// maximum (less the kernel's static shared memory) and never lowered, so a
// context created later with smaller sizes cannot take room away from an
// earlier, larger one; each launch still asks only for what it needs.
cudaError_t raise_smem_limit(const void* fn, size_t optin) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, fn);
  if (e != cudaSuccess) return e;
  const size_t room = optin > a.sharedSizeBytes ? optin - a.sharedSizeBytes : 0;
  if ((size_t)a.maxDynamicSharedSizeBytes >= room) return cudaSuccess;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room);
}

// y-tile from the shared-memory budget (two CTAs per SM where it fits), and
// enough y-ranges per x-point for about two waves of CTAs.
template <typename R>
int plan_ladder(ocn_val_ctx* c) {
  int ytile = 16;
  // cubic kernel: in FP32 two x-points per CTA and the largest y-tile that
  // leaves two CTAs per SM (measured on the 8^3 k-mesh, 10^3 x-mesh case: 5.9 ms
  // per H psi with one x-point and 56 KB, 5.2 ms with two and 56 KB, 5.0 ms with
  // two and 110 KB); in FP64 two x-points spill registers (85 -> 104 ms), so one
  c->xper = (use_cube_kernel(c) && c->nx >= 2 && sizeof(R) == 4) ? 2 : 1;
  const size_t target = std::min<size_t>(c->smem_optin, 110 * 1024);
  // two x-points' A must fit with at least a one-y tile, else one x-point per CTA
  if (c->xper == 2 && ladder_smem<R>(c, 1) > c->smem_optin) c->xper = 1;
  while (ytile > 1 && ladder_smem<R>(c, ytile) > target) --ytile;
  if (ladder_smem<R>(c, ytile) > c->smem_optin)
    return vset_err(c, OCN_ERR_UNSUPPORTED,
                    "ocn_val: Nv*Nk too large for the direct-term kernel's shared memory");
  c->ytile = ytile;
  c->lad_smem = ladder_smem<R>(c, ytile);
  const bool cube = use_cube_kernel(c);
  const void* fn = cube ? (const void*)ladder_cube_fn<R>(c) : (const void*)ladder_fn<R>(c);
  cudaError_t e = raise_smem_limit(fn, c->smem_optin);
  if (e != cudaSuccess) return vcuda(c, e, "cudaFuncSetAttribute(kv_ladder)");
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, VAL_THREADS, c->lad_smem);
  if (e != cudaSuccess) return vcuda(c, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(kv_ladder)");
  // y-ranges per x-point: the split (up to 8, ranges no shorter than a tile)
  // whose CTA count fills the last wave best
  const double slots = (double)std::max(1, per_sm) * c->sm_count;
  const int maxsplit = std::max(1, std::min(8, c->nx / ytile));
  const int nxb = (c->nx + c->xper - 1) / c->xper;
  int best = 1;
  double best_eff = 0.0;
  for (int sp = 1; sp <= maxsplit; ++sp) {
    const double waves = (double)nxb * sp / slots;
    const double eff = waves / std::ceil(waves);
    if (eff > best_eff + 0.02) {
      best_eff = eff;
      best = sp;
    }
  }
  c->yper = (c->nx + best - 1) / best;
  c->ysplit = (c->nx + c->yper - 1) / c->yper;
  return OCN_OK;
}

size_t final_xchunk(const ocn_val_ctx* c) {
  const size_t outs = sizeof(double2) * (size_t)c->nc * c->nv;
  const size_t budget = outs < 48 * 1024 ? 64 * 1024 - outs : 16 * 1024;
  size_t xc = budget / (sizeof(double2) * c->nv);
  xc = std::max<size_t>(32, std::min<size_t>(xc, (size_t)c->nx));
  return xc;
}

size_t final_smem(const ocn_val_ctx* c) {
  const size_t ct = c->mixed ? sizeof(float2) : sizeof(double2);
  return sizeof(double2) * (size_t)c->nc * c->nv + ct * (size_t)c->nv * final_xchunk(c);
}

size_t bub_fft_smem(const ocn_val_ctx* c) { return sizeof(double2) * (3 * OCN_MAX_KDIM + 2 * (size_t)c->nx); }

int check_ready(ocn_val_ctx* c, const int flags[3]) {
  if (flags[0] && !c->have_e) return vset_err(c, OCN_ERR_STATE, "ocn_val: energies not set");
  if (!c->have_allow) return vset_err(c, OCN_ERR_STATE, "ocn_val: allow mask not set");
  if ((flags[1] || flags[2]) && !c->have_states) return vset_err(c, OCN_ERR_STATE, "ocn_val: states not set");
  if (flags[1] && !c->have_bubble) return vset_err(c, OCN_ERR_STATE, "ocn_val: bubble not set");
  if (flags[2] && !c->have_ladder) return vset_err(c, OCN_ERR_STATE, "ocn_val: ladder not set");
  if (c->have_fxc && !c->have_states) return vset_err(c, OCN_ERR_STATE, "ocn_val: states not set");
  return OCN_OK;
}

// psi holds vspin^2 blocks in the order ibeta = (i - 1) vspin + j of
// OCEAN_ladder_act (OCEAN_ladder.f90:118-133; i the valence spin, j the
// conduction spin, each DFT spin = min(spin, nspn)).  The direct term acts on
// every block; the exchange sums the same-spin blocks (i, i) into one l and
// feeds s back to each of them with spin_prefac 2 (one spin) or 1 (two),
// OCEAN_bubble.f90:465-470,509-760.
template <typename R>
int apply_impl(ocn_val_ctx* c, const double* d_in, double* d_out, const int flags[3], int backwards) {
  typedef typename C2<R>::T CT;
  const size_t n = c->npsi, nb1 = c->nb1;
  const int vs = c->vspin, ns = c->nspn;
  const int use_e = flags[0], use_x = flags[1], use_d = flags[2];
  const int use_f = c->have_fxc ? 1 : 0;  // aldaf: on whenever the kernel is set
  const int use_l = use_x || use_f;       // the exchange-like terms need l(x)
  const size_t nxk = (size_t)c->nx * c->nk;
  const size_t lp_blk = (size_t)c->nx * ((c->nk + 7) / 8), bp_blk = nxk * c->nv * c->ysplit;
  CT* A = static_cast<CT*>(c->d_A);
  CT* Bp = static_cast<CT*>(c->d_Bp);
  const CT* con0 = c->mixed ? reinterpret_cast<const CT*>(c->d_con32) : reinterpret_cast<const CT*>(c->d_con);
  const CT* val0 = c->mixed ? reinterpret_cast<const CT*>(c->d_val32) : reinterpret_cast<const CT*>(c->d_val);
  const CT* valT0 = static_cast<const CT*>(c->d_valT);
  auto con_s = [&](int sp) { return con0 + (size_t)sp * nxk * c->nc; };
  auto val_s = [&](int sp) { return val0 + (size_t)sp * nxk * c->nv; };
  auto valT_s = [&](int sp) { return valT0 + (size_t)sp * nxk * c->nv; };
  for (int iv = 0; iv < vs; ++iv)
    for (int jc = 0; jc < vs; ++jc) {
      const int b = iv * vs + jc;
      const bool diag = iv == jc;
      if (!(use_d || (use_l && diag))) continue;
      const int sc = std::min(jc, ns - 1), sv = std::min(iv, ns - 1);
      // exchange partials of a same-spin block in slot iv; other blocks' go to the spare slot vs
      double2* lp = c->d_lp + (diag ? iv : vs) * lp_blk;
      const double* pr = d_in + b * nb1;
      const double* pi = d_in + n + b * nb1;
      const double* al = c->d_allow + b * nb1;
      dim3 blk(32, 8), grd((c->nx + 31) / 32, (c->nk + 7) / 8);
      const size_t sm = sizeof(CT) * 8 * VAL_CC * c->nv;
      if (c->nv <= 4)
        kv_amat<R, 4><<<grd, blk, sm, c->stream>>>(pr, pi, al, con_s(sc), val_s(sv), c->nc, c->nv, c->nk, c->nx,
                                                   lp, A);
      else if (c->nv <= 8)
        kv_amat<R, 8><<<grd, blk, sm, c->stream>>>(pr, pi, al, con_s(sc), val_s(sv), c->nc, c->nv, c->nk, c->nx,
                                                   lp, A);
      else if (c->nv <= 16)
        kv_amat<R, 16><<<grd, blk, sm, c->stream>>>(pr, pi, al, con_s(sc), val_s(sv), c->nc, c->nv, c->nk, c->nx,
                                                    lp, A);
      else
        kv_amat<R, 32><<<grd, blk, sm, c->stream>>>(pr, pi, al, con_s(sc), val_s(sv), c->nc, c->nv, c->nk, c->nx,
                                                    lp, A);
      ++c->launches;
      VCUDA(c, cudaGetLastError());
      if (use_d) {
        KmeshGeom<R> g = ocn::kmesh_geom<R>(c->dims.kmesh, c->ytile);
        g.slab = (int)ladder_slab<R>(c);
        const CT* tw;
        if constexpr (sizeof(R) == 4) tw = c->d_twk32;
        else tw = c->d_twk;
        if (use_cube_kernel(c))
          ladder_cube_fn<R>(c)<<<dim3((c->nx + c->xper - 1) / c->xper, c->ysplit), VAL_THREADS, c->lad_smem,
                                 c->stream>>>(A, valT_s(sv), static_cast<const R*>(c->d_lad), Bp + b * bp_blk, c->nv,
                                              c->nx, c->ytile, c->yper, tw);
        else
          ladder_fn<R>(c)<<<dim3(c->nx, c->ysplit), VAL_THREADS, c->lad_smem, c->stream>>>(
              A, valT_s(sv), static_cast<const R*>(c->d_lad), Bp + b * bp_blk, c->nv, c->nk, c->nx, c->ytile,
              c->yper, g, g.slab, tw);
        ++c->launches;
        VCUDA(c, cudaGetLastError());
      }
    }
  if (use_l) {
    kv_bub_reduce<<<(c->nx + 31) / 32, dim3(32, 32), 0, c->stream>>>(c->d_lp, vs * ((c->nk + 7) / 8), c->nx,
                                                                      c->d_s);
    kv_bub_fft<<<1, 1024, bub_fft_smem(c), c->stream>>>(
        c->d_s, c->d_bub, use_f ? c->d_fxc : nullptr, use_x,
        make_int3(c->dims.xmesh[0], c->dims.xmesh[1], c->dims.xmesh[2]), c->d_twx);
    c->launches += 2;
    VCUDA(c, cudaGetLastError());
  }
  const int xc = (int)final_xchunk(c);
  const size_t fsm = final_smem(c);
  const double xpref = vs == 1 ? 2.0 : 1.0;
  for (int iv = 0; iv < vs; ++iv)
    for (int jc = 0; jc < vs; ++jc) {
      const int b = iv * vs + jc;
      const int sc = std::min(jc, ns - 1), sv = std::min(iv, ns - 1);
      kv_final<R><<<c->nk, VAL_THREADS, fsm, c->stream>>>(
          d_in + b * nb1, d_in + n + b * nb1, c->d_er + b * nb1, c->ei_nonzero ? c->d_ei + b * nb1 : nullptr,
          c->d_allow + b * nb1, con_s(sc), val_s(sv), c->d_s, Bp + b * bp_blk, c->ysplit, c->nc, c->nv, c->nk,
          c->nx, xc, use_e, use_l && iv == jc, use_d, backwards, xpref, d_out + b * nb1, d_out + n + b * nb1);
      ++c->launches;
      VCUDA(c, cudaGetLastError());
    }
  return OCN_OK;
}

int apply_dev(ocn_val_ctx* c, const double* d_in, double* d_out, const int flags[3], int backwards) {
  if (int rc = check_ready(c, flags)) return rc;
  return c->mixed ? apply_impl<float>(c, d_in, d_out, flags, backwards)
                  : apply_impl<double>(c, d_in, d_out, flags, backwards);
}

int upload(ocn_val_ctx* c, void* dst, const void* src, size_t bytes) {
  VCUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  return OCN_OK;
}

}  // namespace

extern "C" {

int ocn_val_create(const ocn_val_dims* d, ocn_val_ctx** out) {
  if (!d || !out) return vset_err(nullptr, OCN_ERR_ARG, "null argument");
  *out = nullptr;
  if (d->nc < 1 || d->nv < 1 || d->nv > VAL_MAX_NV)
    return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_create: need nc >= 1 and 1 <= nv <= 32");
  for (int i = 0; i < 3; ++i) {
    if (d->kmesh[i] < 1 || d->kmesh[i] > OCN_MAX_KDIM || d->xmesh[i] < 1 || d->xmesh[i] > OCN_MAX_KDIM)
      return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_create: mesh extents must be in 1..32");
  }
  if (d->precision != OCN_PREC_FP64 && d->precision != OCN_PREC_MIXED)
    return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_create: unknown precision");
  if (d->nspn < 0 || d->nspn > 2 || d->vspin < 0 || d->vspin > 2)
    return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_create: nspn and vspin must be 1 or 2");
  ocn_val_ctx* c = new (std::nothrow) ocn_val_ctx();
  if (!c) return vset_err(nullptr, OCN_ERR_ALLOC, "host allocation failed");
  auto fail = [&](int rc) {
    g_val_create_err = c->err;
    ocn_val_destroy(c);
    return rc;
  };
  c->dims = *d;
  c->device = d->device;
  c->nc = d->nc;
  c->nv = d->nv;
  c->nk = d->kmesh[0] * d->kmesh[1] * d->kmesh[2];
  c->nx = d->xmesh[0] * d->xmesh[1] * d->xmesh[2];
  c->nspn = d->nspn > 1 ? 2 : 1;
  c->vspin = d->vspin > 1 ? 2 : 1;
  c->nb1 = (size_t)c->nc * c->nv * c->nk;
  c->npsi = c->nb1 * c->vspin * c->vspin;
  c->mixed = d->precision == OCN_PREC_MIXED;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(vcuda(c, e, "cudaSetDevice"));
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(vcuda(c, e, "cudaStreamCreate"));
  int optin = 0;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  c->smem_optin = (size_t)optin;
  c->red_blocks = (int)std::min<size_t>(2 * (size_t)c->sm_count, std::max<size_t>(1, (c->npsi + 511) / 512));
  const size_t cs = c->mixed ? sizeof(float2) : sizeof(double2);
  const size_t rs = c->mixed ? sizeof(float) : sizeof(double);
  int rc = c->mixed ? plan_ladder<float>(c) : plan_ladder<double>(c);
  if (rc) return fail(rc);
  const size_t nxk = (size_t)c->nx * c->nk;
  if ((rc = valloc(c, &c->d_er, c->npsi)) || (rc = valloc(c, &c->d_ei, c->npsi)) ||
      (rc = valloc(c, &c->d_allow, c->npsi)) || (rc = valloc(c, &c->d_con, nxk * c->nc * c->nspn)) ||
      (rc = valloc(c, &c->d_val, nxk * c->nv * c->nspn)) ||
      (rc = valloc(c, reinterpret_cast<char**>(&c->d_valT), nxk * c->nv * c->nspn * cs)) ||
      (rc = valloc(c, reinterpret_cast<char**>(&c->d_lad), nxk * c->nx * rs)) ||
      (rc = valloc(c, &c->d_bub, c->nx)) || (rc = valloc(c, &c->d_fxc, c->nx)) || (rc = valloc(c, &c->d_twk, 3 * OCN_MAX_KDIM)) ||
      (rc = valloc(c, &c->d_twk32, 3 * OCN_MAX_KDIM)) || (rc = valloc(c, &c->d_twx, 3 * OCN_MAX_KDIM)) ||
      (rc = valloc(c, &c->d_lp, (size_t)(c->vspin + 1) * c->nx * ((c->nk + 7) / 8))) ||
      (rc = valloc(c, &c->d_s, c->nx)) || (rc = valloc(c, reinterpret_cast<char**>(&c->d_A), nxk * c->nv * cs)) ||
      (rc = valloc(c, reinterpret_cast<char**>(&c->d_Bp),
                   nxk * c->nv * c->ysplit * cs * c->vspin * c->vspin)) ||
      (rc = valloc(c, &c->d_vec, 8 * c->npsi)) || (rc = valloc(c, &c->d_red, 4 * (size_t)c->red_blocks)))
    return fail(rc);
  if (c->mixed && ((rc = valloc(c, &c->d_con32, nxk * c->nc * c->nspn)) ||
                   (rc = valloc(c, &c->d_val32, nxk * c->nv * c->nspn))))
    return fail(rc);
  double2 twk[3][OCN_MAX_KDIM], twx[3][OCN_MAX_KDIM];
  float2 twk32[3][OCN_MAX_KDIM];
  twiddles(d->kmesh, twk);
  twiddles(d->xmesh, twx);
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < OCN_MAX_KDIM; ++t) twk32[a][t] = make_float2((float)twk[a][t].x, (float)twk[a][t].y);
  if ((rc = upload(c, c->d_twk, twk, sizeof(twk))) || (rc = upload(c, c->d_twx, twx, sizeof(twx))) ||
      (rc = upload(c, c->d_twk32, twk32, sizeof(twk32))))
    return fail(rc);
  cudaMemsetAsync(c->d_ei, 0, sizeof(double) * c->npsi, c->stream);
  if (bub_fft_smem(c) > c->smem_optin)
    return fail(vset_err(c, OCN_ERR_UNSUPPORTED, "ocn_val_create: x-mesh too large for the exchange transform"));
  e = raise_smem_limit((const void*)kv_bub_fft, c->smem_optin);
  if (e != cudaSuccess) return fail(vcuda(c, e, "cudaFuncSetAttribute(kv_bub_fft)"));
  // dynamic + 4 KB static above the default 48 KB: Nv > 22, the 32-wide instantiation
  if (sizeof(double2) * 8 * VAL_CC * c->nv + 4096 > c->smem_optin && !c->mixed)
    return fail(vset_err(c, OCN_ERR_UNSUPPORTED, "ocn_val_create: Nv too large for the pair contraction"));
  e = raise_smem_limit((const void*)kv_amat<double, 32>, c->smem_optin);
  if (e != cudaSuccess) return fail(vcuda(c, e, "cudaFuncSetAttribute(kv_amat)"));
  const size_t fsm = final_smem(c);
  if (fsm > c->smem_optin) return fail(vset_err(c, OCN_ERR_UNSUPPORTED, "ocn_val_create: Nc*Nv too large"));
  e = raise_smem_limit(c->mixed ? (const void*)kv_final<float> : (const void*)kv_final<double>, c->smem_optin);
  if (e != cudaSuccess) return fail(vcuda(c, e, "cudaFuncSetAttribute(kv_final)"));
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(vcuda(c, e, "ocn_val_create"));
  *out = c;
  return OCN_OK;
}

int ocn_val_destroy(ocn_val_ctx* c) {
  if (!c) return OCN_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* bufs[] = {c->d_er, c->d_ei, c->d_allow, c->d_con, c->d_val, c->d_con32, c->d_val32, c->d_valT, c->d_lad, c->d_bub,
                  c->d_fxc, c->d_twk, c->d_twk32, c->d_twx, c->d_lp, c->d_s, c->d_A, c->d_Bp, c->d_vec, c->d_red,
                  c->d_coef};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return OCN_OK;
}

int ocn_val_last_error(const ocn_val_ctx* c, char* buf, size_t len) {
  if (!buf || len == 0) return OCN_ERR_ARG;
  std::snprintf(buf, len, "%s", (c ? c->err : g_val_create_err).c_str());
  return OCN_OK;
}

long long ocn_val_kernel_launches(const ocn_val_ctx* c) { return c ? c->launches : 0; }
void* ocn_val_stream(ocn_val_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int ocn_val_set_energies(ocn_val_ctx* c, const double* re, const double* im) {
  if (!c || !re) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  if (int rc = upload(c, c->d_er, re, sizeof(double) * c->npsi)) return rc;
  c->ei_nonzero = false;
  if (im) {
    for (size_t i = 0; i < c->npsi && !c->ei_nonzero; ++i) c->ei_nonzero = im[i] != 0.0;
    if (int rc = upload(c, c->d_ei, im, sizeof(double) * c->npsi)) return rc;
  }
  VCUDA(c, cudaStreamSynchronize(c->stream));
  c->have_e = true;
  return OCN_OK;
}

int ocn_val_set_allow(ocn_val_ctx* c, const double* allow) {
  if (!c || !allow) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  if (int rc = upload(c, c->d_allow, allow, sizeof(double) * c->npsi)) return rc;
  VCUDA(c, cudaStreamSynchronize(c->stream));
  c->have_allow = true;
  return OCN_OK;
}

int ocn_val_set_bubble(ocn_val_ctx* c, const double* bubble) {
  if (!c || !bubble) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  if (int rc = upload(c, c->d_bub, bubble, sizeof(double) * c->nx)) return rc;
  VCUDA(c, cudaStreamSynchronize(c->stream));
  c->have_bubble = true;
  return OCN_OK;
}

// OCEAN_fxc_prep's kernel (set by the caller, e.g. from ocn_val_fxc_from_rho);
// NULL switches the f_xc term off.  One valence-Hamiltonian spin only, as
// OCEAN_fxc_act (OCEAN_fxc.f90:154-159).
int ocn_val_set_fxc(ocn_val_ctx* c, const double* fxc) {
  if (!c) return vset_err(c, OCN_ERR_ARG, "null argument");
  if (!fxc) {
    c->have_fxc = false;
    return OCN_OK;
  }
  if (c->vspin != 1) return vset_err(c, OCN_ERR_UNSUPPORTED, "ocn_val_set_fxc: f_xc needs valence_ham_spin = 1");
  cudaSetDevice(c->device);
  if (int rc = upload(c, c->d_fxc, fxc, sizeof(double) * c->nx)) return rc;
  VCUDA(c, cudaStreamSynchronize(c->stream));
  c->have_fxc = true;
  return OCN_OK;
}

static int set_states_impl(ocn_val_ctx* c, const double* conr, const double* coni, const double* valr,
                           const double* vali, bool on_device) {
  if (!c || !conr || !coni || !valr || !vali) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  const size_t ncon = (size_t)c->nx * c->nc * c->nk * c->nspn, nval = (size_t)c->nx * c->nv * c->nk * c->nspn;
  const size_t nval1 = nval / c->nspn;
  double* tmp = nullptr;
  const double *cr = conr, *ci = coni, *vr = valr, *vi = vali;
  if (!on_device) {
    if (int rc = valloc(c, &tmp, 2 * std::max(ncon, nval))) return rc;
    cr = tmp;
    ci = tmp + ncon;
  }
  const int g = 4 * c->sm_count;
  int rc = OCN_OK;
  if (!on_device) {
    if ((rc = upload(c, tmp, conr, sizeof(double) * ncon)) || (rc = upload(c, tmp + ncon, coni, sizeof(double) * ncon)))
      goto done;
  }
  kv_interleave<<<g, 256, 0, c->stream>>>(cr, ci, ncon, c->d_con);
  if (!on_device) {
    vr = tmp;
    vi = tmp + nval;
    if ((rc = upload(c, tmp, valr, sizeof(double) * nval)) || (rc = upload(c, tmp + nval, vali, sizeof(double) * nval)))
      goto done;
  }
  kv_interleave<<<g, 256, 0, c->stream>>>(vr, vi, nval, c->d_val);
  if (c->mixed) {
    for (int sp = 0; sp < c->nspn; ++sp)
      kv_transpose_val<float><<<g, 256, 0, c->stream>>>(c->d_val + sp * nval1, c->nv, c->nk, c->nx,
                                                        static_cast<float2*>(c->d_valT) + sp * nval1);
    kv_to_float<<<g, 256, 0, c->stream>>>(reinterpret_cast<const double*>(c->d_con), 2 * ncon,
                                          reinterpret_cast<float*>(c->d_con32));
    kv_to_float<<<g, 256, 0, c->stream>>>(reinterpret_cast<const double*>(c->d_val), 2 * nval,
                                          reinterpret_cast<float*>(c->d_val32));
  }
  else
    for (int sp = 0; sp < c->nspn; ++sp)
      kv_transpose_val<double><<<g, 256, 0, c->stream>>>(c->d_val + sp * nval1, c->nv, c->nk, c->nx,
                                                         static_cast<double2*>(c->d_valT) + sp * nval1);
  {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = vcuda(c, e, "ocn_val_set_states");
  }
done:
  if (tmp) {
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
  }
  if (rc == OCN_OK) c->have_states = true;
  return rc;
}

int ocn_val_set_states(ocn_val_ctx* c, const double* conr, const double* coni, const double* valr,
                       const double* vali) {
  return set_states_impl(c, conr, coni, valr, vali, false);
}

int ocn_val_set_states_dev(ocn_val_ctx* c, const double* conr, const double* coni, const double* valr,
                           const double* vali) {
  return set_states_impl(c, conr, coni, valr, vali, true);
}

static int set_ladder_impl(ocn_val_ctx* c, const double* lad, bool on_device) {
  if (!c || !lad) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  const size_t n = (size_t)c->nk * c->nx * c->nx;
  if (!c->mixed) {
    VCUDA(c, cudaMemcpyAsync(c->d_lad, lad, sizeof(double) * n,
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  } else if (on_device) {
    kv_to_float<<<4 * c->sm_count, 256, 0, c->stream>>>(lad, n, static_cast<float*>(c->d_lad));
    VCUDA(c, cudaGetLastError());
  } else {  // staged through a bounded device buffer
    const size_t chunk = std::min<size_t>(n, (size_t)1 << 26);
    double* tmp = nullptr;
    if (int rc = valloc(c, &tmp, chunk)) return rc;
    int rc = OCN_OK;
    for (size_t o = 0; o < n && rc == OCN_OK; o += chunk) {
      const size_t m = std::min(chunk, n - o);
      rc = upload(c, tmp, lad + o, sizeof(double) * m);
      if (rc == OCN_OK) kv_to_float<<<4 * c->sm_count, 256, 0, c->stream>>>(tmp, m, static_cast<float*>(c->d_lad) + o);
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (rc) return rc;
    if (e != cudaSuccess) return vcuda(c, e, "ocn_val_set_ladder");
  }
  VCUDA(c, cudaStreamSynchronize(c->stream));
  c->have_ladder = true;
  return OCN_OK;
}

int ocn_val_set_ladder(ocn_val_ctx* c, const double* ladder) { return set_ladder_impl(c, ladder, false); }
int ocn_val_set_ladder_dev(ocn_val_ctx* c, const double* d_ladder) { return set_ladder_impl(c, d_ladder, true); }

int ocn_val_apply_H_dev(ocn_val_ctx* c, const double* d_in, double* d_out, const int flags[3], int backwards) {
  if (!c || !d_in || !d_out || !flags) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  return apply_dev(c, d_in, d_out, flags, backwards);
}

int ocn_val_apply_H(ocn_val_ctx* c, const double* in_r, const double* in_i, double* out_r, double* out_i,
                    const int flags[3], int backwards) {
  if (!c || !in_r || !in_i || !out_r || !out_i || !flags) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* din = c->d_vec;
  double* dout = c->d_vec + 2 * n;
  if (int rc = upload(c, din, in_r, sizeof(double) * n)) return rc;
  if (int rc = upload(c, din + n, in_i, sizeof(double) * n)) return rc;
  if (int rc = apply_dev(c, din, dout, flags, backwards)) return rc;
  VCUDA(c, cudaMemcpyAsync(out_r, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  VCUDA(c, cudaMemcpyAsync(out_i, dout + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  VCUDA(c, cudaStreamSynchronize(c->stream));
  return OCN_OK;
}

// OCEAN_haydock_Herm_do over the valence action (OCEAN_haydock.f90:190-320,
// 824-938); psi0 is a device vector (real plane, then imaginary plane).
int ocn_val_haydock_dev(ocn_val_ctx* c, const double* d_psi0, int niter, const int flags[3], double* real_a,
                        double* imag_a, double* real_b, int* niter_done) {
  if (!c || !d_psi0 || !flags || !real_a || !imag_a || !real_b || !niter_done || niter < 1)
    return vset_err(c, OCN_ERR_ARG, "bad argument");
  cudaSetDevice(c->device);
  if (int rc = check_ready(c, flags)) return rc;
  const size_t n = c->npsi;
  if (c->coef_cap < niter + 1) {
    if (c->d_coef) cudaFree(c->d_coef);
    c->d_coef = nullptr;
    c->coef_cap = 0;
    if (int rc = valloc(c, &c->d_coef, 3 * (size_t)(niter + 1))) return rc;
    c->coef_cap = niter + 1;
  }
  double* ra = c->d_coef;
  double* ia = ra + (niter + 1);
  double* rb = ia + (niter + 1);
  VCUDA(c, cudaMemsetAsync(c->d_coef, 0, sizeof(double) * 3 * (niter + 1), c->stream));
  double* psi = c->d_vec;
  double* h = c->d_vec + 2 * n;
  double* old = c->d_vec + 4 * n;
  VCUDA(c, cudaMemcpyAsync(psi, d_psi0, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice, c->stream));
  VCUDA(c, cudaMemsetAsync(old, 0, sizeof(double) * 2 * n, c->stream));
  const int nb = c->red_blocks;
  for (int it = 1; it <= niter; ++it) {
    if (int rc = apply_dev(c, psi, h, flags, 0)) return rc;
    kv_lz1<<<nb, VAL_THREADS, 0, c->stream>>>(h, old, psi, n, rb, it, c->d_red);
    kv_lz2<<<nb, VAL_THREADS, 0, c->stream>>>(c->d_red, nb, h, psi, n, ra, ia, it, c->d_red + 2 * nb);
    kv_lz3<<<nb, VAL_THREADS, 0, c->stream>>>(c->d_red + 2 * nb, nb, h, n, rb, it);
    c->launches += 3;
    VCUDA(c, cudaGetLastError());
    double* t = old;  // old <- psi, psi <- h (now h / b), h <- the old buffer
    old = psi;
    psi = h;
    h = t;
  }
  VCUDA(c, cudaMemcpyAsync(real_a, ra, sizeof(double) * (niter + 1), cudaMemcpyDeviceToHost, c->stream));
  VCUDA(c, cudaMemcpyAsync(imag_a, ia, sizeof(double) * (niter + 1), cudaMemcpyDeviceToHost, c->stream));
  VCUDA(c, cudaMemcpyAsync(real_b, rb, sizeof(double) * (niter + 1), cudaMemcpyDeviceToHost, c->stream));
  VCUDA(c, cudaStreamSynchronize(c->stream));
  int done = niter;
  for (int i = 0; i < niter; ++i)
    if (std::isnan(real_a[i])) {
      done = i + 1;
      break;
    }
  *niter_done = done;
  return done < niter || std::isnan(real_a[niter - 1]) ? OCN_ERR_NAN : OCN_OK;
}

int ocn_val_gmres(ocn_val_ctx* c, const double* hay_r, const double* hay_i, double kpref, double celvol,
                  const double* energies_ev, int nomega, const ocn_gmres_params* p, const int flags[3],
                  double* out_re, double* out_im, double* rel_err, int* iters) {
  if (!c || !hay_r || !hay_i || !energies_ev || nomega < 1 || !p || p->depth < 1 || p->depth > 1024)
    return vset_err(c, OCN_ERR_ARG, "ocn_val_gmres: bad argument");
  cudaSetDevice(c->device);
  int fl[3] = {1, 1, 1};
  if (flags)
    for (int i = 0; i < 3; ++i) fl[i] = flags[i];
  if (int rc = check_ready(c, fl)) return rc;
  const size_t n = c->npsi;
  double* d_hay = nullptr;
  if (int rc = valloc(c, &d_hay, 2 * n)) return rc;
  int rc = upload(c, d_hay, hay_r, sizeof(double) * n);
  if (rc == OCN_OK) rc = upload(c, d_hay + n, hay_i, sizeof(double) * n);
  if (rc == OCN_OK) {
    ocn::GmresOp op;
    op.n = n;
    op.dfmt = c->mixed != 0;
    op.sm_count = c->sm_count;
    op.stream = c->stream;
    op.launches = &c->launches;
    op.nvec = 1;
    op.allow = c->d_allow;
    op.mask_ones = true;  // OCEAN_energies_allow_full on the ones (OCEAN_gmres.f90:603-606)
    op.H = [c, &fl](const double* in, double* out) { return apply_dev(c, in, out, fl, 0); };
    op.err = [c](int code, const std::string& msg) { return vset_err(c, code, msg); };
    // fact = kpref 2 celvol for a valence run (OCEAN_gmres.f90:544-548)
    rc = ocn::gmres_solve_op(op, d_hay, kpref * 2.0 * celvol, energies_ev, nomega, p, 1, out_re, out_im, rel_err,
                             iters, nullptr, false);
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(d_hay);
  return rc;
}

int ocn_val_haydock(ocn_val_ctx* c, const double* psi0_r, const double* psi0_i, int niter, const int flags[3],
                    double* real_a, double* imag_a, double* real_b, int* niter_done) {
  if (!c || !psi0_r || !psi0_i) return vset_err(c, OCN_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* d0 = c->d_vec + 6 * n;
  if (int rc = upload(c, d0, psi0_r, sizeof(double) * n)) return rc;
  if (int rc = upload(c, d0 + n, psi0_i, sizeof(double) * n)) return rc;
  return ocn_val_haydock_dev(c, d0, niter, flags, real_a, imag_a, real_b, niter_done);
}

// Local-density exchange and correlation energies per electron of an
// unpolarised, non-relativistic gas, as cacorr forms them (OCEAN_fxc.f90:333-470):
// Slater exchange and the Ceperley-Alder correlation in the Perdew-Zunger
// (Phys. Rev. B 23, 5048) parametrisation, zeta = 0.
static void lda_energies(double n, double* ex, double* ec) {
  if (n < 0.00000001) {
    *ex = 0.0;
    *ec = 0.0;
    return;
  }
  const double pi = 3.1415926535897932384626433832795;
  const double third = 1.0 / 3.0;
  const double rs = std::pow(3.0 / (4.0 * pi * n), third);
  const double spin_n = n / 2.0;                                   // each spin channel
  const double e1 = -1.5 * std::pow(0.75 / pi, third) * std::pow(spin_n, third);
  *ex = (spin_n * e1 + spin_n * e1) / n;
  if (rs >= 1.0) {
    *ec = -0.1423 / (1.0 + 1.0529 * std::sqrt(rs) + 0.3334 * rs);
  } else {
    const double lrs = std::log(rs);
    *ec = 0.0311 * lrs + (-0.048) + 0.002 * (rs * lrs) + (-0.0116) * rs;
  }
}

// OCEAN_fxc_prep (OCEAN_fxc.f90:35-123): f_xc(x) = second derivative of
// n (ex + ec) at n = rho(x) by the five-point rule with step n/100, times
// Nx / (Nk V).  rho in the x-mesh order (x3 fastest).  Host only.
int ocn_val_fxc_from_rho(int nx, const double* rho, double celvol, int nkpts, double* fxc) {
  if (nx < 1 || !rho || !fxc || nkpts < 1 || !(celvol > 0.0))
    return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_fxc_from_rho: bad argument");
  for (int i = 0; i < nx; ++i) {
    const double n = rho[i], dn = 0.01 * n;
    const double pts[5] = {n + 2 * dn, n + dn, n, n - dn, n - 2 * dn};
    double f[5];
    for (int j = 0; j < 5; ++j) {
      double ex, ec;
      lda_energies(pts[j], &ex, &ec);
      f[j] = pts[j] * (ex + ec);
    }
    fxc[i] = (16.0 * (f[3] + f[1]) - (f[4] + f[0]) - 30.0 * f[2]) / (12.0 * dn * dn) * (double)nx /
             ((double)nkpts * celvol);
  }
  return OCN_OK;
}

// AI_bubble_populate with wall_search_old_way (OCEAN_bubble.f90:238-407).
int ocn_val_bubble_populate(const int xmesh[3], const double bvec[9], const double qinb[3], double celvol,
                            int nkpts, double* bubble, int* ngvec) {
  if (!xmesh || !bvec || !qinb || !bubble || nkpts < 1 || !(celvol > 0.0))
    return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_bubble_populate: bad argument");
  const int n1 = xmesh[0], n2 = xmesh[1], n3 = xmesh[2];
  if (n1 < 1 || n2 < 1 || n3 < 1) return vset_err(nullptr, OCN_ERR_ARG, "ocn_val_bubble_populate: bad mesh");
  auto glen = [&](int a, int b, int cc) {  // squared length of B g (gvec_length, :38-47)
    double s = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double t = bvec[i] * a + bvec[i + 3] * b + bvec[i + 6] * cc;
      s += t * t;
    }
    return s;
  };
  auto lo = [](int n) { return (int)std::floor(-(double)n / 2.0); };
  auto hi = [](int n) { return (int)std::ceil((double)n / 2.0); };
  double length = HUGE_VAL;
  for (int a = lo(n1); a <= hi(n1); ++a)
    for (int b = lo(n2); b <= hi(n2); ++b)
      for (int cc = lo(n3); cc <= hi(n3); ++cc)
        if (2 * std::abs(cc) >= n3 || 2 * std::abs(b) >= n2 || 2 * std::abs(a) >= n1)
          length = std::min(length, glen(a, b, cc));
  double next = 0.0;
  for (int a = lo(n1); a <= hi(n1); ++a)
    for (int b = lo(n2); b <= hi(n2); ++b)
      for (int cc = lo(n3); cc <= hi(n3); ++cc) {
        const double t = glen(a, b, cc);
        if (t < length && t > next) next = t;
      }
  length = 0.5 * (length + next);
  double bmet[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int q = 0; q < 3; ++q) s += bvec[q + 3 * i] * bvec[q + 3 * j];
      bmet[i][j] = s;
    }
  const double pi = 3.1415926535897932384626433832795;
  const double g2min = 8.0 * pi * pi * pi / (celvol * (double)(n1 * n2 * n3));
  std::fill(bubble, bubble + (size_t)n1 * n2 * n3, 0.0);
  int count = 0;
  for (int a = (int)std::ceil(-(double)n1 / 2.0); a <= (int)std::floor((double)n1 / 2.0); ++a)
    for (int b = (int)std::ceil(-(double)n2 / 2.0); b <= (int)std::floor((double)n2 / 2.0); ++b)
      for (int cc = (int)std::ceil(-(double)n3 / 2.0); cc <= (int)std::floor((double)n3 / 2.0); ++cc) {
        const double qq[3] = {qinb[0] + a, qinb[1] + b, qinb[2] + cc};
        double g2 = 0.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) g2 += qq[i] * qq[j] * bmet[i][j];
        if (g2 < g2min) g2 = g2min;
        const int ix = a < 0 ? a + n1 : a, iy = b < 0 ? b + n2 : b, iz = cc < 0 ? cc + n3 : cc;
        double mul = 0.0;
        if (glen(a, b, cc) < length) {
          mul = 4.0 * pi / (celvol * g2 * (double)nkpts);
          ++count;
        }
        bubble[iz + (size_t)n3 * (iy + (size_t)n2 * ix)] = mul;
      }
  bubble[0] = 0.0;
  if (ngvec) *ngvec = count - 1;
  return OCN_OK;
}

}  // extern "C"
