// ocn_kernels.cu -- FP64 kernels of the BSE action and the vector steps of the
// Haydock and GMRES solvers.
//
// Device layouts
//   psi-like vectors  two planes re[npsi], im[npsi], npsi = Nb*Nk*Na, element
//                     (n,k,a) at n + Nb*(k + Nk*a)  (OCEAN_psi.f90:63-76)
//   u                 double2 [s][x][k][n]            (long_range.f90:168-179)
//   W                 double  [x][k]                  (long_range.f90:1846)
//   phi (FP64 path)   double2 [k][x][a]
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdio>
#include <new>

#include "ocn_df.cuh"
#include "ocn_internal.h"
#include "ocn_kmesh_dft.cuh"

namespace ocn {

namespace {


// ------------------------------------------------------------ phase of u2

// u(n,k,x,s) *= exp(i phi(x,k)) exactly as OCEAN_bloch_lrLOAD writes it
// (OCEAN_bloch.f90:191-197); explicit _rn intrinsics keep the products unfused.
__global__ void k_phase_bloch(const double* __restrict__ ur, const double* __restrict__ ui,
                              const double* __restrict__ pc, const double* __restrict__ ps,
                              double2* __restrict__ u, long long total, int nb, int nk, int nx) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long q = i / nb;         // k + nk*(x + nx*s)
    long long xk = q % ((long long)nk * nx);
    double c = pc[xk], s = ps[xk];
    double r = ur[i], m = ui[i];
    u[i] = make_double2(__dsub_rn(__dmul_rn(c, r), __dmul_rn(s, m)),
                        __dadd_rn(__dmul_rn(c, m), __dmul_rn(s, r)));
  }
}

// ---------------------------------------------------- LR: band -> x-mesh

// phi[k][x][a] = sum_n u(n,k,x) * (allow o psi)(n,k,a)   (long_range.f90:897-906)
// grid (ceil(Nx/128), Nk), 128 threads: thread = x.  u staged through shared
// memory transposed so each thread reads its own column conflict-free.
constexpr int G1_X = 128;
constexpr int G1_N = 32;
__global__ void __launch_bounds__(G1_X) k_lr_gemm1_fp64(
    const double2* __restrict__ u, const double* __restrict__ pr, const double* __restrict__ pi,
    const double* __restrict__ allow, double2* __restrict__ phi, int nb, int nk, int nx, int na,
    int nspn) {
  extern __shared__ double2 smem[];
  double2* us = smem;                          // [nspn][G1_N][G1_X+1]
  double2* ps = smem + nspn * G1_N * (G1_X + 1);  // [na][G1_N]
  const int k = blockIdx.y;
  const int x0 = blockIdx.x * G1_X;
  const int tx = threadIdx.x;
  const int x = x0 + tx;
  double2 acc[OCN_MAX_NA];
#pragma unroll
  for (int a = 0; a < OCN_MAX_NA; ++a) acc[a] = make_double2(0.0, 0.0);

  for (int n0 = 0; n0 < nb; n0 += G1_N) {
    const int nn = min(G1_N, nb - n0);
    __syncthreads();
    // stage u[s][x0..x0+127][k][n0..n0+nn): each warp walks x rows, lanes along n
    for (int s = 0; s < nspn; ++s)
      for (int e = tx; e < G1_X * G1_N; e += G1_X) {
        const int xl = e / G1_N, nl = e % G1_N;
        double2 v = make_double2(0.0, 0.0);
        if (x0 + xl < nx && nl < nn)
          v = u[(((size_t)s * nx + (x0 + xl)) * nk + k) * nb + n0 + nl];
        us[(s * G1_N + nl) * (G1_X + 1) + xl] = v;
      }
    for (int e = tx; e < na * G1_N; e += G1_X) {
      const int a = e / G1_N, nl = e % G1_N;
      double2 v = make_double2(0.0, 0.0);
      if (nl < nn) {
        const size_t idx = (size_t)n0 + nl + (size_t)nb * ((size_t)k + (size_t)nk * a);
        const double m = allow[idx];
        v = make_double2(pr[idx] * m, pi[idx] * m);
      }
      ps[a * G1_N + nl] = v;
    }
    __syncthreads();
    for (int nl = 0; nl < nn; ++nl) {
      const double2 u0 = us[nl * (G1_X + 1) + tx];
      const double2 u1 = (nspn == 2) ? us[(G1_N + nl) * (G1_X + 1) + tx] : u0;
#pragma unroll
      for (int a = 0; a < OCN_MAX_NA; ++a) {
        if (a < na) {
          const double2 uu = (a & 1) ? u1 : u0;
          const double2 q = ps[a * G1_N + nl];
          acc[a].x += uu.x * q.x - uu.y * q.y;
          acc[a].y += uu.x * q.y + uu.y * q.x;
        }
      }
    }
  }
  if (x < nx) {
    double2* o = phi + ((size_t)k * nx + x) * na;
#pragma unroll
    for (int a = 0; a < OCN_MAX_NA; ++a)
      if (a < na) o[a] = acc[a];
  }
}

// ------------------------------------------------ LR: k <-> R and x W(R,x)

// phi'(.,x,a) = FFT_fwd[ W(.,x) o FFT_bwd[ phi(.,x,a) ] ] / Nk   (long_range.f90:928-939,
// FFTW signs +1 backward / -1 forward, Modules/FFT_wrapper.f90:24-25).  One CTA per x,
// transform in shared memory (ocn_kmesh_dft.cuh).
__global__ void k_lr_fft_w_fp64(double2* __restrict__ phi, const double* __restrict__ W, int nx,
                                const KmeshGeom<double> g, const double2* __restrict__ twg) {
  extern __shared__ double2 smem[];
  double2* tw = smem;
  double2* buf = smem + 3 * OCN_MAX_KDIM;
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  kmesh_convolve<double>(phi, W, nx, blockIdx.x, g, buf, tw);
}

template <int N, int NTC>
__global__ void k_fft_cube_fp64(double2* __restrict__ phi, const double* __restrict__ W, int nx, int nt,
                                const double2* __restrict__ twg) {
  extern __shared__ double2 smem[];
  double2* tw = smem;
  double2* buf = smem + 3 * OCN_MAX_KDIM;
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  kmesh_convolve_cube<double, N, NTC>(phi, W, nx, blockIdx.x, nt, nt, buf, tw);
}
typedef void (*CubeFnD)(double2*, const double*, int, int, const double2*);

template <int N>
__global__ void k_wgrad_cube_fp64(const double2* __restrict__ phx, const double2* __restrict__ phy, int nx,
                                  int nt, double* __restrict__ gW, double ca, double cb,
                                  const double2* __restrict__ twg) {
  extern __shared__ double2 smem[];
  double2* tw = smem;
  double2* buf = smem + 3 * OCN_MAX_KDIM;
  for (int i = threadIdx.x; i < 3 * OCN_MAX_KDIM; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  kmesh_wgrad_cube<double, N>(phx, phy, nx, blockIdx.x, nt, buf, tw, gW, ca, cb);
}
typedef void (*WgradFnD)(const double2*, const double2*, int, int, double*, double, double, const double2*);

WgradFnD wgrad_fn(int n) {
  switch (n) {
    case 2: return k_wgrad_cube_fp64<2>;
    case 3: return k_wgrad_cube_fp64<3>;
    case 4: return k_wgrad_cube_fp64<4>;
    case 5: return k_wgrad_cube_fp64<5>;
    case 6: return k_wgrad_cube_fp64<6>;
    case 8: return k_wgrad_cube_fp64<8>;
  }
  return nullptr;
}

// ------------------------------------------------------ LR: x-mesh -> band

// part[split][re|im][a][k][n] = - sum_{x in split} conj(u(n,k,x)) phi'(k,x,a)
// (long_range.f90:943-961).  grid (Nk, nsplit), one thread per band.
constexpr int G2_XC = 32;
__global__ void k_lr_gemm2_fp64(const double2* __restrict__ u, const double2* __restrict__ phi,
                                double* __restrict__ part, int nb, int nk, int nx, int na, int nspn,
                                int xper, size_t npsi) {
  __shared__ double2 fs[G2_XC * OCN_MAX_NA];
  const int k = blockIdx.x;
  const int split = blockIdx.y;
  const int xa = split * xper, xb = min(nx, xa + xper);
  const int n = threadIdx.x;
  double2 acc[OCN_MAX_NA];
#pragma unroll
  for (int a = 0; a < OCN_MAX_NA; ++a) acc[a] = make_double2(0.0, 0.0);
  for (int x0 = xa; x0 < xb; x0 += G2_XC) {
    const int xn = min(G2_XC, xb - x0);
    __syncthreads();
    for (int e = threadIdx.x; e < xn * na; e += blockDim.x)
      fs[e] = phi[((size_t)k * nx + x0) * na + e];
    __syncthreads();
    if (n < nb) {
      for (int xl = 0; xl < xn; ++xl) {
        const double2 u0 = u[(((size_t)0 * nx + x0 + xl) * nk + k) * nb + n];
        const double2 u1 = (nspn == 2) ? u[(((size_t)1 * nx + x0 + xl) * nk + k) * nb + n] : u0;
#pragma unroll
        for (int a = 0; a < OCN_MAX_NA; ++a) {
          if (a < na) {
            const double2 uu = (a & 1) ? u1 : u0;
            const double2 f = fs[xl * na + a];
            acc[a].x += uu.x * f.x + uu.y * f.y;
            acc[a].y += uu.x * f.y - uu.y * f.x;
          }
        }
      }
    }
  }
  if (n < nb) {
    double* pr = part + (size_t)split * 2 * npsi;
    double* pim = pr + npsi;
#pragma unroll
    for (int a = 0; a < OCN_MAX_NA; ++a)
      if (a < na) {
        const size_t idx = (size_t)n + (size_t)nb * ((size_t)k + (size_t)nk * a);
        pr[idx] = -acc[a].x;
        pim[idx] = -acc[a].y;
      }
  }
}

// ----------------------------------------------------------- combination

// out(n,k,ic) = E o psi (conj when backwards) + allow o (acc + sum of LR parts)
//             + sum_jc S(ic,jc) psi(n,k,jc)        (OCEAN_action.f90:337-372,596-608)
// Optionally fused with the first Lanczos stage (ocean_hay_ab_twoterm,
// OCEAN_haydock.f90:848-860): out -= b_{i-1} old, partial <out|psi>.
// PT: element type of the long-range / multiplet partials (double on the FP64
// path, float from the tensor-core contractions).
template <int NA, bool SO, typename PT>
__device__ __forceinline__ void combine_body(const double* __restrict__ pr, const double* __restrict__ pi,
                          const double* __restrict__ er, const double* __restrict__ ei,
                          const double* __restrict__ allow, const double* __restrict__ acc,
                          const PT* __restrict__ part, int nparts, const double2* __restrict__ so,
                          double* __restrict__ outr, double* __restrict__ outi, int nbk, int na,
                          size_t npsi, int use_e0, int use_so, int backwards,
                          const double* __restrict__ oldr, const double* __restrict__ oldi,
                          const double* __restrict__ rb_base, const int* __restrict__ itp,
                          double* __restrict__ red, const BlockStrides bs, int bx, int by, int nbx) {
  __shared__ double sh[2][32];
  // chain / vector v = by of a block of psi vectors
  const size_t v = by;
  pr += v * bs.vec;
  pi += v * bs.vec;
  outr += v * bs.vec;
  outi += v * bs.vec;
  if (acc) acc += v * bs.vec;
  part += v * 2 * npsi;
  if (oldr) {
    oldr += v * bs.vec;
    oldi += v * bs.vec;
    rb_base += v * bs.coef;
  }
  if (red) red += v * bs.red;
  double dr = 0.0, di = 0.0;
  double bm = 0.0;
  if (oldr) bm = -rb_base[*itp - 1];  // b_{i-1}
  // one thread per psi element idx = e + Nb*Nk*ic: the spin-orbit sum reads the
  // other channels of the same (n, k), which neighbouring threads also load
  const size_t nall = (size_t)nbk * NA;
  for (size_t idx = bx * (size_t)blockDim.x + threadIdx.x; idx < nall;
       idx += (size_t)nbx * blockDim.x) {
    const int ic = (int)(idx / (size_t)nbk);
    const size_t e = idx - (size_t)ic * nbk;
    const double qrc = pr[idx], qic = pi[idx];
    double fr = 0.0, fi = 0.0;
    if (acc) {
      fr = acc[idx];
      fi = acc[npsi + idx];
    }
    for (int s = 0; s < nparts; ++s) {
      fr += (double)part[(size_t)s * bs.part + idx];
      fi += (double)part[(size_t)s * bs.part + npsi + idx];
    }
    const double m = allow[idx];
    fr *= m;
    fi *= m;
    if (SO) {  // spin-orbit (use_so selects the instantiation)
#pragma unroll
      for (int jc = 0; jc < NA; ++jc) {
        const double2 sv = so[jc * NA + ic];
        const size_t j = e + (size_t)nbk * jc;
        const double qr = pr[j], qi = pi[j];
        if (backwards) {
          fr = fr + sv.x * qr + sv.y * qi;
          fi = fi + sv.x * qi - sv.y * qr;
        } else {
          fr = fr + sv.x * qr - sv.y * qi;
          fi = fi + sv.x * qi + sv.y * qr;
        }
      }
    }
    double hr = 0.0, hi = 0.0;
    if (use_e0) {
      const double a_ = er[idx], b_ = ei ? ei[idx] : 0.0;
      if (backwards) {
        hr = a_ * qrc + b_ * qic;
        hi = a_ * qic - b_ * qrc;
      } else {
        hr = a_ * qrc - b_ * qic;
        hi = a_ * qic + b_ * qrc;
      }
    }
    hr += fr;
    hi += fi;
    if (oldr) {
      hr += bm * oldr[idx];
      hi += bm * oldi[idx];
      // psi_dot(hpsi, psi): sum conj(h) psi  (OCEAN_psi.f90:2029-2034)
      dr += hr * qrc + hi * qic;
      di += hr * qic - hi * qrc;
    }
    outr[idx] = hr;
    outi[idx] = hi;
  }
  if (!red) return;
  // deterministic block reduction
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_down_sync(0xffffffffu, dr, o);
    di += __shfl_down_sync(0xffffffffu, di, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = dr;
    sh[1][w] = di;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      s0 += sh[0][i];
      s1 += sh[1][i];
    }
    red[2 * bx] = s0;
    red[2 * bx + 1] = s1;
  }
}


template <int NA, bool SO, typename PT>
__global__ void __launch_bounds__(LZ_THREADS)
    k_combine(const double* __restrict__ pr, const double* __restrict__ pi, const double* __restrict__ er,
              const double* __restrict__ ei, const double* __restrict__ allow, const double* __restrict__ acc,
              const void* __restrict__ part, int nparts, const double2* __restrict__ so,
              double* __restrict__ outr, double* __restrict__ outi, int nbk, int na, size_t npsi, int use_e0,
              int use_so, int backwards, const double* __restrict__ oldr, const double* __restrict__ oldi,
              const double* __restrict__ rb_base, const int* __restrict__ itp, double* __restrict__ red,
              const BlockStrides bs) {
  combine_body<NA, SO, PT>(pr, pi, er, ei, allow, acc, static_cast<const PT*>(part), nparts, so, outr, outi, nbk, na,
                           npsi, use_e0, use_so, backwards, oldr, oldi, rb_base, itp, red, bs, blockIdx.x,
                           blockIdx.y, gridDim.x);
}

// ------------------------------------------- double-float Lanczos step (mixed precision)
// The mixed-precision Haydock loop keeps its vectors as double-float planes
// (ocn_df.cuh): a float2 (h, l) per real value, at the offsets of the FP64
// layout.  The operator data are double-float / binary32 copies (energies,
// masks, spin-orbit matrix) and the long-range / multiplet partials are the
// binary32 outputs of the tensor-core contractions; every per-element operation
// runs on the FP32 pipe.  Reduction partials are double-float pairs in the
// (double-sized) partial arrays; a, b are recorded in FP64.

// Deterministic block reduction of K double-float sums; thread 0 writes them to
// out[0..K-1].  sh: 32 float2 per sum.
template <int K>
__device__ __forceinline__ void block_reduce_df(df (&v)[K], float2 (*sh)[32], float2* __restrict__ out) {
#pragma unroll
  for (int j = 0; j < K; ++j)
    for (int o = 16; o > 0; o >>= 1) {
      const float bh = __shfl_down_sync(0xffffffffu, v[j].h, o);
      const float bl = __shfl_down_sync(0xffffffffu, v[j].l, o);
      v[j] = df_add(v[j], df{bh, bl});
    }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int j = 0; j < K; ++j) sh[j][w] = make_float2(v[j].h, v[j].l);
  __syncthreads();
  if (w == 0) {  // the warp partials, summed by a fixed shuffle tree
    const int nw = (int)(blockDim.x >> 5);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      df t = l < nw ? df{sh[j][l].x, sh[j][l].y} : df{0.0f, 0.0f};
      for (int o = 16; o > 0; o >>= 1)
        t = df_add(t, df{__shfl_down_sync(0xffffffffu, t.h, o), __shfl_down_sync(0xffffffffu, t.l, o)});
      if (l == 0) out[j] = make_float2(t.h, t.l);
    }
  }
}

// Sum of nblk double-float partial pairs, in the same order in every thread of
// every block.
__device__ __forceinline__ void reduce_pairs_df(const float2* __restrict__ red, int nblk, df* s0, df* s1) {
  __shared__ float2 sh[2][32];
  df a{0.0f, 0.0f}, b{0.0f, 0.0f};
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a = df_add(a, df{red[2 * i].x, red[2 * i].y});
    b = df_add(b, df{red[2 * i + 1].x, red[2 * i + 1].y});
  }
  for (int o = 16; o > 0; o >>= 1) {
    a = df_add(a, df{__shfl_down_sync(0xffffffffu, a.h, o), __shfl_down_sync(0xffffffffu, a.l, o)});
    b = df_add(b, df{__shfl_down_sync(0xffffffffu, b.h, o), __shfl_down_sync(0xffffffffu, b.l, o)});
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sh[0][w] = make_float2(a.h, a.l);
    sh[1][w] = make_float2(b.h, b.l);
  }
  __syncthreads();
  df ta{0.0f, 0.0f}, tb{0.0f, 0.0f};
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
    ta = df_add(ta, df{sh[0][i].x, sh[0][i].y});
    tb = df_add(tb, df{sh[1][i].x, sh[1][i].y});
  }
  *s0 = ta;
  *s1 = tb;
}

// combine + first Lanczos stage (as combine_body with the Lanczos fields set,
// OCEAN_action.f90:337-372 then OCEAN_haydock.f90:848-860): h = E o psi + allow o
// (partials) + S psi - b_{i-1} old, and the block partials of <h|psi> (red[2 bx],
// red[2 bx + 1]) and of |h|^2, |psi|^2 (red[2 nbx + 2 bx], red[2 nbx + 2 bx + 1]),
// from which the normalisation forms b_i without another pass over h.
template <int NA, bool SO>
__device__ __forceinline__ void combine_df_body(const float2* __restrict__ pr, const float2* __restrict__ pi,
                                                const float2* __restrict__ er, const float2* __restrict__ ei,
                                                const float* __restrict__ allow, const float* __restrict__ part,
                                                int nparts, const float2* __restrict__ so, float2* __restrict__ outr,
                                                float2* __restrict__ outi, int nbk, size_t npsi, int use_e0,
                                                const float2* __restrict__ oldr, const float2* __restrict__ oldi,
                                                const double* __restrict__ rb_base, const int* __restrict__ itp,
                                                float2* __restrict__ red, const BlockStrides bs, int bx, int by,
                                                int nbx) {
  __shared__ float2 sh[4][32];
  const size_t v = by;
  pr += v * bs.vec;
  pi += v * bs.vec;
  outr += v * bs.vec;
  outi += v * bs.vec;
  oldr += v * bs.vec;
  oldi += v * bs.vec;
  part += v * 2 * npsi;
  rb_base += v * bs.coef;
  red += v * bs.red;
  // -b_{i-1}, formed by each warp's lane 0 (no block barrier before the element loop)
  df bm{0.0f, 0.0f};
  if ((threadIdx.x & 31) == 0) bm = df_split(-rb_base[*itp - 1]);
  bm.h = __shfl_sync(0xffffffffu, bm.h, 0);
  bm.l = __shfl_sync(0xffffffffu, bm.l, 0);
  df dr{0.0f, 0.0f}, di{0.0f, 0.0f}, hh{0.0f, 0.0f}, pp{0.0f, 0.0f};
  const size_t nall = (size_t)nbk * NA;
  for (size_t idx = bx * (size_t)blockDim.x + threadIdx.x; idx < nall; idx += (size_t)nbx * blockDim.x) {
    const int ic = (int)(idx / (size_t)nbk);
    const size_t e = idx - (size_t)ic * nbk;
    const df qr = df_ld(pr, idx), qi = df_ld(pi, idx);
    df fr{0.0f, 0.0f}, fi{0.0f, 0.0f};
    for (int s = 0; s < nparts; ++s) {
      fr = df_add(fr, part[(size_t)s * bs.part + idx]);
      fi = df_add(fi, part[(size_t)s * bs.part + npsi + idx]);
    }
    const float m = allow[idx];
    fr = df_mul(fr, m);
    fi = df_mul(fi, m);
    if (SO) {
#pragma unroll
      for (int jc = 0; jc < NA; ++jc) {
        const float2 sv = so[jc * NA + ic];
        const size_t j = e + (size_t)nbk * jc;
        const df qr2 = df_ld(pr, j), qi2 = df_ld(pi, j);
        fr = df_add(fr, df_mul(qr2, sv.x));
        fr = df_add(fr, df_mul(qi2, -sv.y));
        fi = df_add(fi, df_mul(qi2, sv.x));
        fi = df_add(fi, df_mul(qr2, sv.y));
      }
    }
    df hr = fr, hi = fi;
    if (use_e0) {
      const df a = df_ld(er, idx);
      hr = df_add(hr, df_mul(a, qr));
      hi = df_add(hi, df_mul(a, qi));
      if (ei) {
        const df b = df_ld(ei, idx);
        hr = df_add(hr, df_neg(df_mul(b, qi)));
        hi = df_add(hi, df_mul(b, qr));
      }
    }
    hr = df_add(hr, df_mul(bm, df_ld(oldr, idx)));
    hi = df_add(hi, df_mul(bm, df_ld(oldi, idx)));
    // psi_dot(hpsi, psi): sum conj(h) psi
    df_fma(dr.h, dr.l, hr, qr);
    df_fma(dr.h, dr.l, hi, qi);
    df_fma(di.h, di.l, hr, qi);
    df_fma(di.h, di.l, df_neg(hi), qr);
    df_fma(hh.h, hh.l, hr, hr);
    df_fma(hh.h, hh.l, hi, hi);
    df_fma(pp.h, pp.l, qr, qr);
    df_fma(pp.h, pp.l, qi, qi);
    df_st(outr, idx, hr);
    df_st(outi, idx, hi);
  }
  df q[4] = {dr, di, hh, pp};
  float2 tot[4];
  block_reduce_df<4>(q, sh, tot);
  if (threadIdx.x == 0) {
    red[2 * bx] = tot[0];
    red[2 * bx + 1] = tot[1];
    red[2 * nbx + 2 * bx] = tot[2];
    red[2 * nbx + 2 * bx + 1] = tot[3];
  }
}

template <int NA, bool SO>
__global__ void __launch_bounds__(LZ_DF_THREADS)
    k_combine_df(const float2* __restrict__ pr, const float2* __restrict__ pi, const float2* __restrict__ er,
                 const float2* __restrict__ ei, const float* __restrict__ allow, const float* __restrict__ part,
                 int nparts, const float2* __restrict__ so, float2* __restrict__ outr, float2* __restrict__ outi,
                 int nbk, size_t npsi, int use_e0, const float2* __restrict__ oldr, const float2* __restrict__ oldi,
                 const double* __restrict__ rb_base, const int* __restrict__ itp, float2* __restrict__ red,
                 const BlockStrides bs) {
  combine_df_body<NA, SO>(pr, pi, er, ei, allow, part, nparts, so, outr, outi, nbk, npsi, use_e0, oldr, oldi, rb_base,
                          itp, red, bs, blockIdx.x, blockIdx.y, gridDim.x);
}

// The combine + first Lanczos stage of several contexts of one (Na, spin-orbit)
// class in one launch: grid (blocks per context, largest block of vectors,
// contexts); every context keeps the block partition (and so the reduction
// order) of its own launches.
template <int NA, bool SO>
__global__ void __launch_bounds__(LZ_DF_THREADS) k_combine_df_group(const CombineArgs* __restrict__ tab) {
  const CombineArgs& a = tab[blockIdx.z];
  if ((int)blockIdx.y >= a.nv || (int)blockIdx.x >= a.nblk) return;
  combine_df_body<NA, SO>(reinterpret_cast<const float2*>(a.pr), reinterpret_cast<const float2*>(a.pi), a.er_df,
                          a.ei_df, a.allow_f, reinterpret_cast<const float*>(a.part), a.nparts, a.so_f,
                          reinterpret_cast<float2*>(a.outr), reinterpret_cast<float2*>(a.outi), a.nbk, a.npsi,
                          a.use_e0, reinterpret_cast<const float2*>(a.oldr), reinterpret_cast<const float2*>(a.oldi),
                          a.rb_base, a.itp, reinterpret_cast<float2*>(a.red), a.bs, blockIdx.x, blockIdx.y, a.nblk);
}

// Operator data of the double-float loop, from the FP64 copies: energies as
// double-float, the mask and the spin-orbit matrix as binary32.
__global__ void k_df_operators(const double* __restrict__ er, const double* __restrict__ ei,
                               const double* __restrict__ allow, const double2* __restrict__ so, float2* __restrict__ erd,
                               float2* __restrict__ eid, float* __restrict__ allowf, float2* __restrict__ sof, size_t n,
                               int nso) {
  const size_t m = n > (size_t)nso ? n : (size_t)nso;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) {
    if (i < n) {
      df_st(erd, i, df_split(er[i]));
      df_st(eid, i, df_split(ei[i]));
      allowf[i] = (float)allow[i];
    }
    if (i < (size_t)nso) sof[i] = make_float2((float)so[i].x, (float)so[i].y);
  }
}

// FP64 values -> double-float in place (element i keeps its 8 bytes)
__global__ void k_to_df_inplace(double* __restrict__ v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const df d = df_split(v[i]);
    reinterpret_cast<float2*>(v)[i] = make_float2(d.h, d.l);
  }
}

// Sum of nb partial pairs in a fixed order, done identically by every block.
__device__ __forceinline__ void reduce_pairs(const double* __restrict__ red, int nblk, double* s0,
                                             double* s1) {
  __shared__ double sh[2][32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += red[2 * i];
    b += red[2 * i + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
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

__device__ __forceinline__ void block_partial(double v0, double v1, double* __restrict__ red,
                                              int bx = -1) {
  if (bx < 0) bx = blockIdx.x;
  __shared__ double sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = v0;
    sh[1][w] = v1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      s0 += sh[0][i];
      s1 += sh[1][i];
    }
    red[2 * bx] = s0;
    red[2 * bx + 1] = s1;
  }
}

// Iteration counter of the device-resident Lanczos loop (coefficient index i).
__global__ void k_advance(int* __restrict__ itp) { *itp += 1; }
__global__ void k_advance_group(int* const* __restrict__ itps, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) *itps[i] += 1;
}

// Lanczos stage 2: a_{i-1} = Re<h|psi>; h -= a psi; partial |h|^2.
__device__ __forceinline__ void lanczos2_body(const double* __restrict__ red1, int nblk, double* __restrict__ hr,
                           double* __restrict__ hi, const double* __restrict__ pr,
                           const double* __restrict__ pi, size_t n, double* __restrict__ red2,
                           double* __restrict__ ra_base, double* __restrict__ ia_base,
                           const int* __restrict__ itp, const BlockStrides bs, int bx, int by,
                           int nbx) {
  const size_t v = by;
  red1 += v * bs.red;
  red2 += v * bs.red;
  hr += v * bs.vec;
  hi += v * bs.vec;
  pr += v * bs.vec;
  pi += v * bs.vec;
  ra_base += v * bs.coef;
  ia_base += v * bs.coef;
  double a, ia;
  reduce_pairs(red1, nblk, &a, &ia);
  if (bx == 0 && threadIdx.x == 0) {
    const int it = *itp;
    ra_base[it - 1] = a;
    ia_base[it - 1] = ia;
  }
  const double am = -a;
  double s = 0.0;
  for (size_t e = bx * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)nbx * blockDim.x) {
    const double r = hr[e] + am * pr[e];
    const double i = hi[e] + am * pi[e];
    hr[e] = r;
    hi[e] = i;
    s += r * r + i * i;
  }
  __syncthreads();
  block_partial(s, 0.0, red2, bx);
}

__global__ void __launch_bounds__(LZ_THREADS)
    k_lanczos2(const double* __restrict__ red1, int nblk, double* __restrict__ hr, double* __restrict__ hi,
               const double* __restrict__ pr, const double* __restrict__ pi, size_t n,
               double* __restrict__ red2, double* __restrict__ ra_base, double* __restrict__ ia_base,
               const int* __restrict__ itp, const BlockStrides bs) {
  lanczos2_body(red1, nblk, hr, hi, pr, pi, n, red2, ra_base, ia_base, itp, bs, blockIdx.x, blockIdx.y, gridDim.x);
}


// Lanczos stage 3: b_i = sqrt(sum); psi_new = h / b_i (in place in h).
__global__ void __launch_bounds__(LZ_THREADS) k_lanczos3(const double* __restrict__ red2, int nblk, double* __restrict__ hr,
                           double* __restrict__ hi, size_t n, double* __restrict__ rb_base,
                           const int* __restrict__ itp, const BlockStrides bs) {
  const size_t v = blockIdx.y;
  red2 += v * bs.red;
  hr += v * bs.vec;
  hi += v * bs.vec;
  rb_base += v * bs.coef;
  double bb, dummy;
  reduce_pairs(red2, nblk, &bb, &dummy);
  const double b = sqrt(bb);
  if (blockIdx.x == 0 && threadIdx.x == 0) rb_base[*itp] = b;
  const double inv = 1.0 / b;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    hr[e] *= inv;
    hi[e] *= inv;
  }
}

// ---------------------------------------------------------------- multiplet

// amp_part[chunk][p][a] = sum_{e in chunk} (allow o psi)(e,a) * mpc_s(p)(e), e = (n,k)
// (OCEAN_multiplet.f90:1730-1783).  One warp per projector at a time.
__global__ void k_mult_amp(const double* __restrict__ pr, const double* __restrict__ pi,
                           const double* __restrict__ allow, const double2* __restrict__ mpc,
                           double2* __restrict__ amp_part, int nbk, int np, int na, int nspn,
                           int chunk) {
  extern __shared__ double2 qs[];  // [a][chunk]
  const int c0 = blockIdx.x * chunk;
  const int cn = min(chunk, nbk - c0);
  for (int e = threadIdx.x; e < na * chunk; e += blockDim.x) {
    const int a = e / chunk, j = e % chunk;
    double2 v = make_double2(0.0, 0.0);
    if (j < cn) {
      const size_t idx = (size_t)c0 + j + (size_t)nbk * a;
      const double m = allow[idx];
      v = make_double2(pr[idx] * m, pi[idx] * m);
    }
    qs[e] = v;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int p = warp; p < np; p += nw) {
    double2 s[OCN_MAX_NA];
#pragma unroll
    for (int a = 0; a < OCN_MAX_NA; ++a) s[a] = make_double2(0.0, 0.0);
    for (int j = lane; j < cn; j += 32) {
      const double2 m0 = mpc[((size_t)0 * np + p) * nbk + c0 + j];
      const double2 m1 = (nspn == 2) ? mpc[((size_t)1 * np + p) * nbk + c0 + j] : m0;
#pragma unroll
      for (int a = 0; a < OCN_MAX_NA; ++a)
        if (a < na) {
          const double2 m = ((a & 1) && nspn == 2) ? m1 : m0;
          const double2 q = qs[a * chunk + j];
          s[a].x += q.x * m.x - q.y * m.y;
          s[a].y += q.x * m.y + q.y * m.x;
        }
    }
#pragma unroll
    for (int a = 0; a < OCN_MAX_NA; ++a) {
      if (a >= na) break;
      for (int o = 16; o > 0; o >>= 1) {
        s[a].x += __shfl_down_sync(0xffffffffu, s[a].x, o);
        s[a].y += __shfl_down_sync(0xffffffffu, s[a].y, o);
      }
      if (lane == 0) amp_part[((size_t)blockIdx.x * np + p) * na + a] = s[a];
    }
  }
}

__global__ void k_mult_amp_reduce(const double2* __restrict__ part, double2* __restrict__ amp,
                                  int nchunk, int npa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npa) return;
  double2 s = make_double2(0.0, 0.0);
  for (int c = 0; c < nchunk; ++c) {
    const double2 v = part[(size_t)c * npa + i];
    s.x += v.x;
    s.y += v.y;
  }
  amp[i] = s;
}

// hamp(p,a) = mul * ( -sum_nu' mpm(nu,nu',l) amp((nu',m,l),a)
//                     + sum_jj MH_l(ii(nu,m,a), jj) pw_l(jj) )
// (OCEAN_multiplet.f90:1819-1936).  One warp per (p, a).
__global__ void k_mult_hamp(const double2* __restrict__ amp, double2* __restrict__ hamp,
                            const int* __restrict__ pl, const int* __restrict__ pm,
                            const int* __restrict__ pnu, const int* __restrict__ pfirst,
                            const double* __restrict__ mpm, const double2* __restrict__ mh,
                            const long long* __restrict__ jbeg, const int* __restrict__ nprojv,
                            int np, int na, int lmin, int npmax, double mul) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= np * na) return;
  const int p = gw / na, a = gw % na;
  const int l = pl[p], m = pm[p], nu = pnu[p];
  const int li = l - lmin;
  const int npl = nprojv[li];
  const int first = pfirst[li];  // first projector index of block l (m = -l, nu = 0)
  double2 s = make_double2(0.0, 0.0);
  // direct term
  for (int nup = lane; nup < npl; nup += 32) {
    const double mm = mpm[(size_t)nu + (size_t)npmax * ((size_t)nup + (size_t)npmax * li)];
    const int q = first + (m + l) * npl + nup;
    const double2 v = amp[(size_t)q * na + a];
    s.x -= mm * v.x;
    s.y -= mm * v.y;
  }
  // exchange term: pw_l(jj), jj = nu' + (m'+l) npl + a' (2l+1) npl
  const int mham = na * (2 * l + 1) * npl;
  const int ii = nu + (m + l) * npl + a * (2 * l + 1) * npl;
  const double2* row = mh + jbeg[li] + (size_t)ii * mham;
  for (int jj = lane; jj < mham; jj += 32) {
    const int nup = jj % npl;
    const int mp = (jj / npl) % (2 * l + 1);
    const int ap = jj / (npl * (2 * l + 1));
    const int q = first + mp * npl + nup;
    const double2 v = amp[(size_t)q * na + ap];
    const double2 h = row[jj];
    s.x += h.x * v.x - h.y * v.y;
    s.y += h.x * v.y + h.y * v.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, o);
    s.y += __shfl_down_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) hamp[(size_t)p * na + a] = make_double2(s.x * mul, s.y * mul);
}

// acc(e,a) += sum_p conj(mpc_s(p)(e)) hamp(p,a)   (OCEAN_multiplet.f90:1943-1998)
__global__ void k_mult_back(const double2* __restrict__ mpc, const double2* __restrict__ hamp,
                            double* __restrict__ acc, int nbk, int np, int na, int nspn,
                            size_t npsi) {
  extern __shared__ double2 hs[];  // [p][a]
  for (int i = threadIdx.x; i < np * na; i += blockDim.x) hs[i] = hamp[i];
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nbk) return;
  double2 s[OCN_MAX_NA];
#pragma unroll
  for (int a = 0; a < OCN_MAX_NA; ++a) s[a] = make_double2(0.0, 0.0);
  for (int p = 0; p < np; ++p) {
    const double2 m0 = mpc[((size_t)0 * np + p) * nbk + e];
    const double2 m1 = (nspn == 2) ? mpc[((size_t)1 * np + p) * nbk + e] : m0;
#pragma unroll
    for (int a = 0; a < OCN_MAX_NA; ++a)
      if (a < na) {
        const double2 m = ((a & 1) && nspn == 2) ? m1 : m0;
        const double2 h = hs[p * na + a];
        s[a].x += m.x * h.x + m.y * h.y;
        s[a].y += m.x * h.y - m.y * h.x;
      }
  }
#pragma unroll
  for (int a = 0; a < OCN_MAX_NA; ++a)
    if (a < na) {
      acc[e + (size_t)nbk * a] += s[a].x;
      acc[npsi + e + (size_t)nbk * a] += s[a].y;
    }
}

// ------------------------------------------------------------ BLAS-1 (GMRES)

// y = (rv + i iv) x - y   (OCEAN_psi_axmy, OCEAN_psi.f90:1515-1522)
__global__ void k_axmy(const double* __restrict__ x, double* __restrict__ y, size_t n, double rv,
                       double iv) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double xr = x[e], xi = x[n + e];
    const double br = rv * xr - y[e];
    const double bi = rv * xi - y[n + e];
    y[e] = br - iv * xi;
    y[n + e] = bi + iv * xr;
  }
}
// y = x - z
__global__ void k_axmz(const double* __restrict__ x, double* __restrict__ y,
                       const double* __restrict__ z, size_t n2) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n2;
       e += (size_t)gridDim.x * blockDim.x)
    y[e] = x[e] - z[e];
}
// y += (ar + i ai) x
__global__ void k_axpy(double ar, double ai, const double* __restrict__ x, double* __restrict__ y,
                       size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double xr = x[e], xi = x[n + e];
    y[e] += ar * xr - ai * xi;
    y[n + e] += ar * xi + ai * xr;
  }
}
// z = x o y (complex)
__global__ void k_cmul(const double* __restrict__ x, const double* __restrict__ y,
                       double* __restrict__ z, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double a = x[e], b = x[n + e], c = y[e], d = y[n + e];
    z[e] = a * c - b * d;
    z[n + e] = a * d + b * c;
  }
}
// pcdiv = (E - (h_r + i(h_i + g))) / ((E - h)^2 + g^2)  (OCEAN_psi.f90:2961-2965)
__global__ void k_set_prec(double energy, double gprc, const double* __restrict__ h,
                           double* __restrict__ out, size_t n) {
  const double g2 = gprc * gprc;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double hr = h[e], hi = h[n + e];
    const double er = energy - hr, ei = -hi;
    const double dr = er * er - ei * ei + g2, di = 2.0 * er * ei;
    const double nr = energy - hr, ni = -(hi + gprc);
    const double den = dr * dr + di * di;
    out[e] = (nr * dr + ni * di) / den;
    out[n + e] = (ni * dr - nr * di) / den;
  }
}
__global__ void k_mask_copy(const double* __restrict__ in, const double* __restrict__ allow,
                            double* __restrict__ out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double m = allow[e];
    out[e] = m * in[e];
    out[n + e] = m * in[n + e];
  }
}
// x = allow o x in place (OCEAN_energies_allow)
__global__ void k_mask_inplace(double* __restrict__ x, const double* __restrict__ allow, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double m = allow[e];
    x[e] *= m;
    x[n + e] *= m;
  }
}
// x /= (rv + i iv) as OCEAN_psi_divide does it (OCEAN_psi.f90:1797-1808)
__global__ void k_cdivide(double* __restrict__ x, size_t n, double rn, double in) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double xr = x[e], xi = x[n + e];
    const double buf = -in * xr;
    x[e] = rn * xr + in * xi;
    x[n + e] = buf + rn * xi;
  }
}
__global__ void k_fill(double* __restrict__ x, size_t n, double vr, double vi) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    x[e] = vr;
    x[n + e] = vi;
  }
}
// partial <p|q> = sum conj(p) q
__global__ void k_dot(const double* __restrict__ p, const double* __restrict__ q, size_t n,
                      double* __restrict__ red) {
  double a = 0.0, b = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const double pr = p[e], pi = p[n + e], qr = q[e], qi = q[n + e];
    a += pr * qr + pi * qi;
    b += pr * qi - pi * qr;
  }
  block_partial(a, b, red);
}
__global__ void k_reduce_final(const double* __restrict__ red, int nblk, double* __restrict__ out) {
  double a, b;
  reduce_pairs(red, nblk, &a, &b);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}


typedef decltype(&k_combine<4, false, double>) CombineFn;
// f32_parts: the partials come from the tensor-core contractions (mixed precision)
CombineFn combine_kernel(int na, int use_so, bool f32_parts) {
  if (f32_parts) {
    if (na == 4) return use_so ? k_combine<4, true, float> : k_combine<4, false, float>;
    return use_so ? k_combine<12, true, float> : k_combine<12, false, float>;
  }
  if (na == 4) return use_so ? k_combine<4, true, double> : k_combine<4, false, double>;
  return use_so ? k_combine<12, true, double> : k_combine<12, false, double>;
}
typedef decltype(&k_combine_df<4, false>) CombineDfFn;
CombineDfFn combine_df_kernel(int na, int use_so) {
  if (na == 4) return use_so ? k_combine_df<4, true> : k_combine_df<4, false>;
  return use_so ? k_combine_df<12, true> : k_combine_df<12, false>;
}

inline int grid_for(size_t n, int block, int cap) {
  size_t g = (n + block - 1) / block;
  if (g > (size_t)cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

// ======================================================================= host

int upload_twiddles(ocn_ctx* c) {
  double2 tw[3][OCN_MAX_KDIM];
  const double pi = 3.1415926535897932384626433832795;
  for (int a = 0; a < 3; ++a) {
    const int n = c->dims.kmesh[a];
    for (int t = 0; t < OCN_MAX_KDIM; ++t) {
      if (t < n) {
        const double ang = 2.0 * pi * (double)t / (double)n;
        tw[a][t] = make_double2(cos(ang), sin(ang));
      } else {
        tw[a][t] = make_double2(0.0, 0.0);
      }
    }
  }
  // per context: contexts with different k-meshes coexist in one process
  if (!c->d_tw) OCN_CUDA(c, cudaMalloc(reinterpret_cast<void**>(&c->d_tw), sizeof(tw)));
  OCN_CUDA(c, cudaMemcpyAsync(c->d_tw, tw, sizeof(tw), cudaMemcpyHostToDevice, c->stream));
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  return OCN_OK;
}

int kernels_init(ocn_ctx* c) {
  int optin = 0;
  OCN_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  const size_t g1 = sizeof(double2) * ((size_t)c->nspn * G1_N * (G1_X + 1) + (size_t)c->na * G1_N);
  const size_t ma = sizeof(double2) * (size_t)c->na * 256;
  const bool cube = kmesh_cube_supported(c->dims.kmesh);
  const size_t ff = cube ? kmesh_cube_smem<double>(c->dims.kmesh[0], c->na)
                         : kmesh_smem(kmesh_geom<double>(c->dims.kmesh, c->na));
  if (g1 > (size_t)optin || ma > (size_t)optin || ff > (size_t)optin)
    return set_err(c, OCN_ERR_ARG, "k-mesh or nalpha too large for the shared-memory kernels");
  if (int rc_ = allow_max_smem(c, k_lr_gemm1_fp64)) return rc_;
  if (int rc_ = allow_max_smem(c, k_lr_fft_w_fp64)) return rc_;
  if (cube) {
    CubeFnD f;
    OCN_CUBE_DISPATCH(k_fft_cube_fp64, c->dims.kmesh[0], c->na, f);
    if (int rc_ = allow_max_smem(c, f)) return rc_;
  }
  if (int rc_ = allow_max_smem(c, k_mult_amp)) return rc_;
  return OCN_OK;
}

int phase_bloch(ocn_ctx* c, const double* d_ur, const double* d_ui, const double* d_cos,
                const double* d_sin) {
  const long long total = (long long)c->nb * c->nk * c->nx * c->nspn;
  k_phase_bloch<<<grid_for((size_t)total, 256, 8 * c->sm_count), 256, 0, c->stream>>>(
      d_ur, d_ui, d_cos, d_sin, c->d_u, total, c->nb, c->nk, c->nx);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int zero_acc(ocn_ctx* c, int nv) {
  OCN_CUDA(c, cudaMemsetAsync(c->d_acc, 0, sizeof(double) * 2 * c->npsi * nv, c->stream));
  return OCN_OK;
}

int lr_apply_fp64(ocn_ctx* c, const double* d_pr, const double* d_pi) {
  const int nb = c->nb, nk = c->nk, nx = c->nx, na = c->na;
  {
    const size_t sm = sizeof(double2) * ((size_t)c->nspn * G1_N * (G1_X + 1) + (size_t)na * G1_N);
    dim3 grid((nx + G1_X - 1) / G1_X, nk);
    TimedScope ts(c, T_LR_GEMM1);
    k_lr_gemm1_fp64<<<grid, G1_X, sm, c->stream>>>(c->d_u, d_pr, d_pi, c->d_allow, c->d_phi, nb, nk,
                                                   nx, na, c->nspn);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  {
    const KmeshGeom<double> g = kmesh_geom<double>(c->dims.kmesh, na);
    TimedScope ts(c, T_LR_FFT);
    CubeFnD f = nullptr;
    if (kmesh_cube_supported(c->dims.kmesh)) OCN_CUBE_DISPATCH(k_fft_cube_fp64, c->dims.kmesh[0], na, f);
    if (f)
      f<<<nx, 128, kmesh_cube_smem<double>(c->dims.kmesh[0], na), c->stream>>>(c->d_phi, c->d_W, nx, na,
                                                                               c->d_tw);
    else
      k_lr_fft_w_fp64<<<nx, 256, kmesh_smem(g), c->stream>>>(c->d_phi, c->d_W, nx, g, c->d_tw);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  {
    const int xs = c->lr_xsplit;
    const int xper = (nx + xs - 1) / xs;
    const int block = ((nb + 31) / 32) * 32;
    dim3 grid(nk, xs);
    TimedScope ts(c, T_LR_GEMM2);
    k_lr_gemm2_fp64<<<grid, block, 0, c->stream>>>(c->d_u, c->d_phi, c->d_accpart, nb, nk, nx, na,
                                                   c->nspn, xper, c->npsi);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  return OCN_OK;
}

bool lr_wgrad_supported(const ocn_ctx* c) {
  return kmesh_cube_supported(c->dims.kmesh) &&
         kmesh_cube_smem<double>(c->dims.kmesh[0], 2 * c->na) <= (size_t)227 * 1024;
}

int lr_wgrad_fp64(ocn_ctx* c, const double* x, const double* y, double2* phi, double a, double b, double* gW) {
  if (!lr_wgrad_supported(c)) return set_err(c, OCN_ERR_UNSUPPORTED, "W gradient needs a supported cubic k-mesh");
  const int nb = c->nb, nk = c->nk, nx = c->nx, na = c->na;
  const size_t n = c->npsi;
  double2* phx = phi;
  double2* phy = phi + (size_t)nk * nx * na;
  const size_t sm = sizeof(double2) * ((size_t)c->nspn * G1_N * (G1_X + 1) + (size_t)na * G1_N);
  const dim3 grid((nx + G1_X - 1) / G1_X, nk);
  k_lr_gemm1_fp64<<<grid, G1_X, sm, c->stream>>>(c->d_u, x, x + n, c->d_allow, phx, nb, nk, nx, na, c->nspn);
  k_lr_gemm1_fp64<<<grid, G1_X, sm, c->stream>>>(c->d_u, y, y + n, c->d_allow, phy, nb, nk, nx, na, c->nspn);
  c->launches += 2;
  OCN_CUDA(c, cudaGetLastError());
  WgradFnD f = wgrad_fn(c->dims.kmesh[0]);
  const size_t wsm = kmesh_cube_smem<double>(c->dims.kmesh[0], 2 * na);
  if (int rc_ = allow_max_smem(c, f)) return rc_;
  f<<<nx, 128, wsm, c->stream>>>(phx, phy, nx, na, gW, a, b, c->d_tw);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

// hamp = mul (-mpm amp + MH amp) of one vector (k_mult_hamp), amp/hamp [p][a]
int mult_hamp(ocn_ctx* c, const double2* amp, double2* hamp) {
  MultDev& m = c->mult;
  const double mul = c->sys.interaction_scale / ((double)c->nk * c->sys.celvol);
  const int npa = m.np * c->na;
  const int threads = 256;
  const int blocks = (npa * 32 + threads - 1) / threads;
  k_mult_hamp<<<blocks, threads, 0, c->stream>>>(amp, hamp, m.p_l, m.p_m, m.p_nu, m.d_pfirst, m.mpm, m.mh,
                                                m.d_jbeg, m.d_nproj, m.np, c->na, m.lmin, m.npmax, mul);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

// Slices of d_accpart that hold terms of the current action: the long-range
// K-split partials, followed (mixed precision) by the multiplet's.
void active_parts(const ocn_ctx* c, const int* hf, const void** base, int* count) {
  const bool lr = c->sys.long_range && hf[0] == 1;
  const bool mm = c->mult_parts > 0 && c->sys.mult && hf[4] == 1 && c->have_mult;
  const size_t off = lr ? 0 : (size_t)c->lr_xsplit * c->part_stride;  // elements
  if (mixed_parts(c)) *base = reinterpret_cast<const float*>(c->d_accpart) + off;
  else *base = c->d_accpart + off;
  *count = (lr ? c->lr_xsplit : 0) + (mm ? c->mult_parts : 0);
}

int mult_apply(ocn_ctx* c, const double* d_pr, const double* d_pi, double* acc) {
  MultDev& m = c->mult;
  TimedScope ts(c, T_MULT);
  const int nbk = c->nb * c->nk;
  const int chunk = 256;
  const int nchunk = (nbk + chunk - 1) / chunk;
  {
    const size_t sm = sizeof(double2) * (size_t)c->na * chunk;
    k_mult_amp<<<nchunk, 256, sm, c->stream>>>(d_pr, d_pi, c->d_allow, m.mpc, m.amp_part, nbk, m.np,
                                              c->na, c->nspn, chunk);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  const int npa = m.np * c->na;
  k_mult_amp_reduce<<<(npa + 127) / 128, 128, 0, c->stream>>>(m.amp_part, m.amp, nchunk, npa);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  {
    const double mul = c->sys.interaction_scale / ((double)c->nk * c->sys.celvol);
    const int warps = npa;
    const int threads = 256;
    const int blocks = (warps * 32 + threads - 1) / threads;
    k_mult_hamp<<<blocks, threads, 0, c->stream>>>(m.amp, m.hamp, m.p_l, m.p_m, m.p_nu, m.d_pfirst,
                                                  m.mpm, m.mh, m.d_jbeg, m.d_nproj, m.np, c->na,
                                                  m.lmin, m.npmax, mul);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  {
    const size_t sm = sizeof(double2) * (size_t)npa;
    const int block = 64;
    k_mult_back<<<(nbk + block - 1) / block, block, sm, c->stream>>>(m.mpc, m.hamp, acc, nbk, m.np,
                                                                    c->na, c->nspn, c->npsi);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
  }
  return OCN_OK;
}

int combine(ocn_ctx* c, int nv, const double* d_pr, const double* d_pi, double* d_or, double* d_oi,
            size_t vstride, const int* hflag, int backwards, int v0) {
  const int nbk = c->nb * c->nk;
  const int use_so = (c->sys.mult && hflag[5] == 1 && c->have_so) ? 1 : 0;
  const void* parts;
  int nparts;
  active_parts(c, hflag, &parts, &nparts);
  const BlockStrides bs = {vstride, c->part_stride, 0, 0};
  const bool f32 = mixed_parts(c);
  auto kern = combine_kernel(c->na, use_so, f32);
  dim3 grid(grid_for(c->npsi, LZ_THREADS, 4 * c->sm_count), nv);
  // vector v0 of the block: its long-range partials and multiplet accumulator
  const void* pv = f32 ? static_cast<const void*>(static_cast<const float*>(parts) + (size_t)v0 * 2 * c->npsi)
                       : static_cast<const void*>(static_cast<const double*>(parts) + (size_t)v0 * 2 * c->npsi);
  kern<<<grid, LZ_THREADS, 0, c->stream>>>(
      d_pr, d_pi, c->d_er, c->ei_nonzero ? c->d_ei : nullptr, c->d_allow,
      c->acc_valid ? c->d_acc + (size_t)v0 * vstride : nullptr, pv, nparts,
      c->d_so, d_or, d_oi, nbk, c->na, c->npsi, c->sys.e0, use_so, backwards, nullptr, nullptr,
      nullptr, nullptr, nullptr, bs);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

// Fused combine + ocean_hay_ab_twoterm for iteration i = *itp of nv chains:
// reads b_{i-1} from rb, writes a_{i-1}, Im a_{i-1} and b_i
// (OCEAN_haydock.f90:848-889).  old/psi/h are block bases (vector stride 2*npsi),
// ra/ia/rb coefficient bases with cstride between chains.  Mixed precision: the
// vectors are double-float planes (haydock_to_df) and the step runs on the FP32
// pipe; FP64: the reference's arithmetic in FP64.
int lanczos_launch(ocn_ctx* c, int nv, const double* old, const double* psi, double* h, double* ra,
                   double* ia, double* rb, size_t cstride, const int* itp) {
  const int nbk = c->nb * c->nk;
  const size_t n = c->npsi;
  const int* hf = c->sys.nhflag;
  const int use_so = (c->sys.mult && hf[5] == 1 && c->have_so) ? 1 : 0;
  const void* parts;
  int nparts;
  active_parts(c, hf, &parts, &nparts);
  const int nblk = c->red_blocks;
  const BlockStrides bs = {2 * n, c->part_stride, cstride, (size_t)4 * nblk};
  TimedScope ts(c, T_LANCZOS);
  dim3 grid(nblk, nv);
  if (mixed_parts(c)) {
    typedef const float2* cf2;
    auto kd = combine_df_kernel(c->na, use_so);
    kd<<<grid, LZ_DF_THREADS, 0, c->stream>>>(
        reinterpret_cast<cf2>(psi), reinterpret_cast<cf2>(psi + n), c->d_er_df, c->ei_nonzero ? c->d_ei_df : nullptr,
        c->d_allow_f, static_cast<const float*>(parts), nparts, c->d_so_f, reinterpret_cast<float2*>(h),
        reinterpret_cast<float2*>(h + n), nbk, n, c->sys.e0, reinterpret_cast<cf2>(old), reinterpret_cast<cf2>(old + n),
        rb, itp, reinterpret_cast<float2*>(c->d_red), bs);
    ++c->launches;
    OCN_CUDA(c, cudaGetLastError());
    // a_{i-1}, b_i, psi = (h - a psi) / b_i and the next psi operand
    return mixed_norm_prep(c, nv, psi, h, ra, ia, rb, cstride, itp);
  }
  auto kern = combine_kernel(c->na, use_so, false);
  kern<<<grid, LZ_THREADS, 0, c->stream>>>(psi, psi + n, c->d_er, c->ei_nonzero ? c->d_ei : nullptr,
                                    c->d_allow, c->acc_valid ? c->d_acc : nullptr, parts,
                                    nparts, c->d_so, h, h + n, nbk, c->na, n, c->sys.e0, use_so, 0,
                                    old, old + n, rb, itp, c->d_red, bs);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  k_lanczos2<<<grid, LZ_THREADS, 0, c->stream>>>(c->d_red, nblk, h, h + n, psi, psi + n, n, c->d_red + 2 * nblk,
                                          ra, ia, itp, bs);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  k_lanczos3<<<grid, LZ_THREADS, 0, c->stream>>>(c->d_red + 2 * nblk, nblk, h, h + n, n, rb, itp, bs);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

// The double-float operator copies (allocated by the caller) and the first
// vectors of a mixed-precision Haydock run: nv chains of FP64 planes at buf
// (vector stride 2n) converted in place.
int haydock_to_df(ocn_ctx* c, double* buf, int nv) {
  const size_t n = c->npsi;
  const int nso = c->na * c->na;
  k_df_operators<<<grid_for(std::max(n, (size_t)nso), 256, 4 * c->sm_count), 256, 0, c->stream>>>(
      c->d_er, c->d_ei, c->d_allow, c->d_so, c->d_er_df, c->d_ei_df, c->d_allow_f, c->d_so_f, n, nso);
  k_to_df_inplace<<<grid_for(2 * n * nv, 256, 4 * c->sm_count), 256, 0, c->stream>>>(buf, 2 * n * nv);
  c->launches += 2;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int advance_iter(ocn_ctx* c, int* itp) {
  k_advance<<<1, 1, 0, c->stream>>>(itp);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int vec_axmy(ocn_ctx* c, const double* x, double* y, double rv, double iv) {
  k_axmy<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, y, c->npsi, rv, iv);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_axmz(ocn_ctx* c, const double* x, double* y, const double* z) {
  k_axmz<<<grid_for(2 * c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, y, z, 2 * c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_axpy(ocn_ctx* c, double ar, double ai, const double* x, double* y) {
  k_axpy<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(ar, ai, x, y, c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_mul(ocn_ctx* c, const double* x, const double* y, double* z) {
  k_cmul<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, y, z, c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_set_prec(ocn_ctx* c, double energy, double gprc, const double* h, double* out) {
  k_set_prec<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(energy, gprc, h, out,
                                                                              c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_mask_copy(ocn_ctx* c, const double* in, double* out) {
  k_mask_copy<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(in, c->d_allow, out,
                                                                               c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_mask_inplace(ocn_ctx* c, double* x) {
  k_mask_inplace<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, c->d_allow, c->npsi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_divide(ocn_ctx* c, double* x, double rv, double iv) {
  const double denom = rv * rv + iv * iv;
  k_cdivide<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, c->npsi, rv / denom, iv / denom);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
int vec_fill(ocn_ctx* c, double* x, double vr, double vi) {
  k_fill<<<grid_for(c->npsi, 256, 4 * c->sm_count), 256, 0, c->stream>>>(x, c->npsi, vr, vi);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}
// Device-resident <p|q>; result pair written to d_out (2 doubles).
int vec_dot_dev(ocn_ctx* c, const double* p, const double* q, double* d_out) {
  const int nblk = c->red_blocks;
  k_dot<<<nblk, 256, 0, c->stream>>>(p, q, c->npsi, c->d_red);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  k_reduce_final<<<1, 256, 0, c->stream>>>(c->d_red, nblk, d_out);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

// ---------------------------------------------------- grouped Lanczos steps

struct LzGroup {
  int n = 0, nvmax = 1, nblk = 0;
  // members ordered by (Na, spin-orbit) class; class c covers records cls[c].first ..
  struct Cls {
    int na, so, first, count;
  };
  std::vector<Cls> cls;
  std::vector<int> order;  // member index of each record
  CombineArgs* d_comb[3] = {nullptr, nullptr, nullptr};
  int** d_iters = nullptr;
};

void lz_group_destroy(LzGroup* g) {
  if (!g) return;
  for (int r = 0; r < 3; ++r) {
    if (g->d_comb[r]) cudaFree(g->d_comb[r]);
  }
  if (g->d_iters) cudaFree(g->d_iters);
  delete g;
}

// The records of lanczos_launch for every member and each of the three buffer
// rotations of a captured three-iteration graph (grouped members are mixed
// precision: double-float vectors).
int lz_group_create(const std::vector<BatchMember>& mem, LzGroup** out) {
  *out = nullptr;
  if (mem.empty()) return OCN_ERR_ARG;
  ocn_ctx* c0 = mem[0].c;
  LzGroup* g = new (std::nothrow) LzGroup();
  if (!g) return set_err(c0, OCN_ERR_ALLOC, "host allocation failed");
  g->n = (int)mem.size();
  g->nblk = c0->red_blocks;
  std::vector<int*> iters;
  std::vector<CombineArgs> ca(mem.size());
  int rc = OCN_OK;
  for (const BatchMember& b : mem) {
    g->nvmax = std::max(g->nvmax, b.nv);
    g->nblk = std::max(g->nblk, b.c->red_blocks);
    iters.push_back(b.c->d_iter);
  }
  for (int na : {4, 12})
    for (int so : {0, 1}) {
      LzGroup::Cls k{na, so, (int)g->order.size(), 0};
      for (size_t i = 0; i < mem.size(); ++i) {
        const ocn_ctx* c = mem[i].c;
        const int cso = (c->sys.mult && c->sys.nhflag[5] == 1 && c->have_so) ? 1 : 0;
        if (c->na == na && cso == so) {
          g->order.push_back((int)i);
          ++k.count;
        }
      }
      if (k.count) g->cls.push_back(k);
    }
  if (g->order.size() != mem.size()) rc = set_err(c0, OCN_ERR_UNSUPPORTED, "batched context with Na other than 4, 12");
  for (int r = 0; r < 3 && rc == OCN_OK; ++r) {
    for (size_t i = 0; i < g->order.size(); ++i) {
      const BatchMember& b = mem[g->order[i]];
      ocn_ctx* c = b.c;
      const size_t n = c->npsi;
      const double* old = b.buf[r % 3];
      const double* psi = b.buf[(r + 1) % 3];
      double* h = b.buf[(r + 2) % 3];
      const int* hf = c->sys.nhflag;
      const void* parts;  // binary32 partials (grouped members are mixed precision)
      int nparts;
      active_parts(c, hf, &parts, &nparts);
      const int nblk = c->red_blocks;
      const BlockStrides bs = {2 * n, c->part_stride, b.cstride, (size_t)4 * nblk};
      CombineArgs& a = ca[i];
      a.pr = psi;
      a.pi = psi + n;
      a.er = c->d_er;
      a.ei = c->ei_nonzero ? c->d_ei : nullptr;
      a.allow = c->d_allow;
      a.acc = nullptr;  // grouped members have no multiplet term
      a.part = static_cast<const double*>(parts);  // read as binary32 by k_combine_df_group
      a.nparts = nparts;
      a.so = c->d_so;
      a.outr = h;
      a.outi = h + n;
      a.nbk = c->nb * c->nk;
      a.na = c->na;
      a.npsi = n;
      a.use_e0 = c->sys.e0;
      a.use_so = (c->sys.mult && hf[5] == 1 && c->have_so) ? 1 : 0;
      a.backwards = 0;
      a.oldr = old;
      a.oldi = old + n;
      a.rb_base = b.rb;
      a.itp = c->d_iter;
      a.red = c->d_red;
      a.bs = bs;
      a.er_df = c->d_er_df;
      a.ei_df = c->ei_nonzero ? c->d_ei_df : nullptr;
      a.allow_f = c->d_allow_f;
      a.so_f = c->d_so_f;
      a.nv = b.nv;
      a.nblk = nblk;
    }
    cudaError_t e = cudaMalloc(&g->d_comb[r], ca.size() * sizeof(CombineArgs));
    if (e == cudaSuccess) e = cudaMemcpy(g->d_comb[r], ca.data(), ca.size() * sizeof(CombineArgs), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(c0, e, "batched Lanczos tables");
  }
  if (rc == OCN_OK) {
    cudaError_t e = cudaMalloc(&g->d_iters, iters.size() * sizeof(int*));
    if (e == cudaSuccess) e = cudaMemcpy(g->d_iters, iters.data(), iters.size() * sizeof(int*), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(c0, e, "batched Lanczos tables");
  }
  if (rc != OCN_OK) {
    lz_group_destroy(g);
    return rc;
  }
  *out = g;
  return OCN_OK;
}

// Kernels of one lz_group_advance + lz_group_step.
int lz_group_launches(const LzGroup* g) { return 1 + (int)g->cls.size(); }

int lz_group_advance(LzGroup* g, cudaStream_t s) {
  k_advance_group<<<(g->n + 127) / 128, 128, 0, s>>>(g->d_iters, g->n);
  return cudaGetLastError() == cudaSuccess ? OCN_OK : OCN_ERR_CUDA;
}

// combine (E, masks, long-range parts, -b psi_old, <h|psi>) and stage 2 for
// every member, buffer rotation rot
int lz_group_step(LzGroup* g, int rot, cudaStream_t s) {
  for (const LzGroup::Cls& k : g->cls) {
    const dim3 gc(g->nblk, g->nvmax, k.count);
    const CombineArgs* t = g->d_comb[rot] + k.first;
    if (k.na == 4) {
      if (k.so) k_combine_df_group<4, true><<<gc, LZ_DF_THREADS, 0, s>>>(t);
      else k_combine_df_group<4, false><<<gc, LZ_DF_THREADS, 0, s>>>(t);
    } else {
      if (k.so) k_combine_df_group<12, true><<<gc, LZ_DF_THREADS, 0, s>>>(t);
      else k_combine_df_group<12, false><<<gc, LZ_DF_THREADS, 0, s>>>(t);
    }
    if (cudaGetLastError() != cudaSuccess) return OCN_ERR_CUDA;
  }
  return OCN_OK;
}

}  // namespace ocn
