// ocn_kmesh_dft.cuh -- the k <-> R transform of the long-range term
// (long_range.f90:928-939 with FFTW's conventions, Modules/FFT_wrapper.f90:24-25):
//
//   phi'(.,x,a) = FFT_fwd[ W(.,x) o FFT_bwd[ phi(.,x,a) ] ] / Nk
//
// for every x-point, on the k-mesh (n1, n2, n3), flat index k3 fastest.  The
// mesh is tiny (<= a few hundred points), so one CTA holds all Na transforms of
// one x-point in shared memory and every thread owns whole 1-D lines: a line is
// loaded into registers, transformed by a fully unrolled direct DFT (the
// twiddle index (j*m) mod n is a compile-time constant, so every thread of a warp
// reads the same twiddle at the same time), and written back in place.  The
// shared layout pads the fastest axis by one element so that lines along it do
// not collide in shared-memory banks.
#pragma once

#include <cuda_runtime.h>

namespace ocn {

template <typename R>
struct C2;
template <>
struct C2<float> {
  typedef float2 T;
};
template <>
struct C2<double> {
  typedef double2 T;
};

template <typename R>
struct KmeshGeom {
  int n[3];      // k-mesh extents
  int nk;        // n1*n2*n3
  int na;        // transforms per x-point
  int pad3;      // n3 + 1
  int slab;      // padded elements per transform: n1*n2*(n3+1)
};

template <typename R>
inline KmeshGeom<R> kmesh_geom(const int kmesh[3], int na) {
  KmeshGeom<R> g;
  for (int i = 0; i < 3; ++i) g.n[i] = kmesh[i];
  g.nk = kmesh[0] * kmesh[1] * kmesh[2];
  g.na = na;
  g.pad3 = kmesh[2] + 1;
  g.slab = kmesh[0] * kmesh[1] * g.pad3;
  return g;
}

// dynamic shared memory of a kmesh_convolve CTA: twiddles + padded transforms
template <typename R>
inline size_t kmesh_smem(const KmeshGeom<R>& g) {
  return sizeof(typename C2<R>::T) * (3 * OCN_MAX_KDIM + (size_t)g.na * g.slab);
}

template <typename R>
__device__ __forceinline__ int kpad(const KmeshGeom<R>& g, int k) {
  const int k3 = k % g.n[2];
  return (k - k3) / g.n[2] * g.pad3 + k3;
}

// One pass along `ax` for every line, size N known at compile time.
// tw: exp(+2 pi i t / N), t < N; sgn = +1 backward, -1 forward.
template <typename R, int N>
__device__ __forceinline__ void dft_pass_fixed(typename C2<R>::T* buf, const KmeshGeom<R>& g, int ax,
                                               const typename C2<R>::T* __restrict__ tw, R sgn) {
  typedef typename C2<R>::T CT;
  // element stride along the axis in the padded layout
  const int st = (ax == 2) ? 1 : ((ax == 1) ? g.pad3 : g.n[1] * g.pad3);
  // lines: all (a, other two indices)
  const int o1 = (ax == 0) ? g.n[1] : g.n[0];  // first "other" extent (slow)
  const int o2 = (ax == 2) ? g.n[1] : g.n[2];  // second "other" extent (fast)
  const int lines = g.na * o1 * o2;
  CT w[N];
#pragma unroll
  for (int t = 0; t < N; ++t) {
    w[t] = tw[t];
    w[t].y *= sgn;
  }
  for (int l = threadIdx.x; l < lines; l += blockDim.x) {
    const int a = l / (o1 * o2);
    const int r = l % (o1 * o2);
    const int i1 = r / o2, i2 = r % o2;
    int base;
    if (ax == 0) base = i1 * g.pad3 + i2;                       // (k2, k3)
    else if (ax == 1) base = i1 * g.n[1] * g.pad3 + i2;         // (k1, k3)
    else base = (i1 * g.n[1] + i2) * g.pad3;                    // (k1, k2)
    CT* p = buf + a * g.slab + base;
    CT v[N];
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j * st];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      R sr = v[0].x, si = v[0].y;
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const CT ww = w[(j * m) % N];
        sr += v[j].x * ww.x - v[j].y * ww.y;
        si += v[j].x * ww.y + v[j].y * ww.x;
      }
      p[m * st].x = sr;
      p[m * st].y = si;
    }
  }
}

// Fallback for extents without a compiled specialisation (out-of-place via registers
// in chunks is not needed: extents are <= OCN_MAX_KDIM).
template <typename R>
__device__ void dft_pass_generic(typename C2<R>::T* buf, const KmeshGeom<R>& g, int ax,
                                 const typename C2<R>::T* __restrict__ tw, R sgn) {
  typedef typename C2<R>::T CT;
  const int N = g.n[ax];
  const int st = (ax == 2) ? 1 : ((ax == 1) ? g.pad3 : g.n[1] * g.pad3);
  const int o1 = (ax == 0) ? g.n[1] : g.n[0];
  const int o2 = (ax == 2) ? g.n[1] : g.n[2];
  const int lines = g.na * o1 * o2;
  for (int l = threadIdx.x; l < lines; l += blockDim.x) {
    const int a = l / (o1 * o2);
    const int r = l % (o1 * o2);
    const int i1 = r / o2, i2 = r % o2;
    int base;
    if (ax == 0) base = i1 * g.pad3 + i2;
    else if (ax == 1) base = i1 * g.n[1] * g.pad3 + i2;
    else base = (i1 * g.n[1] + i2) * g.pad3;
    CT* p = buf + a * g.slab + base;
    CT v[OCN_MAX_KDIM];
    for (int j = 0; j < N; ++j) v[j] = p[j * st];
    for (int m = 0; m < N; ++m) {
      R sr = 0, si = 0;
      int t = 0;
      for (int j = 0; j < N; ++j) {
        const CT ww = tw[t];
        const R wy = sgn * ww.y;
        sr += v[j].x * ww.x - v[j].y * wy;
        si += v[j].x * wy + v[j].y * ww.x;
        t += m;
        if (t >= N) t -= N;
      }
      p[m * st].x = sr;
      p[m * st].y = si;
    }
  }
}

template <typename R>
__device__ __forceinline__ void dft_pass(typename C2<R>::T* buf, const KmeshGeom<R>& g, int ax,
                                         const typename C2<R>::T* __restrict__ tw, R sgn) {
  switch (g.n[ax]) {
    case 1: return;
    case 2: dft_pass_fixed<R, 2>(buf, g, ax, tw, sgn); return;
    case 3: dft_pass_fixed<R, 3>(buf, g, ax, tw, sgn); return;
    case 4: dft_pass_fixed<R, 4>(buf, g, ax, tw, sgn); return;
    case 5: dft_pass_fixed<R, 5>(buf, g, ax, tw, sgn); return;
    case 6: dft_pass_fixed<R, 6>(buf, g, ax, tw, sgn); return;
    case 7: dft_pass_fixed<R, 7>(buf, g, ax, tw, sgn); return;
    case 8: dft_pass_fixed<R, 8>(buf, g, ax, tw, sgn); return;
    case 10: dft_pass_fixed<R, 10>(buf, g, ax, tw, sgn); return;
    case 12: dft_pass_fixed<R, 12>(buf, g, ax, tw, sgn); return;
    case 16: dft_pass_fixed<R, 16>(buf, g, ax, tw, sgn); return;
    default: dft_pass_generic<R>(buf, g, ax, tw, sgn); return;
  }
}

// --------------------------------------------------------------------------
// Compile-time specialisation for cubic meshes n^3 and NA transforms per x:
// every index computation folds to shifts and multiplies, and 2/4/8-point lines
// use radix-2 butterflies (sgn = +1 backward, -1 forward).

template <typename CT, typename R>
__device__ __forceinline__ CT cadd(CT a, CT b) {
  CT r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename CT, typename R>
__device__ __forceinline__ CT csub(CT a, CT b) {
  CT r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
// (sgn * i) * z
template <typename CT, typename R>
__device__ __forceinline__ CT cmul_si(CT z, R sgn) {
  CT r;
  r.x = -sgn * z.y;
  r.y = sgn * z.x;
  return r;
}

template <typename CT, typename R, int N>
__device__ __forceinline__ void line_dft(CT (&v)[N], const CT* __restrict__ tw, R sgn) {
  if constexpr (N == 2) {
    const CT a = v[0], b = v[1];
    v[0] = cadd<CT, R>(a, b);
    v[1] = csub<CT, R>(a, b);
  } else if constexpr (N == 4) {
    const CT s02 = cadd<CT, R>(v[0], v[2]), d02 = csub<CT, R>(v[0], v[2]);
    const CT s13 = cadd<CT, R>(v[1], v[3]), d13 = cmul_si<CT, R>(csub<CT, R>(v[1], v[3]), sgn);
    v[0] = cadd<CT, R>(s02, s13);
    v[2] = csub<CT, R>(s02, s13);
    v[1] = cadd<CT, R>(d02, d13);
    v[3] = csub<CT, R>(d02, d13);
  } else if constexpr (N == 8) {
    CT e[4] = {v[0], v[2], v[4], v[6]};
    CT o[4] = {v[1], v[3], v[5], v[7]};
    line_dft<CT, R, 4>(e, tw, sgn);
    line_dft<CT, R, 4>(o, tw, sgn);
    const R h = (R)0.70710678118654752440;  // cos(pi/4)
    // w^m = exp(sgn i pi m / 4), m = 1..3
    CT t1, t2, t3;
    t1.x = h * (o[1].x - sgn * o[1].y);
    t1.y = h * (o[1].y + sgn * o[1].x);
    t2 = cmul_si<CT, R>(o[2], sgn);
    t3.x = -h * (o[3].x + sgn * o[3].y);
    t3.y = h * (sgn * o[3].x - o[3].y);
    v[0] = cadd<CT, R>(e[0], o[0]);
    v[4] = csub<CT, R>(e[0], o[0]);
    v[1] = cadd<CT, R>(e[1], t1);
    v[5] = csub<CT, R>(e[1], t1);
    v[2] = cadd<CT, R>(e[2], t2);
    v[6] = csub<CT, R>(e[2], t2);
    v[3] = cadd<CT, R>(e[3], t3);
    v[7] = csub<CT, R>(e[3], t3);
  } else {
    CT w[N];
#pragma unroll
    for (int t = 0; t < N; ++t) {
      w[t] = tw[t];
      w[t].y *= sgn;
    }
    CT out[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      R sr = v[0].x, si = v[0].y;
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const CT ww = w[(j * m) % N];
        sr += v[j].x * ww.x - v[j].y * ww.y;
        si += v[j].x * ww.y + v[j].y * ww.x;
      }
      out[m].x = sr;
      out[m].y = si;
    }
#pragma unroll
    for (int m = 0; m < N; ++m) v[m] = out[m];
  }
}

// Elements per alpha plane of a cubic transform: n*n*(n+1), padded so that
// consecutive alpha planes start 8 banks apart (float2: 2 words per element,
// double2: 4 words) -- four alpha values of one k-point then never share a bank.
template <typename CT>
__host__ __device__ constexpr int cube_slab(int n) {
  return ((n * n * (n + 1) + 15) / 16) * 16 + (sizeof(CT) == 8 ? 4 : 2);
}

// NTC: the transform count when it is known at compile time (0: runtime nt).
template <typename R, int N, int NTC>
__device__ __forceinline__ void cube_pass(typename C2<R>::T* buf, int nt_rt, int ax,
                                          const typename C2<R>::T* __restrict__ tw, R sgn) {
  typedef typename C2<R>::T CT;
  constexpr int P3 = N + 1;
  constexpr int SLAB = cube_slab<CT>(N);
  const int nt = NTC ? NTC : nt_rt;
  const int lines = nt * N * N;
  const int st = (ax == 2) ? 1 : ((ax == 1) ? P3 : N * P3);
  for (int l = threadIdx.x; l < lines; l += blockDim.x) {
    const int a = l / (N * N);
    const int r = l % (N * N);
    const int i1 = r / N, i2 = r % N;
    int base;
    if (ax == 0) base = i1 * P3 + i2;
    else if (ax == 1) base = i1 * N * P3 + i2;
    else base = (i1 * N + i2) * P3;
    CT* p = buf + a * SLAB + base;
    CT v[N];
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j * st];
    line_dft<CT, R, N>(v, tw, sgn);
#pragma unroll
    for (int j = 0; j < N; ++j) p[j * st] = v[j];
  }
}

// nt transforms of the x-point (alpha, or (vector, alpha) for a block of psi):
// transform t of k-point k at phi[(k*nx + x)*ld + t], ld >= nt (a CTA may own a
// slice of the transforms of its x-point).  Leaves Nk * phi'(k) of transform t
// in buf[t*SLAB + (k/N)*(N+1) + k%N] (not yet divided by Nk); ends with a barrier.
template <typename R, int N, int NTC>
__device__ void kmesh_cube_transform(const typename C2<R>::T* __restrict__ phi, const R* __restrict__ W, int nx,
                                     int x, int nt_rt, int ld, typename C2<R>::T* buf,
                                     const typename C2<R>::T* __restrict__ tw) {
  typedef typename C2<R>::T CT;
  const int nt = NTC ? NTC : nt_rt;
  constexpr int NK = N * N * N;
  constexpr int P3 = N + 1;
  constexpr int SLAB = cube_slab<CT>(N);
  // t fastest across threads: a warp reads whole 32-byte sectors of phi, and the
  // padded slab puts neighbouring transforms on different shared-memory banks.
  // A compile-time count keeps a plain unrollable loop (several loads in
  // flight); a runtime count advances (k, t) incrementally instead of dividing.
  const int dt = blockDim.x % nt, dk = blockDim.x / nt;
  if constexpr (NTC > 0) {
    for (int e = threadIdx.x; e < NTC * NK; e += blockDim.x) {
      const int k = e / NTC, t = e % NTC;
      buf[t * SLAB + (k / N) * P3 + k % N] = phi[((size_t)k * nx + x) * ld + t];
    }
  } else {
    int t = threadIdx.x % nt, k = threadIdx.x / nt;
    while (k < NK) {
      buf[t * SLAB + (k / N) * P3 + k % N] = phi[((size_t)k * nx + x) * ld + t];
      t += dt;
      k += dk;
      if (t >= nt) {
        t -= nt;
        ++k;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    cube_pass<R, N, NTC>(buf, nt, ax, tw + ax * OCN_MAX_KDIM, (R)1);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nt * NK; e += blockDim.x) {
    const int a = e / NK, k = e % NK;
    const R wv = W[(size_t)x * NK + k];
    CT& v = buf[a * SLAB + (k / N) * P3 + k % N];
    v.x *= wv;
    v.y *= wv;
  }
  __syncthreads();
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    cube_pass<R, N, NTC>(buf, nt, ax, tw + ax * OCN_MAX_KDIM, (R)-1);
    __syncthreads();
  }
}

// The transformed planes of kmesh_cube_transform, divided by Nk, back into phi.
template <typename R, int N, int NTC>
__device__ void kmesh_cube_store(typename C2<R>::T* __restrict__ phi, int nx, int x, int nt_rt, int ld,
                                 const typename C2<R>::T* buf) {
  typedef typename C2<R>::T CT;
  const int nt = NTC ? NTC : nt_rt;
  constexpr int NK = N * N * N;
  constexpr int P3 = N + 1;
  constexpr int SLAB = cube_slab<CT>(N);
  const int dt = blockDim.x % nt, dk = blockDim.x / nt;
  const R norm = (R)1 / (R)NK;
  if constexpr (NTC > 0) {
    for (int e = threadIdx.x; e < NTC * NK; e += blockDim.x) {
      const int k = e / NTC, t = e % NTC;
      const CT v = buf[t * SLAB + (k / N) * P3 + k % N];
      CT o;
      o.x = v.x * norm;
      o.y = v.y * norm;
      phi[((size_t)k * nx + x) * ld + t] = o;
    }
  } else {
    int t = threadIdx.x % nt, k = threadIdx.x / nt;
    while (k < NK) {
      const CT v = buf[t * SLAB + (k / N) * P3 + k % N];
      CT o;
      o.x = v.x * norm;
      o.y = v.y * norm;
      phi[((size_t)k * nx + x) * ld + t] = o;
      t += dt;
      k += dk;
      if (t >= nt) {
        t -= nt;
        ++k;
      }
    }
  }
}

template <typename R, int N, int NTC>
__device__ void kmesh_convolve_cube(typename C2<R>::T* __restrict__ phi, const R* __restrict__ W, int nx,
                                    int x, int nt_rt, int ld, typename C2<R>::T* buf,
                                    const typename C2<R>::T* __restrict__ tw) {
  kmesh_cube_transform<R, N, NTC>(phi, W, nx, x, nt_rt, ld, buf, tw);
  kmesh_cube_store<R, N, NTC>(phi, nx, x, nt_rt, ld, buf);
}

// dL/dW of the long-range term for the x-point of this CTA, from the band-to-x
// results of a solution pair (phx: x, phy: the adjoint y; layout [k][x][t]):
// both are transformed back over the k-mesh (the F_b half of the convolution),
// then gW[x*NK + R] += ca Re(D) + cb Im(D) with D = -(1/NK) sum_t conj(Y_t) X_t.
template <typename R, int N>
__device__ void kmesh_wgrad_cube(const typename C2<R>::T* __restrict__ phx, const typename C2<R>::T* __restrict__ phy,
                                 int nx, int x, int nt, typename C2<R>::T* buf,
                                 const typename C2<R>::T* __restrict__ tw, double* __restrict__ gW, double ca,
                                 double cb) {
  typedef typename C2<R>::T CT;
  constexpr int NK = N * N * N;
  constexpr int P3 = N + 1;
  constexpr int SLAB = cube_slab<CT>(N);
  for (int e = threadIdx.x; e < 2 * nt * NK; e += blockDim.x) {
    const int half = e / (nt * NK);
    const int r = e % (nt * NK);
    const int k = r / nt, t = r % nt;
    const CT* src = half ? phy : phx;
    buf[(half * nt + t) * SLAB + (k / N) * P3 + k % N] = src[((size_t)k * nx + x) * nt + t];
  }
  __syncthreads();
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    cube_pass<R, N, 0>(buf, 2 * nt, ax, tw + ax * OCN_MAX_KDIM, (R)1);
    __syncthreads();
  }
  for (int k = threadIdx.x; k < NK; k += blockDim.x) {
    double sr = 0.0, si = 0.0;
    const int o = (k / N) * P3 + k % N;
    for (int t = 0; t < nt; ++t) {
      const CT X = buf[t * SLAB + o];
      const CT Y = buf[(nt + t) * SLAB + o];
      sr += (double)Y.x * (double)X.x + (double)Y.y * (double)X.y;
      si += (double)Y.x * (double)X.y - (double)Y.y * (double)X.x;
    }
    const double inv = -1.0 / (double)NK;
    gW[(size_t)x * NK + k] += ca * (sr * inv) + cb * (si * inv);
  }
}

// dynamic shared memory of a kmesh_convolve_cube CTA: twiddles + padded planes
template <typename R>
inline size_t kmesh_cube_smem(int n, int nt) {
  typedef typename C2<R>::T CT;
  return sizeof(CT) * (3 * OCN_MAX_KDIM + (size_t)nt * cube_slab<CT>(n));
}

// A cubic specialisation exists for these extents.
inline bool kmesh_cube_supported(const int kmesh[3]) {
  if (kmesh[0] != kmesh[1] || kmesh[1] != kmesh[2]) return false;
  const int n = kmesh[0];
  return n == 2 || n == 3 || n == 4 || n == 5 || n == 6 || n == 8;
}

// Selects the instantiation kern<N, NTC> of a kernel template for a supported
// cubic mesh (kmesh_cube_supported) and nt transforms per x-point: NTC = nt for
// the common counts 4 (1s edge) and 12 (2p edge, or three 1s vectors), where
// the index arithmetic folds at compile time, else 0 (runtime nt).  nullptr if
// the mesh is not supported.
#define OCN_CUBE_NT(KERN, N, nt) (((nt) == 4) ? KERN<N, 4> : ((nt) == 12) ? KERN<N, 12> : KERN<N, 0>)
#define OCN_CUBE_DISPATCH(KERN, n, nt, out)          \
  do {                                               \
    out = nullptr;                                   \
    switch (n) {                                     \
      case 2: out = OCN_CUBE_NT(KERN, 2, nt); break; \
      case 3: out = OCN_CUBE_NT(KERN, 3, nt); break; \
      case 4: out = OCN_CUBE_NT(KERN, 4, nt); break; \
      case 5: out = OCN_CUBE_NT(KERN, 5, nt); break; \
      case 6: out = OCN_CUBE_NT(KERN, 6, nt); break; \
      case 8: out = OCN_CUBE_NT(KERN, 8, nt); break; \
    }                                                \
  } while (0)

// Whole k-mesh step for the x-point of this CTA.  phi layout [k][x][a].
// twiddles: tw + ax*OCN_MAX_KDIM.  kmesh_transform leaves Nk * phi'(k) of
// transform a in buf[a*g.slab + kpad(g, k)] and ends with a barrier.
template <typename R>
__device__ void kmesh_transform(const typename C2<R>::T* __restrict__ phi, const R* __restrict__ W, int nx, int x,
                                const KmeshGeom<R>& g, typename C2<R>::T* buf,
                                const typename C2<R>::T* __restrict__ tw) {
  typedef typename C2<R>::T CT;
  const int tot = g.na * g.nk;
  for (int k = threadIdx.x; k < g.nk; k += blockDim.x) {
    const CT* src = phi + ((size_t)k * nx + x) * g.na;
    const int pos = kpad(g, k);
    for (int a = 0; a < g.na; ++a) buf[a * g.slab + pos] = src[a];
  }
  __syncthreads();
  for (int ax = 0; ax < 3; ++ax) {
    dft_pass<R>(buf, g, ax, tw + ax * OCN_MAX_KDIM, (R)1);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int a = e / g.nk, k = e % g.nk;
    const R wv = W[(size_t)x * g.nk + k];
    CT& v = buf[a * g.slab + kpad(g, k)];
    v.x *= wv;
    v.y *= wv;
  }
  __syncthreads();
  for (int ax = 0; ax < 3; ++ax) {
    dft_pass<R>(buf, g, ax, tw + ax * OCN_MAX_KDIM, (R)-1);
    __syncthreads();
  }
}

template <typename R>
__device__ void kmesh_convolve(typename C2<R>::T* __restrict__ phi, const R* __restrict__ W, int nx, int x,
                               const KmeshGeom<R>& g, typename C2<R>::T* buf,
                               const typename C2<R>::T* __restrict__ tw) {
  typedef typename C2<R>::T CT;
  kmesh_transform<R>(phi, W, nx, x, g, buf, tw);
  const R norm = (R)1 / (R)g.nk;
  for (int k = threadIdx.x; k < g.nk; k += blockDim.x) {
    CT* dst = phi + ((size_t)k * nx + x) * g.na;
    const int pos = kpad(g, k);
    for (int a = 0; a < g.na; ++a) {
      const CT v = buf[a * g.slab + pos];
      CT o;
      o.x = v.x * norm;
      o.y = v.y * norm;
      dst[a] = o;
    }
  }
}

}  // namespace ocn
