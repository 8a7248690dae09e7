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

// Whole k-mesh step for the x-point of this CTA.  phi layout [k][x][a].
// twiddles: tw + ax*OCN_MAX_KDIM.
template <typename R>
__device__ void kmesh_convolve(typename C2<R>::T* __restrict__ phi, const R* __restrict__ W, int nx, int x,
                               const KmeshGeom<R>& g, typename C2<R>::T* buf,
                               const typename C2<R>::T* __restrict__ tw) {
  typedef typename C2<R>::T CT;
  const int tot = g.na * g.nk;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int k = e / g.na, a = e % g.na;
    buf[a * g.slab + kpad(g, k)] = phi[((size_t)k * nx + x) * g.na + a];
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
  const R norm = (R)1 / (R)g.nk;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int k = e / g.na, a = e % g.na;
    const CT v = buf[a * g.slab + kpad(g, k)];
    CT o;
    o.x = v.x * norm;
    o.y = v.y * norm;
    phi[((size_t)k * nx + x) * g.na + a] = o;
  }
}

}  // namespace ocn
