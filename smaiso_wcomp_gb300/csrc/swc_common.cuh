// swc_common.cuh -- shared definitions of the sm_103a kernels of libswc.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

namespace swc {

template <typename T> struct Cx;
template <> struct Cx<double> { using type = double2; };
template <> struct Cx<float> { using type = float2; };
template <typename T> using cx_t = typename Cx<T>::type;

template <typename C> __device__ __forceinline__ C cmake(decltype(C::x) a, decltype(C::x) b) {
  C r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  return cmake<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __device__ __forceinline__ C cswap(C a) { return cmake<C>(a.y, a.x); }

// Geometry of an nx x ny x nz array (all powers of two), index = (i*ny + j)*nz + k.
struct Grid {
  int nx, ny, nz;
  int lx, ly, lz;  // log2 of the extents
  long long ng;
};

// Grid of power-of-two extents (validated by the caller).
inline Grid make_grid(int nx, int ny, int nz) {
  Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.lx = __builtin_ctz((unsigned)nx); g.ly = __builtin_ctz((unsigned)ny); g.lz = __builtin_ctz((unsigned)nz);
  g.ng = (long long)nx * ny * nz;
  return g;
}

// Per-axis wavenumber tables in the work precision T, exactly as the reference builds
// them (smaiso-wcomp.cpp:445-481): Vq[i] = pi i/(d n), Vs[i] = pi (i+1)/(d n).
template <typename T> struct Wavenumbers {
  const T* vq[3];
  const T* vs[3];
};

}  // namespace swc
