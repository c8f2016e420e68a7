// Common device/host definitions for the PolyFields GB300 engine.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

namespace pf {

// Complex value in working precision T (float or double); 8- or 16-byte aligned so that a
// plane of them moves with vector loads.
template <typename T>
struct alignas(2 * sizeof(T)) Cx {
  T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ Cx<T> cx(T a, T b) {
  Cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename T>
__device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) { return cx<T>(a.x + b.x, a.y + b.y); }
template <typename T>
__device__ __forceinline__ Cx<T> operator-(Cx<T> a, Cx<T> b) { return cx<T>(a.x - b.x, a.y - b.y); }
// float32 complex sums as one packed two-lane instruction (sm_100-family f32x2 arithmetic):
// both lanes round as two scalar additions would.
__device__ __forceinline__ Cx<float> operator+(Cx<float> a, Cx<float> b) {
  const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
  return cx<float>(r.x, r.y);
}
__device__ __forceinline__ Cx<float> operator-(Cx<float> a, Cx<float> b) {
  const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(-b.x, -b.y));
  return cx<float>(r.x, r.y);
}
template <typename T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
  return cx<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ Cx<T> cscale(Cx<T> a, T s) { return cx<T>(a.x * s, a.y * s); }
template <typename T>
__device__ __forceinline__ Cx<T> conj(Cx<T> a) { return cx<T>(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV>
__device__ __forceinline__ Cx<T> mul_mi(Cx<T> a) {
  return INV ? cx<T>(-a.y, a.x) : cx<T>(a.y, -a.x);
}

// Status codes shared with the C-ABI (include/polyfields_gpu.h).
enum Status : int {
  OK = 0,
  E_ARG = 1,
  E_CUDA = 2,
  E_NAN = 3,
  E_SINGULAR = 4,
  E_TIMEOUT = 5,
  E_STATE = 6,
  E_NOMEM = 7,
  E_UNSUPPORTED = 8,
  E_TOOLARGE = 9,
};

// Transform lengths along one axis supported by the in-shared-memory FFTs.
__host__ __device__ inline bool fft_length_supported(int n) {
  switch (n) {
    case 8: case 16: case 32: case 48: case 64: case 96: case 128: case 256:
      return true;
    default:
      return false;
  }
}

// Twiddle table for one transform length N: tw[m] = exp(-2 pi i m / N), m in [0, N).
template <typename T>
struct Twiddles {
  const Cx<T>* x;  // length Nx
  const Cx<T>* y;  // length Ny
  const Cx<T>* z;  // length Nz
};

}  // namespace pf
