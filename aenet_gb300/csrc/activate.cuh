// Activation functions of the per-species networks and their derivatives
// (ff_activate, src/ext/feedforward.f90:932-969): 0 linear, 1 tanh,
// 2 sigmoid, 3 scaled tanh 1.7159 tanh(2x/3), 4 twisted tanh
// (scaled tanh + 0.1 x).
#pragma once

static __device__ __forceinline__ float tanh_t(float x) { return tanhf(x); }
static __device__ __forceinline__ double tanh_t(double x) { return tanh(x); }
static __device__ __forceinline__ float exp_t(float x) { return expf(x); }
static __device__ __forceinline__ double exp_t(double x) { return exp(x); }

template <typename T>
__device__ __forceinline__ void activate(int t, T x, T& y, T& dy) {
  const T a = T(1.7159), b = T(0.666666666666667), c = T(0.1);
  switch (t) {
    case 0: y = x; dy = T(1); break;
    case 1: y = tanh_t(x); dy = T(1) - y * y; break;
    case 2: y = T(1) / (T(1) + exp_t(-x)); dy = y * (T(1) - y); break;
    case 3: { T tb = tanh_t(b * x); y = a * tb; dy = a * (T(1) - tb * tb) * b; } break;
    case 4: { T tb = tanh_t(b * x); y = a * tb + c * x; dy = a * (T(1) - tb * tb) * b + c; } break;
    default: y = T(0); dy = T(0);
  }
}
