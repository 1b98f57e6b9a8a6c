// ff.cuh -- float-float ("double-single") arithmetic for the FP64-accurate
// sigma on GB300, whose FP64 units run at a small fraction of the FP32 rate.
//
// A value is the unevaluated sum h + l of two floats.  Products use the exact
// product error of an FMA (p = a*b, e = fma(a, b, -p) gives a*b = p + e
// exactly), sums use Knuth's branch-free two-sum (s = a + b, z = s - a,
// err = (a - (s - z)) + (b - z) gives a + b = s + err exactly); the low
// parts are carried in plain float arithmetic without renormalisation, which
// keeps about 48 significant bits (Dekker, "A floating-point technique for
// extending the available precision", 1971; Knuth, TAOCP vol. 2, 4.2.2).
// The sigma accumulates 2(L-N)N + 1 such terms per determinant, so its
// relative error stays near 1e-14, well inside the 1e-12 sigma tolerance.
#pragma once

#include <cuda_runtime.h>

namespace doci {

struct __align__(8) ff {
  float h, l;
  ff() = default;
  __host__ __device__ constexpr ff(int z) : h(static_cast<float>(z)), l(0.f) {}
  __host__ __device__ constexpr ff(float a, float b) : h(a), l(b) {}
};

__device__ __forceinline__ ff ff_from(double v) {
  const float h = __double2float_rn(v);
  return ff(h, __double2float_rn(v - static_cast<double>(h)));
}
__device__ __forceinline__ double ff_to(ff a) { return static_cast<double>(a.h) + static_cast<double>(a.l); }

__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return ff(p, e);
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const float s = a.h + b.h;
  const float z = s - a.h;
  const float err = (a.h - (s - z)) + (b.h - z);
  return ff(s, a.l + b.l + err);
}
__device__ __forceinline__ ff &operator+=(ff &a, ff b) {
  a = a + b;
  return a;
}

// Storage type of the tables, the diagonal and the output of a kernel that
// computes in Real: the same type, except float-float, which reads and
// writes double (x alone is staged as float-float, converted once per call).
template <typename Real>
struct Io {
  using T = Real;
  __device__ __forceinline__ static Real in(T v) { return v; }
  __device__ __forceinline__ static T out(Real v) { return v; }
};
template <>
struct Io<ff> {
  using T = double;
  __device__ __forceinline__ static ff in(double v) { return ff_from(v); }
  __device__ __forceinline__ static double out(ff v) { return ff_to(v); }
};

template <typename Real>
__device__ __forceinline__ Real ldg_val(const Real *p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ ff ldg_val<ff>(const ff *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return ff(v.x, v.y);
}

}  // namespace doci
