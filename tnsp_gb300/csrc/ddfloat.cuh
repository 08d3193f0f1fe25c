// Double-float arithmetic: a value is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// about 46 bits of precision carried on the FP32 pipe, which GB300 runs at 64 times the FP64 rate.
//
// The operations are built from the error-free transformations of Knuth (two-sum) and Dekker
// (two-product, here with a fused multiply-add) followed by a renormalisation (fast two-sum); see
// T. J. Dekker, "A floating-point technique for extending the available precision", Numer. Math. 18
// (1971) 224-242, and D. E. Knuth, TAOCP vol. 2, 4.2.2.  Addition is the accurate variant (two-sum on
// both components); the multiply-add and the two-term linear combination two-sum the high parts and
// renormalise once.  Division and square root take one Newton correction of the float approximation.  The exponent range is that of float: the sampler keeps every tensor
// normalised to O(1) and carries magnitudes in separate integer exponents.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace tnsp {
// The type and its functions live in a nested namespace: argument-dependent lookup finds them for dd
// operands, while unqualified calls on double or float inside tnsp keep resolving to the CUDA math
// functions (an overload declared in tnsp itself would hide them).
namespace ddf {

struct __align__(8) dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ dd(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ constexpr dd(float x) : hi(x), lo(0.f) {}
  __host__ __device__ constexpr dd(int x) : hi((float)x), lo(0.f) {}  // exact for |x| < 2^24
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return dd(s, e);
}
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {  // requires |a| >= |b| (or a == 0)
  const float s = a + b;
  return dd(s, b - (s - a));
}

__device__ __forceinline__ dd operator+(dd x, dd y) {
  dd s = dd_two_sum(x.hi, y.hi);
  const dd t = dd_two_sum(x.lo, y.lo);
  s.lo += t.hi;
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd operator-(dd x) { return dd(-x.hi, -x.lo); }
__device__ __forceinline__ dd operator-(dd x, dd y) { return x + (-y); }
__device__ __forceinline__ dd operator*(dd x, dd y) {
  const float p = x.hi * y.hi;
  const float e = fmaf(x.hi, y.hi, -p);
  return dd_fast_two_sum(p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e)));
}
__device__ __forceinline__ dd operator/(dd x, dd y) {
  const float q1 = x.hi / y.hi;
  const dd r = x - y * dd(q1);
  const float q2 = r.hi / y.hi;
  return dd_fast_two_sum(q1, q2);
}
__device__ __forceinline__ dd& operator+=(dd& x, dd y) { return x = x + y; }
__device__ __forceinline__ dd& operator-=(dd& x, dd y) { return x = x - y; }
__device__ __forceinline__ dd& operator*=(dd& x, dd y) { return x = x * y; }

// a * b + c: exact product of the high parts (p, its rounding error in the cross terms), two-sum with
// c's high part, one renormalisation: 15 FP32 instructions.  Its error is bounded relative to the
// operands (|a b| + |c|), as a float64 dot product's is relative to the sum of |terms|.
__device__ __forceinline__ dd fma(dd a, dd b, dd c) {
  const float p = a.hi * b.hi;
  const float pe = fmaf(a.hi, b.hi, -p);
  const float cross = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, pe));
  const dd s = dd_two_sum(c.hi, p);
  return dd_fast_two_sum(s.hi, s.lo + (c.lo + cross));
}

// a * x + b * y with one two-sum of the high products and one renormalisation (19 FP32 instructions
// against 34 for two products and an addition): the Jacobi rotations
__device__ __forceinline__ dd dd_lincomb(dd a, dd x, dd b, dd y) {
  const float p1 = a.hi * x.hi;
  const float e1 = fmaf(a.hi, x.hi, -p1);
  const float p2 = b.hi * y.hi;
  const float e2 = fmaf(b.hi, y.hi, -p2);
  const dd h = dd_two_sum(p1, p2);
  float t = fmaf(a.hi, x.lo, e1);
  t = fmaf(a.lo, x.hi, t);
  t = fmaf(b.hi, y.lo, t);
  t = fmaf(b.lo, y.hi, t);
  return dd_fast_two_sum(h.hi, h.lo + (t + e2));
}

__device__ __forceinline__ bool operator<(dd x, dd y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
__device__ __forceinline__ bool operator>(dd x, dd y) { return y < x; }
__device__ __forceinline__ bool operator<=(dd x, dd y) { return !(y < x); }
__device__ __forceinline__ bool operator>=(dd x, dd y) { return !(x < y); }
__device__ __forceinline__ bool operator==(dd x, dd y) { return x.hi == y.hi && x.lo == y.lo; }
__device__ __forceinline__ bool operator!=(dd x, dd y) { return !(x == y); }

__device__ __forceinline__ dd fabs(dd x) { return x.hi < 0.f ? -x : x; }
__device__ __forceinline__ dd fmax(dd x, dd y) { return x < y ? y : x; }
__device__ __forceinline__ bool isfinite(dd x) { return ::isfinite(x.hi) && ::isfinite(x.lo); }
__device__ __forceinline__ dd sqrt(dd x) {
  if (!(x.hi > 0.f)) return dd(0.f, 0.f);
  const float s = sqrtf(x.hi);
  const float p = s * s;
  const float pe = fmaf(s, s, -p);
  const float corr = ((x.hi - p) - pe + x.lo) / (2.f * s);
  return dd_fast_two_sum(s, corr);
}

__device__ __forceinline__ dd shfl_xor(dd v, int o) {
  return dd(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}

}  // namespace ddf
using ddf::dd;
}  // namespace tnsp
