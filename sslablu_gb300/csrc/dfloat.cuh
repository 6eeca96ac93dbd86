// Double-float numbers: x = h + l with two float32s (|l| <= ulp(h) / 2), about
// 48 significant bits, with arithmetic on the float32 units built from
// error-free transformations (Dekker's product via one fused multiply-add,
// Knuth's TwoSum; the published double-double algorithms, here on float32
// pairs).  Used as the element type of the ULV solve bodies, so that the
// mixed-precision path solves on the float32 pipe -- about 5x the float64
// throughput on GB300 -- to ~1e-14 relative accuracy, instead of iterating
// from a float32 solve.
#pragma once

namespace slu {

struct __align__(8) dfloat {
  float h, l;
  dfloat() = default;
  __host__ __device__ constexpr dfloat(float v) : h(v), l(0.f) {}
  __host__ __device__ constexpr dfloat(int v) : h(static_cast<float>(v)), l(0.f) {}
  __host__ __device__ constexpr dfloat(float hi, float lo) : h(hi), l(lo) {}
  // no implicit narrowing from double (use to_dfloat): a double argument
  // must never reach a dfloat overload by conversion
  dfloat(double) = delete;
};
static_assert(sizeof(dfloat) == 8, "dfloat is a pair of float32");

// The float/double overloads stay visible next to the dfloat ones declared in
// this namespace (otherwise unqualified calls from slu code would find only
// the dfloat forms).
using ::fma;
using ::__shfl_sync;
using ::__shfl_xor_sync;
using ::__ldg;
using ::__ldcg;

namespace dfops {
// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly, |a| >= |b|
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
}  // namespace dfops

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  float s, e;
  dfops::two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  float h, l;
  dfops::fast_two_sum(s, e, h, l);
  return dfloat(h, l);
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.h, -a.l); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);                       // exact product error
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));          // cross terms
  float h, l;
  dfops::fast_two_sum(p, e, h, l);
  return dfloat(h, l);
}
// c + a b with one renormalisation
__device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
  const float p = __fmul_rn(a.h, b.h);
  float pe = __fmaf_rn(a.h, b.h, -p);
  pe = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, pe));
  float s, e;
  dfops::two_sum(c.h, p, s, e);
  e = __fadd_rn(e, __fadd_rn(c.l, pe));
  float h, l;
  dfops::fast_two_sum(s, e, h, l);
  return dfloat(h, l);
}
// a / b: a float32 quotient, corrected once by the double-float remainder
__device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) {
  const float q0 = __fdiv_rn(a.h, b.h);
  const dfloat r = a - b * dfloat(q0);
  const float q1 = __fdiv_rn(r.h, b.h);
  float h, l;
  dfops::fast_two_sum(q0, q1, h, l);
  return dfloat(h, l);
}
__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }
__device__ __forceinline__ dfloat& operator/=(dfloat& a, dfloat b) { return a = a / b; }

__device__ __forceinline__ dfloat __shfl_sync(unsigned mask, dfloat v, int src) {
  return dfloat(::__shfl_sync(mask, v.h, src), ::__shfl_sync(mask, v.l, src));
}
__device__ __forceinline__ dfloat __shfl_xor_sync(unsigned mask, dfloat v, int m) {
  return dfloat(::__shfl_xor_sync(mask, v.h, m), ::__shfl_xor_sync(mask, v.l, m));
}
__device__ __forceinline__ dfloat __ldg(const dfloat* p) {
  const float2 v = ::__ldg(reinterpret_cast<const float2*>(p));
  return dfloat(v.x, v.y);
}
__device__ __forceinline__ dfloat __ldcg(const dfloat* p) {
  const float2 v = ::__ldcg(reinterpret_cast<const float2*>(p));
  return dfloat(v.x, v.y);
}

// Dot-product accumulators.  For float and double the accumulator is the
// value itself.  For double-float, the sum is kept unnormalised (Ogita, Rump
// and Oishi's Dot2 scheme, with the cross terms of double-float inputs): the
// exact product's high part goes through TwoSum into h, every error term
// into l, and one renormalisation at the end gives the double-float result
// -- 12 float32 operations per term instead of 15.
template <typename T>
struct DotAcc {
  T v;
  __device__ __forceinline__ void zero() { v = T(0); }
  __device__ __forceinline__ void add(T a, T b) { v = fma(a, b, v); }
  __device__ __forceinline__ T value() const { return v; }
};
template <>
struct DotAcc<dfloat> {
  float h, l;
  __device__ __forceinline__ void zero() { h = l = 0.f; }
  __device__ __forceinline__ void add(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.h, b.h);
    float pe = __fmaf_rn(a.h, b.h, -p);
    pe = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, pe));
    float s, e;
    dfops::two_sum(h, p, s, e);
    h = s;
    l = __fadd_rn(l, __fadd_rn(e, pe));
  }
  // TwoSum, not the fast form: after cancellation |l| may exceed |h|
  __device__ __forceinline__ dfloat value() const {
    float hh, ll;
    dfops::two_sum(h, l, hh, ll);
    return dfloat(hh, ll);
  }
};

__device__ __forceinline__ dfloat to_dfloat(double x) {
  const float h = __double2float_rn(x);
  return dfloat(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double to_double(dfloat x) { return (double)x.h + (double)x.l; }

}  // namespace slu
