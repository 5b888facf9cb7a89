// Float-float ("double-single") arithmetic on the FP32 pipes: a value is a
// pair (hi, lo) of FP32 numbers with hi = fl32(x) and lo = fl32(x - hi), about
// 48 significant bits.  GB300 executes FP64 at 1/58 of its FP32 rate, so the
// FP64-accurate parts of the solver (translations, Arnoldi) use these pairs.
// Round-to-nearest intrinsics throughout, so that the compiler cannot contract
// or reassociate the steps (the error-free transformations depend on them).
#pragma once

#include <cuda_runtime.h>

namespace pibem
{
  // s + c += a * b: the leading product split exactly with an FMA (Dekker's
  // TwoProduct), the cross terms added to its error, the leading sum carried
  // exactly with Knuth's TwoSum; the lo * lo term (2^-48 relative) is dropped.
  // Relative error of a K-term dot product ~ K 2^-47.
  __device__ __forceinline__ void ff_mac(float &s, float &c, float2 a, float2 b)
  {
    const float p = __fmul_rn(a.x, b.x);
    float       e = __fmaf_rn(a.x, b.x, -p);
    e             = __fmaf_rn(a.x, b.y, e);
    e             = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float d = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    c             = __fadd_rn(c, __fadd_rn(d, e));
    s             = t;
  }

  // (hi, lo) of an FP64 value, and back
  __device__ __forceinline__ float2 ff_split(double x)
  {
    const float hi = __double2float_rn(x);
    return make_float2(hi, __double2float_rn(__dsub_rn(x, double(hi))));
  }
  __device__ __forceinline__ double ff_join(float2 v) { return __dadd_rn(double(v.x), double(v.y)); }

  // (h, l) renormalised so that l is below half an ulp of h
  __device__ __forceinline__ float2 ff_norm(float h, float l)
  {
    const float t = __fadd_rn(h, l);
    return make_float2(t, __fsub_rn(l, __fsub_rn(t, h)));
  }

  // a + b: Knuth's TwoSum of the leading parts, the trailing parts added to
  // its error, renormalised
  __device__ __forceinline__ float2 ff_add(float2 a, float2 b)
  {
    const float t = __fadd_rn(a.x, b.x);
    const float z = __fsub_rn(t, a.x);
    const float d = __fadd_rn(__fsub_rn(a.x, __fsub_rn(t, z)), __fsub_rn(b.x, z));
    const float e = __fadd_rn(d, __fadd_rn(a.y, b.y));
    const float h = __fadd_rn(t, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, t)));
  }

  __device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
  __device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return ff_add(a, ff_neg(b)); }

  // a * b: TwoProduct of the leading parts plus the cross terms, renormalised
  __device__ __forceinline__ float2 ff_mul(float2 a, float2 b)
  {
    const float p = __fmul_rn(a.x, b.x);
    float       e = __fmaf_rn(a.x, b.x, -p);
    e             = __fmaf_rn(a.x, b.y, e);
    e             = __fmaf_rn(a.y, b.x, e);
    const float h = __fadd_rn(p, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, p)));
  }

  // 1 / a: the FP32 reciprocal r refined by one Newton step in float-float,
  // r + r (1 - a r)
  __device__ __forceinline__ float2 ff_recip(float2 a)
  {
    const float2 r = make_float2(__frcp_rn(a.x), 0.f);
    const float2 e = ff_sub(make_float2(1.f, 0.f), ff_mul(a, r));
    return ff_add(r, ff_mul(r, e));
  }

  // sqrt(a), a >= 0: the FP32 root s refined by one Newton step,
  // s + (a - s^2) / (2 s) (the correction needs FP32 accuracy only)
  __device__ __forceinline__ float2 ff_sqrt(float2 a)
  {
    if (!(a.x > 0.f))
      return make_float2(0.f, 0.f);
    const float  s = __fsqrt_rn(a.x);
    const float2 t = ff_sub(a, ff_mul(make_float2(s, 0.f), make_float2(s, 0.f)));
    return ff_add(make_float2(s, 0.f), make_float2(__fmul_rn(t.x, __frcp_rn(__fmul_rn(2.f, s))), 0.f));
  }
} // namespace pibem
