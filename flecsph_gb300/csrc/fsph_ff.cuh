// fsph_ff.cuh -- float-float ("double-float") arithmetic for the neighbour
// sums of the mixed-precision path whose terms cancel.
//
// A value is the unevaluated sum h + l of two floats.  On a lattice, or in
// any region of uniform pressure, the pressure-gradient terms of a
// particle's neighbours cancel to a small fraction of any one term (KH
// bulk: ~1e-4 of sum |term|), so plain FP32 per-pair rounding (~6e-8 of each
// term) leaves a relative acceleration error of ~1e-3.  The density feeds
// P/rho^2 of every neighbour into the same sum, so it needs the same care.
// These helpers carry ~44 bits through the pair geometry, the kernel
// polynomial and the sum, for ~3x the FP32 instruction count of a pair.
//
// The error-free transformations (two-sum, exact product error by FMA)
// follow Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2); the "lazy" variants
// below do not renormalise after each operation (the low word may exceed
// half an ulp of the high word by a few ulps), which costs nothing in
// accuracy at this depth and saves three instructions per operation.
// Every product and sum of an error-free transformation is written with
// the _rn intrinsics, which the compiler never contracts into an FMA: a
// contracted s = a*b + c would no longer be the rounded sum the two-sum's
// error term assumes.
#pragma once
#include <cuda_runtime.h>

namespace fsph {

struct ffloat {
  float h, l;
};

__device__ __forceinline__ ffloat ff_make(float h, float l) {
  ffloat r;
  r.h = h;
  r.l = l;
  return r;
}

// a + b, any magnitudes (Knuth's two-sum on the high words)
__device__ __forceinline__ ffloat ff_add(ffloat a, ffloat b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  return ff_make(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}

// a + b with |a.h| >= |b.h| (Dekker's fast two-sum)
__device__ __forceinline__ ffloat ff_add_big(ffloat a, ffloat b) {
  const float s = __fadd_rn(a.h, b.h);
  const float e = __fsub_rn(b.h, __fsub_rn(s, a.h));
  return ff_make(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}

// c + b for a float constant c with |c| >= |b.h|
__device__ __forceinline__ ffloat ff_cadd(float c, ffloat b) {
  const float s = __fadd_rn(c, b.h);
  const float e = __fsub_rn(b.h, __fsub_rn(s, c));
  return ff_make(s, __fadd_rn(e, b.l));
}

// a + b for a float b, any magnitudes
__device__ __forceinline__ ffloat ff_add_f(ffloat a, float b) {
  const float s = __fadd_rn(a.h, b);
  const float bb = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff_make(s, __fadd_rn(e, a.l));
}

// renormalise: |l| <= ulp(h) / 2 afterwards
__device__ __forceinline__ ffloat ff_norm(ffloat a) {
  const float s = __fadd_rn(a.h, a.l);
  return ff_make(s, __fsub_rn(a.l, __fsub_rn(s, a.h)));
}

// a * b (the l*l term, ~2^-48 relative, is dropped)
__device__ __forceinline__ ffloat ff_mul(ffloat a, ffloat b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return ff_make(p, e);
}

// a * b for a float b
__device__ __forceinline__ ffloat ff_mul_f(ffloat a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return ff_make(p, e);
}

// a * c for a power of two c: exact, word by word
__device__ __forceinline__ ffloat ff_scale2(ffloat a, float c) {
  return ff_make(__fmul_rn(a.h, c), __fmul_rn(a.l, c));
}

__device__ __forceinline__ ffloat ff_sqr(ffloat a) {
  const float p = __fmul_rn(a.h, a.h);
  float e = __fmaf_rn(a.h, a.h, -p);
  e = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e);
  return ff_make(p, e);
}

// a^2 keeping l*l: for a position difference, whose low word (the
// difference of two residuals) is far above half an ulp of the high word
__device__ __forceinline__ ffloat ff_sqr_wide(ffloat a) {
  const float p = __fmul_rn(a.h, a.h);
  float e = __fmaf_rn(a.h, a.h, -p);
  e = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e);
  e = __fmaf_rn(a.l, a.l, e);
  return ff_make(p, e);
}

// sqrt(a) for a normalised a >= 0: one Newton correction of the FP32 root,
// from the exact residual a - r^2 (an approximate rsqrt is enough)
__device__ __forceinline__ ffloat ff_sqrt(ffloat a) {
  const float rs = a.h > 0.f ? rsqrtf(a.h) : 0.f;
  const float r = __fmul_rn(a.h, rs);
  const float d = __fadd_rn(__fmaf_rn(-r, r, a.h), a.l);
  return ff_make(r, __fmul_rn(d, __fmul_rn(0.5f, rs)));
}

// c / a for a float constant c (c = 1 or 2 here; exact scaling): one
// Newton correction of an approximate reciprocal from the exact residual
__device__ __forceinline__ ffloat ff_rcp_scaled(ffloat a, float c) {
  const float r = 1.0f / a.h;
  float e = __fmaf_rn(-a.h, r, 1.0f);
  e = __fmaf_rn(-a.l, r, e);
  return ff_make(__fmul_rn(c, r), __fmul_rn(c, __fmul_rn(e, r)));
}

// running sum: s += t, the error of the high-word sum kept in the low word
__device__ __forceinline__ void ff_acc(ffloat & s, ffloat t) {
  const float n = __fadd_rn(s.h, t.h);
  const float bb = __fsub_rn(n, s.h);
  const float e = __fadd_rn(__fsub_rn(s.h, __fsub_rn(n, bb)), __fsub_rn(t.h, bb));
  s.h = n;
  s.l = __fadd_rn(s.l, __fadd_rn(e, t.l));
}

__device__ __forceinline__ double ff_to_double(ffloat a) {
  return (double)a.h + (double)a.l;
}

__device__ __forceinline__ ffloat ff_from_double(double x) {
  const float h = (float)x;
  return ff_make(h, (float)(x - (double)h));
}

}  // namespace fsph

// ---- two float-float values at once (one per float2 lane) ------------------
// The same operations on float2 words with Blackwell's packed FP32x2
// instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn): two neighbours' pair
// terms per instruction, which halves the issue slots of the float-float
// passes' arithmetic (the FMA pipe's work stays the same).  a - b is
// __ffma2_rn(b, -1, a): one rounding, as a subtraction.
namespace fsph {

struct ffloat2 {
  float2 h, l;
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2s(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, f2s(-1.f), a);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 neg2(float2 a) { return f2(-a.x, -a.y); }

__device__ __forceinline__ ffloat2 ff2_make(float2 h, float2 l) {
  ffloat2 r;
  r.h = h;
  r.l = l;
  return r;
}
__device__ __forceinline__ ffloat2 ff2_bcast(ffloat a) {
  return ff2_make(f2s(a.h), f2s(a.l));
}
__device__ __forceinline__ ffloat ff2_lane(const ffloat2 & a, int k) {
  return k == 0 ? ff_make(a.h.x, a.l.x) : ff_make(a.h.y, a.l.y);
}

__device__ __forceinline__ ffloat2 ff2_add(ffloat2 a, ffloat2 b) {
  const float2 s = add2(a.h, b.h);
  const float2 bb = sub2(s, a.h);
  const float2 e = add2(sub2(a.h, sub2(s, bb)), sub2(b.h, bb));
  return ff2_make(s, add2(e, add2(a.l, b.l)));
}
__device__ __forceinline__ ffloat2 ff2_cadd(float c, ffloat2 b) {
  const float2 s = add2(f2s(c), b.h);
  const float2 e = sub2(b.h, sub2(s, f2s(c)));
  return ff2_make(s, add2(e, b.l));
}
__device__ __forceinline__ ffloat2 ff2_norm(ffloat2 a) {
  const float2 s = add2(a.h, a.l);
  return ff2_make(s, sub2(a.l, sub2(s, a.h)));
}
__device__ __forceinline__ ffloat2 ff2_mul(ffloat2 a, ffloat2 b) {
  const float2 p = mul2(a.h, b.h);
  float2 e = fma2(a.h, b.h, neg2(p));
  e = fma2(a.h, b.l, e);
  e = fma2(a.l, b.h, e);
  return ff2_make(p, e);
}
__device__ __forceinline__ ffloat2 ff2_scale2(ffloat2 a, float c) {
  return ff2_make(mul2(a.h, f2s(c)), mul2(a.l, f2s(c)));
}
__device__ __forceinline__ ffloat2 ff2_sqr(ffloat2 a) {
  const float2 p = mul2(a.h, a.h);
  float2 e = fma2(a.h, a.h, neg2(p));
  e = fma2(add2(a.h, a.h), a.l, e);
  return ff2_make(p, e);
}
__device__ __forceinline__ ffloat2 ff2_sqr_wide(ffloat2 a) {
  const float2 p = mul2(a.h, a.h);
  float2 e = fma2(a.h, a.h, neg2(p));
  e = fma2(add2(a.h, a.h), a.l, e);
  e = fma2(a.l, a.l, e);
  return ff2_make(p, e);
}
// sqrt of a normalised a >= 0 (the rsqrt per lane)
__device__ __forceinline__ ffloat2 ff2_sqrt(ffloat2 a) {
  const float2 rs = f2(a.h.x > 0.f ? rsqrtf(a.h.x) : 0.f, a.h.y > 0.f ? rsqrtf(a.h.y) : 0.f);
  const float2 r = mul2(a.h, rs);
  const float2 d = add2(fma2(neg2(r), r, a.h), a.l);
  return ff2_make(r, mul2(d, mul2(f2s(0.5f), rs)));
}
// c / a for a float constant c (the reciprocal per lane)
__device__ __forceinline__ ffloat2 ff2_rcp_scaled(ffloat2 a, float c) {
  const float2 r = f2(1.0f / a.h.x, 1.0f / a.h.y);
  float2 e = fma2(neg2(a.h), r, f2s(1.0f));
  e = fma2(neg2(a.l), r, e);
  return ff2_make(mul2(f2s(c), r), mul2(f2s(c), mul2(e, r)));
}
__device__ __forceinline__ void ff2_acc(ffloat2 & s, ffloat2 t) {
  const float2 n = add2(s.h, t.h);
  const float2 bb = sub2(n, s.h);
  const float2 e = add2(sub2(s.h, sub2(n, bb)), sub2(t.h, bb));
  s.h = n;
  s.l = add2(s.l, add2(e, t.l));
}

}  // namespace fsph
