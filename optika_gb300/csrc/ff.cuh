// Float-float ("double-float") arithmetic for the multilayer kernels.
//
// A value is an unevaluated sum hi + lo of two floats (~48-bit
// significand).  The building blocks are the published error-free
// transformations: Knuth's TwoSum, Dekker's Fast2Sum and the FMA-based
// TwoProduct, combined as in the double-word algorithms of Dekker (1971)
// and Joldes, Muller and Popescu (2017).  Only +, -, *, / and sqrt of
// floats and FMAs are used.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace otx {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_fast2sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_twosum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ ff ff_of(float a) { return ff{a, 0.f}; }

// The double-word sum with one TwoSum (Joldes, Muller and Popescu 2017,
// "sloppy" DWPlusDW): its error is within ~2^-47 of the larger operand,
// not of the sum, which is all the transfer-matrix products need (their
// entries are rescaled to O(1) and R, T are wanted to 1e-5 absolute); it
// takes about half the instructions of the accurate form.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = ff_twosum(a.hi, b.hi);
  return ff_fast2sum(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_fast2sum(p, e);
}

__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  const float p = a.hi * b;
  const float e = fmaf(a.lo, b, fmaf(a.hi, b, -p));
  return ff_fast2sum(p, e);
}

__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = a.hi / b.hi;
  // r = a - q1 b, exactly up to the low parts
  const float p = q1 * b.hi;
  const float pe = fmaf(q1, b.hi, -p);
  const float r = ((a.hi - p) - pe + a.lo) - q1 * b.lo;
  const float q2 = r / b.hi;
  return ff_fast2sum(q1, q2);
}

__device__ __forceinline__ ff ff_sqrt(ff a) {
  if (!(a.hi > 0.f)) return ff{sqrtf(a.hi), 0.f};
  const float s = sqrtf(a.hi);
  const float p = s * s;
  const float pe = fmaf(s, s, -p);
  const float r = ((a.hi - p) - pe + a.lo) / (2.f * s);
  return ff_fast2sum(s, r);
}

__device__ __forceinline__ ff ff_scale2(ff a, float p2) {  // exact power of two
  return ff{a.hi * p2, a.lo * p2};
}

__device__ __forceinline__ float ff_to_f(ff a) { return a.hi + a.lo; }

// ---------------------------------------------------------------- complex

struct cff {
  ff re, im;
};

__device__ __forceinline__ cff cff_of(float re, float im) { return cff{ff_of(re), ff_of(im)}; }
__device__ __forceinline__ cff cff_add(cff a, cff b) {
  return cff{ff_add(a.re, b.re), ff_add(a.im, b.im)};
}
__device__ __forceinline__ cff cff_sub(cff a, cff b) {
  return cff{ff_sub(a.re, b.re), ff_sub(a.im, b.im)};
}
__device__ __forceinline__ cff cff_mul(cff a, cff b) {
  return cff{ff_sub(ff_mul(a.re, b.re), ff_mul(a.im, b.im)),
             ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}
__device__ __forceinline__ cff cff_conj(cff a) { return cff{a.re, ff_neg(a.im)}; }
__device__ __forceinline__ cff cff_scale(cff a, ff s) { return cff{ff_mul(a.re, s), ff_mul(a.im, s)}; }
__device__ __forceinline__ cff cff_scale2(cff a, float p2) {
  return cff{ff_scale2(a.re, p2), ff_scale2(a.im, p2)};
}
__device__ __forceinline__ ff cff_abs2(cff a) {
  return ff_add(ff_mul(a.re, a.re), ff_mul(a.im, a.im));
}
__device__ __forceinline__ cff cff_div(cff a, cff b) {
  const ff inv = ff_div(ff_of(1.f), cff_abs2(b));
  return cff_scale(cff_mul(a, cff_conj(b)), inv);
}
// Principal square root (branch cut on the negative real axis, as numpy).
__device__ __forceinline__ cff cff_sqrt(cff z) {
  const ff m = ff_sqrt(cff_abs2(z));
  const ff ax = z.re.hi >= 0.f ? z.re : ff_neg(z.re);
  const ff h = ff_scale2(ff_add(m, ax), 0.5f);
  if (h.hi == 0.f) return cff{ff_of(0.f), z.im};
  const ff t = ff_sqrt(h);                              // sqrt(h)
  const ff aim = z.im.hi >= 0.f ? z.im : ff_neg(z.im);  // |im|
  const ff u = ff_div(aim, ff_scale2(t, 2.f));          // |im| / (2 sqrt(h))
  if (z.re.hi >= 0.f) return cff{t, z.im.hi >= 0.f ? u : ff_neg(u)};
  return cff{u, z.im.hi >= 0.f ? t : ff_neg(t)};
}

struct cmff {
  cff a, b, c, d;  // [[a, b], [c, d]]
};

__device__ __forceinline__ cmff cmff_mul(const cmff& x, const cmff& y) {
  return cmff{cff_add(cff_mul(x.a, y.a), cff_mul(x.b, y.c)),
              cff_add(cff_mul(x.a, y.b), cff_mul(x.b, y.d)),
              cff_add(cff_mul(x.c, y.a), cff_mul(x.d, y.c)),
              cff_add(cff_mul(x.c, y.b), cff_mul(x.d, y.d))};
}

// x^2 of a complex float-float: (re^2 - im^2, 2 re im).
__device__ __forceinline__ cff cff_sqr(cff a) {
  return cff{ff_sub(ff_mul(a.re, a.re), ff_mul(a.im, a.im)), ff_scale2(ff_mul(a.re, a.im), 2.f)};
}

// M^2 of a 2x2 matrix: [[a^2 + bc, b (a + d)], [c (a + d), d^2 + bc]].
__device__ __forceinline__ cmff cmff_sqr(const cmff& m) {
  const cff bc = cff_mul(m.b, m.c), tr = cff_add(m.a, m.d);
  return cmff{cff_add(cff_sqr(m.a), bc), cff_mul(m.b, tr), cff_mul(m.c, tr),
              cff_add(cff_sqr(m.d), bc)};
}

// A column vector of two complex float-float values.
struct cvff {
  cff x, y;
};

__device__ __forceinline__ cvff cmff_apply(const cmff& m, const cvff& v) {
  return cvff{cff_add(cff_mul(m.a, v.x), cff_mul(m.b, v.y)),
              cff_add(cff_mul(m.c, v.x), cff_mul(m.d, v.y))};
}

// Exact power-of-two rescaling so the largest component is O(1).
__device__ __forceinline__ void cmff_normalize(cmff& m, int& exp2) {
  const float mx = fmaxf(fmaxf(fmaxf(fabsf(m.a.re.hi), fabsf(m.a.im.hi)),
                               fmaxf(fabsf(m.b.re.hi), fabsf(m.b.im.hi))),
                         fmaxf(fmaxf(fabsf(m.c.re.hi), fabsf(m.c.im.hi)),
                               fmaxf(fabsf(m.d.re.hi), fabsf(m.d.im.hi))));
  if (!(mx > 0.f) || !isfinite(mx)) return;
  const int e = ilogbf(mx);
  const float s = ldexpf(1.f, -e);
  m.a = cff_scale2(m.a, s);
  m.b = cff_scale2(m.b, s);
  m.c = cff_scale2(m.c, s);
  m.d = cff_scale2(m.d, s);
  exp2 += e;
}

__device__ __forceinline__ void cvff_normalize(cvff& v, int& exp2) {
  const float mx = fmaxf(fmaxf(fabsf(v.x.re.hi), fabsf(v.x.im.hi)),
                         fmaxf(fabsf(v.y.re.hi), fabsf(v.y.im.hi)));
  if (!(mx > 0.f) || !isfinite(mx)) return;
  const int e = ilogbf(mx);
  const float s = ldexpf(1.f, -e);
  v.x = cff_scale2(v.x, s);
  v.y = cff_scale2(v.y, s);
  exp2 += e;
}

}  // namespace otx
