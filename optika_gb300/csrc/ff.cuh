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

// a b + c d in one pass: the two leading products and their exact errors
// (FMA), one TwoSum of the products, the cross terms accumulated in FP32,
// one Fast2Sum.  Its error is within a few 2^-48 of the larger product, as
// the sloppy sum's is of its larger operand; it issues about a quarter
// fewer instructions than two products and a sum.
__device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d) {
  const float p = a.hi * b.hi, q = c.hi * d.hi;
  const ff s = ff_twosum(p, q);
  float lo = s.lo + (fmaf(a.hi, b.hi, -p) + fmaf(c.hi, d.hi, -q));
  lo = fmaf(a.hi, b.lo, lo);
  lo = fmaf(a.lo, b.hi, lo);
  lo = fmaf(c.hi, d.lo, lo);
  lo = fmaf(c.lo, d.hi, lo);
  return ff_fast2sum(s.hi, lo);
}

// a0 b0 + a1 b1 + a2 b2 + a3 b3 the same way (a tree of three TwoSums).
__device__ __forceinline__ ff ff_dot4(ff a0, ff b0, ff a1, ff b1, ff a2, ff b2, ff a3, ff b3) {
  const float p0 = a0.hi * b0.hi, p1 = a1.hi * b1.hi, p2 = a2.hi * b2.hi, p3 = a3.hi * b3.hi;
  const ff s = ff_twosum(p0, p1), t = ff_twosum(p2, p3);
  const ff u = ff_twosum(s.hi, t.hi);
  float lo = (fmaf(a0.hi, b0.hi, -p0) + fmaf(a1.hi, b1.hi, -p1)) +
             (fmaf(a2.hi, b2.hi, -p2) + fmaf(a3.hi, b3.hi, -p3));
  lo += (s.lo + t.lo) + u.lo;
  lo = fmaf(a0.hi, b0.lo, lo);
  lo = fmaf(a0.lo, b0.hi, lo);
  lo = fmaf(a1.hi, b1.lo, lo);
  lo = fmaf(a1.lo, b1.hi, lo);
  lo = fmaf(a2.hi, b2.lo, lo);
  lo = fmaf(a2.lo, b2.hi, lo);
  lo = fmaf(a3.hi, b3.lo, lo);
  lo = fmaf(a3.lo, b3.hi, lo);
  return ff_fast2sum(u.hi, lo);
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
  return cff{ff_dot2(a.re, b.re, ff_neg(a.im), b.im), ff_dot2(a.re, b.im, a.im, b.re)};
}
// a x + b y of complex values, each part one four-term dot product.
__device__ __forceinline__ cff cff_dot2(cff a, cff x, cff b, cff y) {
  return cff{ff_dot4(a.re, x.re, ff_neg(a.im), x.im, b.re, y.re, ff_neg(b.im), y.im),
             ff_dot4(a.re, x.im, a.im, x.re, b.re, y.im, b.im, y.re)};
}
__device__ __forceinline__ cff cff_conj(cff a) { return cff{a.re, ff_neg(a.im)}; }
__device__ __forceinline__ cff cff_scale(cff a, ff s) { return cff{ff_mul(a.re, s), ff_mul(a.im, s)}; }
__device__ __forceinline__ cff cff_scale2(cff a, float p2) {
  return cff{ff_scale2(a.re, p2), ff_scale2(a.im, p2)};
}
__device__ __forceinline__ ff cff_abs2(cff a) { return ff_dot2(a.re, a.re, a.im, a.im); }
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
  return cmff{cff_dot2(x.a, y.a, x.b, y.c), cff_dot2(x.a, y.b, x.b, y.d),
              cff_dot2(x.c, y.a, x.d, y.c), cff_dot2(x.c, y.b, x.d, y.d)};
}

// M^2 of a 2x2 matrix: [[a^2 + bc, b (a + d)], [c (a + d), d^2 + bc]].
__device__ __forceinline__ cmff cmff_sqr(const cmff& m) {
  const cff tr = cff_add(m.a, m.d);
  return cmff{cff_dot2(m.a, m.a, m.b, m.c), cff_mul(m.b, tr), cff_mul(m.c, tr),
              cff_dot2(m.d, m.d, m.b, m.c)};
}

// A column vector of two complex float-float values.
struct cvff {
  cff x, y;
};

__device__ __forceinline__ cvff cmff_apply(const cmff& m, const cvff& v) {
  return cvff{cff_dot2(m.a, v.x, m.b, v.y), cff_dot2(m.c, v.x, m.d, v.y)};
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
