// Device functions of the fused sequential raytrace.
//
// Each function restates one step of optika's per-surface pipeline
// (optika/surfaces.py:123-198) for one ray held in registers.  Arithmetic
// is FP32; the frame changes between surfaces add their (large) translation
// as a float-float pair so that positions near a surface stay accurate, and
// every curved intercept ends with one Newton step evaluated in the
// surface's own (small) coordinates.  The optical path length accumulates
// as a float-float pair (FP64 throughput on GB300 is a small fraction of
// FP32) and is stored as float64.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/optika_gb300.h"
#include "trace_kernel_decl.h"

namespace otx {

struct Ray {
  float px, py, pz;      // position in the current frame (mm)
  float dx, dy, dz;      // direction cosines (high parts)
  float lx, ly, lz;      // direction low parts (float-float direction)
  float wl;              // wavelength (nm)
  float inten;           // intensity
  float att;             // attenuation coefficient (1/mm)
  float n;               // index of refraction of the current medium
  bool ok;               // unvignetted
  float opl_hi, opl_lo;  // optical path length (mm), float-float
};

// ---------------------------------------------------------------- helpers

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// |d|^2 - 1 of a near-unit float-float vector d = (x, y, z) + (lx, ly, lz),
// accurate to ~1e-14: the squares split exactly by FMA (TwoProduct), their
// sum by TwoSum (Ogita-Rump-Oishi Sum2); s2 is within [0.5, 2], so s2 - 1
// is exact (Sterbenz).
__device__ __forceinline__ float norm2_minus_one(float x, float y, float z, float lx, float ly,
                                                 float lz) {
  const float p1 = x * x, e1 = fmaf(x, x, -p1);
  const float p2 = y * y, e2 = fmaf(y, y, -p2);
  const float p3 = z * z, e3 = fmaf(z, z, -p3);
  float s, t1, s2, t2;
  two_sum(p1, p2, s, t1);
  two_sum(s, p3, s2, t2);
  const float ld = fmaf(x, lx, fmaf(y, ly, z * lz));
  return (s2 - 1.f) + fmaf(2.f, ld, (t1 + t2) + (e1 + e2 + e3));
}

// Make a float-float direction unit to ~1e-14 by moving its low parts
// (d -> d (1 - e / 2), e = |d|^2 - 1); FP32 rounding leaves |e| ~ 1e-7,
// which a 400 mm segment would turn into 4e-5 mm of optical path.  Vectors
// farther from unit length (|e| >= 1e-4: caller-supplied non-unit
// directions) are left as they are.
__device__ __forceinline__ void unit_ff(float x, float y, float z, float& lx, float& ly,
                                        float& lz) {
  const float e = norm2_minus_one(x, y, z, lx, ly, lz);
  if (!(fabsf(e) < 1e-4f)) return;
  const float h = -0.5f * e;
  lx = fmaf(h, x, lx);
  ly = fmaf(h, y, ly);
  lz = fmaf(h, z, lz);
}

// opl += n (t + tl) for a segment parameter held as a float-float pair:
// the product n t split exactly by an FMA (Dekker's TwoProduct), the sum by
// TwoSum; the low parts, with n tl, are gathered in opl_lo.
__device__ __forceinline__ void opl_add(Ray& r, float n, float t, float tl) {
  const float p = n * t;
  const float pe = fmaf(n, t, -p);
  float s, e;
  two_sum(r.opl_hi, p, s, e);
  r.opl_hi = s;
  r.opl_lo += fmaf(n, tl, e + pe);
}

__device__ __forceinline__ float sgnf(float x) {  // numpy.sign: 0 at 0
  return (x > 0.f) ? 1.f : ((x < 0.f) ? -1.f : 0.f);
}

// Apply x' = m x + t to a position: the rotation in FP32, the translation
// as a float-float add.  Returns the high part in (x,y,z) and the low part
// in lo.
__device__ __forceinline__ void affine_point(const otx_affine& f, float& x,
                                             float& y, float& z, float lo[3]) {
  float rx = fmaf(f.m[0], x, fmaf(f.m[1], y, f.m[2] * z));
  float ry = fmaf(f.m[3], x, fmaf(f.m[4], y, f.m[5] * z));
  float rz = fmaf(f.m[6], x, fmaf(f.m[7], y, f.m[8] * z));
  float e;
  two_sum(rx, f.t_hi[0], x, e);
  lo[0] = e + f.t_lo[0];
  two_sum(ry, f.t_hi[1], y, e);
  lo[1] = e + f.t_lo[1];
  two_sum(rz, f.t_hi[2], z, e);
  lo[2] = e + f.t_lo[2];
}

__device__ __forceinline__ void rotate(const otx_affine& f, float& x, float& y,
                                       float& z) {
  float rx = fmaf(f.m[0], x, fmaf(f.m[1], y, f.m[2] * z));
  float ry = fmaf(f.m[3], x, fmaf(f.m[4], y, f.m[5] * z));
  float rz = fmaf(f.m[6], x, fmaf(f.m[7], y, f.m[8] * z));
  x = rx;
  y = ry;
  z = rz;
}

// Full affine map of a position (high + low folded), used for outputs.
__device__ __forceinline__ void affine_point_folded(const otx_affine& f,
                                                    float& x, float& y,
                                                    float& z) {
  if (f.flags & OTX_AFFINE_IDENTITY) return;
  float lo[3];
  affine_point(f, x, y, z, lo);
  x += lo[0];
  y += lo[1];
  z += lo[2];
}

// One row of a rotation with float-float entries applied to a float-float
// vector: products split exactly by FMA, sums by TwoSum (Ogita-Rump-Oishi
// Dot2); returns a float-float pair.
__device__ __forceinline__ void rot_row_ff(const float* mh, const float* ml, float x, float y,
                                           float z, float xl, float yl, float zl, float& hi,
                                           float& lo) {
  const float p1 = mh[0] * x, e1 = fmaf(mh[0], x, -p1);
  const float p2 = mh[1] * y, e2 = fmaf(mh[1], y, -p2);
  const float p3 = mh[2] * z, e3 = fmaf(mh[2], z, -p3);
  float s, t1, s2, t2;
  two_sum(p1, p2, s, t1);
  two_sum(s, p3, s2, t2);
  float l = (t1 + t2) + (e1 + e2 + e3);
  l = fmaf(ml[0], x, fmaf(ml[1], y, fmaf(ml[2], z, l)));
  l = fmaf(mh[0], xl, fmaf(mh[1], yl, fmaf(mh[2], zl, l)));
  hi = s2 + l;
  lo = l - (hi - s2);
}

// a x + b z in float-float for float-float entries (a, b) and vector
// components (x, z): one row of a rotation in a coordinate plane.
__device__ __forceinline__ void rot2_ff(float ah, float al, float bh, float bl, float x, float z,
                                        float xl, float zl, float& hi, float& lo) {
  const float p1 = ah * x, e1 = fmaf(ah, x, -p1);
  const float p2 = bh * z, e2 = fmaf(bh, z, -p2);
  float s, t;
  two_sum(p1, p2, s, t);
  float l = t + (e1 + e2);
  l = fmaf(al, x, fmaf(bl, z, l));
  l = fmaf(ah, xl, fmaf(bh, zl, l));
  hi = s + l;
  lo = l - (hi - s);
}

// Frame change of a ray: position (x, y, z) -> (x, y, z) + lo in the new
// frame, direction (float-float) rotated.  Pure translations (the common
// case) add the translation only; rotations are compensated, because an
// FP32-rounded direction component (~3e-8 for 0.7) would act over the
// whole incoming segment (hundreds of mm) before the intercept.  A
// rotation about y (tilts in the x-z plane: folds, tilted sensors and
// gratings) mixes x and z only, with two-term rows; y passes through.
__device__ __forceinline__ void frame_change(const otx_affine& f, Ray& r, float lo[3]) {
  float px = r.px, py = r.py, pz = r.pz;
  float rh[3], rl[3];
  if (f.flags & OTX_AFFINE_ROT_IDENTITY) {
    rh[0] = px;
    rh[1] = py;
    rh[2] = pz;
    rl[0] = rl[1] = rl[2] = 0.f;
  } else if (f.flags & OTX_AFFINE_ROT_Y) {
    rot2_ff(f.m[0], f.m_lo[0], f.m[2], f.m_lo[2], px, pz, 0.f, 0.f, rh[0], rl[0]);
    rot2_ff(f.m[6], f.m_lo[6], f.m[8], f.m_lo[8], px, pz, 0.f, 0.f, rh[2], rl[2]);
    rh[1] = py;
    rl[1] = 0.f;
    float dxh, dxl, dzh, dzl;
    rot2_ff(f.m[0], f.m_lo[0], f.m[2], f.m_lo[2], r.dx, r.dz, r.lx, r.lz, dxh, dxl);
    rot2_ff(f.m[6], f.m_lo[6], f.m[8], f.m_lo[8], r.dx, r.dz, r.lx, r.lz, dzh, dzl);
    r.dx = dxh;
    r.lx = dxl;
    r.dz = dzh;
    r.lz = dzl;
  } else {
    for (int i = 0; i < 3; ++i)
      rot_row_ff(f.m + 3 * i, f.m_lo + 3 * i, px, py, pz, 0.f, 0.f, 0.f, rh[i], rl[i]);
    float dh[3], dl[3];
    for (int i = 0; i < 3; ++i)
      rot_row_ff(f.m + 3 * i, f.m_lo + 3 * i, r.dx, r.dy, r.dz, r.lx, r.ly, r.lz, dh[i], dl[i]);
    r.dx = dh[0];
    r.dy = dh[1];
    r.dz = dh[2];
    r.lx = dl[0];
    r.ly = dl[1];
    r.lz = dl[2];
  }
  float e;
  two_sum(rh[0], f.t_hi[0], r.px, e);
  lo[0] = e + (rl[0] + f.t_lo[0]);
  two_sum(rh[1], f.t_hi[1], r.py, e);
  lo[1] = e + (rl[1] + f.t_lo[1]);
  two_sum(rh[2], f.t_hi[2], r.pz, e);
  lo[2] = e + (rl[2] + f.t_lo[2]);
}

// ---------------------------------------------------------------- sags

// Sag z(x, y) and its gradient for the curved sag types.
// Conic: optika/sags/_conic.py:31-48 (sag), :50-75 (gradient c x / g).
// Toroid: optika/sags/_toroidal.py:38-57 (sag), :59-88 (gradient).
// FAST_GRAD forms the gradient's quotients approximately (2 ulp), for
// Newton steps, whose root the gradient does not move; the sag value and
// the normals keep exact quotients.
template <bool FAST_GRAD = false>
__device__ __forceinline__ float sag_eval(int sag_type, const otx_surface& s, float x,
                                          float y, float& gx, float& gy) {
  switch (sag_type) {
    case OTX_SAG_SPHERE:
    case OTX_SAG_CONIC:
    case OTX_SAG_PARABOLA: {
      const float c = s.sag_curvature;
      const float kp1 = (sag_type == OTX_SAG_SPHERE) ? 1.f : 1.f + s.sag_conic;
      const float r2 = fmaf(x, x, y * y);
      if (kp1 == 0.f) {  // paraboloid: g = 1 exactly, the same values below
        gx = c * x;
        gy = c * y;
        return 0.5f * (c * r2);
      }
      const float g = sqrtf(1.f - kp1 * c * c * r2);
      const float cg = FAST_GRAD ? __fdividef(c, g) : c / g;
      gx = cg * x;
      gy = cg * y;
      return c * r2 / (1.f + g);
    }
    case OTX_SAG_CYLINDER: {
      // optika/sags/_cylindrical.py:75-91: z = c x^2 / (1 + sqrt(1 - c^2 x^2))
      const float c = s.sag_curvature;
      const float x2 = x * x;
      const float g = sqrtf(1.f - c * c * x2);
      gx = c * x / g;
      gy = 0.f;
      return c * x2 / (1.f + g);
    }
    case OTX_SAG_TOROID: {
      const float c = s.sag_curvature;
      const float r = s.sag_radius_of_rotation;
      const float y2 = y * y;
      const float g = sqrtf(1.f - c * c * y2);
      const float zy = c * y2 / (1.f + g);
      const float rz = r - zy;
      const float f = sqrtf(fmaf(rz, rz, -x * x));
      const float inv_f = FAST_GRAD ? __fdividef(1.f, f) : 1.f / f;
      gx = x * inv_f;
      gy = rz * (FAST_GRAD ? __fdividef(c * y, g) : c * y / g) * inv_f;
      // r - f = (r^2 - f^2) / (r + f) = (z_y (2 r - z_y) + x^2) / (r + f),
      // free of the cancellation of r - f when f ~ r > 0
      if (r >= 0.f) return fmaf(zy, 2.f * r - zy, x * x) / (r + f);
      return r - f;
    }
    default:
      gx = 0.f;
      gy = 0.f;
      return 0.f;
  }
}

// One Newton step on f(t) = z(t) - sag(x(t), y(t)) from the current point.
__device__ __forceinline__ float newton_step(int sag_type, const otx_surface& s, float& x,
                                             float& y, float& z, float ux,
                                             float uy, float uz) {
  float gx, gy;
  const float zs = sag_eval<true>(sag_type, s, x, y, gx, gy);
  const float f = z - zs;
  const float fp = uz - (gx * ux + gy * uy);
  const float dt = __fdividef(f, fp);  // a small correction: 2 ulp of it suffice
  x = fmaf(-dt, ux, x);
  y = fmaf(-dt, uy, y);
  z = fmaf(-dt, uz, z);
  return dt;
}

// Intercept of the ray (origin o = hi + lo, direction u) with the sag.
// On return (x,y,z) is the intercept in the surface frame and t the signed
// distance along u from the origin.
//
// Root choice follows the reference for each type:
//   flat      optika/sags/_flat.py:47-64
//   sphere    optika/sags/_spherical.py:148-191 (root with -sign(r u_z))
//   conic     optika/sags/_conic.py:77-170 (vertex-sheet root nearest o)
//   parabola  optika/sags/_parabolic.py:65-158 (-sign(f u_z) root,
//             linear form when u_x^2 + u_y^2 <= 1e-10)
//   toroid    optika/sags/_abc.py:76-107 (iterative root near the vertex
//             plane; here Newton from the plane intercept)
//   cylinder  optika/sags/_cylindrical.py:115-160 (circle of radius R about
//             the y axis through (0, 0, R): the -sign(R u_z) root of
//             (u_x^2 + u_z^2) t^2 + 2 hb t + cc = 0, and the vertex-plane
//             intercept -o_z / u_z when the discriminant is not positive)
// The closed forms use the cancellation-free product-of-roots identity.
//
// The direction's low parts (lx, ly, lz) enter only the intercept point
// (o_hi + t u_hi) + (o_lo + t u_lo), where they act over the full segment.
//
// The segment parameter is returned as a float-float pair t + tl: t is the
// FP32 value from which the point o + t u is formed (in small coordinates,
// so that point is accurate), and tl the Newton corrections applied to that
// point afterwards.  A rounded FP32 t alone would carry up to half an ulp of
// a ~400 mm segment (1.5e-5 mm) into the optical path length.
__device__ __forceinline__ float intercept(int sag_type, const otx_surface& s,
                                           int newton_max, float ox, float oy,
                                           float oz, const float lo[3],
                                           float ux, float uy, float uz,
                                           float lx, float ly, float lz,
                                           float& x, float& y, float& z, float& tl) {
  const float oxf = ox + lo[0], oyf = oy + lo[1], ozf = oz + lo[2];
  if (sag_type == OTX_SAG_FLAT) {
    // an approximate reciprocal: the Newton step below uses the same one,
    // so the point lands on z = 0 and t + tl stays exact to rounding
    const float inv = __fdividef(1.f, uz);
    const float t0 = -ozf * inv;
    const float t = t0 - (t0 * lz) * inv;  // first order in u_lo
    x = fmaf(t, ux, ox) + fmaf(t, lx, lo[0]);
    y = fmaf(t, uy, oy) + fmaf(t, ly, lo[1]);
    z = fmaf(t, uz, oz) + fmaf(t, lz, lo[2]);
    const float dt = z * inv;  // Newton step on z = 0
    x = fmaf(-dt, ux, x);
    y = fmaf(-dt, uy, y);
    z = 0.f;
    tl = -dt;
    return t;
  }
  float t;
  bool polish = true;
  switch (sag_type) {
    case OTX_SAG_SPHERE: {
      const float R = s.sag_radius;
      // p = o - (0, 0, R); b = u.p; cc = |p|^2 - R^2 = |o|^2 - 2 o_z R
      const float b = fmaf(ux, oxf, fmaf(uy, oyf, uz * (ozf - R)));
      const float cc = fmaf(oxf, oxf, fmaf(oyf, oyf, ozf * (ozf - 2.f * R)));
      const float q = sqrtf(fmaf(b, b, -cc));
      const float sg = sgnf(R * uz);
      // chosen root: -b - sg q ; the other root: -b + sg q ; product = cc
      // (an approximate quotient: the Newton step polishes the root)
      if (sg != 0.f && sgnf(-b) == sg)
        t = __fdividef(cc, -b + sg * q);
      else
        t = -b - sg * q;
      break;
    }
    case OTX_SAG_CONIC: {
      const float c = s.sag_curvature;
      const float kp1 = 1.f + s.sag_conic;
      const float A = c * fmaf(ux, ux, fmaf(uy, uy, kp1 * uz * uz));
      const float B = 2.f * (c * fmaf(oxf, ux, fmaf(oyf, uy, kp1 * ozf * uz)) - uz);
      const float C = fmaf(c, fmaf(oxf, oxf, fmaf(oyf, oyf, kp1 * ozf * ozf)),
                           -2.f * ozf);
      const float disc = fmaf(B, B, -4.f * A * C);
      const bool real = disc >= 0.f;
      const float sq = sqrtf(real ? disc : 0.f);
      float ta, tb;  // roots with -sqrt and +sqrt
      if (fabsf(A) < 1e-12f) {
        ta = -C / B;
        tb = ta;
      } else {
        const float qq = -0.5f * (B + copysignf(sq, B));
        // approximate quotients: the Newton step polishes the chosen root
        const float r1 = __fdividef(qq, A), r2 = __fdividef(C, qq);
        if (B >= 0.f) {
          ta = r1;
          tb = r2;
        } else {
          ta = r2;
          tb = r1;
        }
      }
      // vertex-sheet test z (c r^2 - z) >= 0 on each candidate
      const float za = fmaf(ta, uz, ozf), xa = fmaf(ta, ux, oxf), ya = fmaf(ta, uy, oyf);
      const float zb = fmaf(tb, uz, ozf), xb = fmaf(tb, ux, oxf), yb = fmaf(tb, uy, oyf);
      const bool va = real && (za * (c * fmaf(xa, xa, ya * ya) - za) >= 0.f);
      const bool vb = real && (zb * (c * fmaf(xb, xb, yb * yb) - zb) >= 0.f);
      ta = va ? ta : INFINITY;
      tb = vb ? tb : INFINITY;
      t = (fabsf(ta) <= fabsf(tb)) ? ta : tb;
      break;
    }
    case OTX_SAG_PARABOLA: {
      const float f = s.sag_focal_length;
      const float a = fmaf(ux, ux, uy * uy);
      // a t^2 + 2 hb t + cc = 0
      const float hb = fmaf(oxf, ux, oyf * uy) - 2.f * f * uz;
      const float cc = fmaf(oxf, oxf, oyf * oyf) - 4.f * f * ozf;
      if (a > 1e-10f) {
        const float sq = sqrtf(fmaf(hb, hb, -a * cc));
        const float sg = sgnf(f * uz);
        if (sg != 0.f && sgnf(-hb) == sg)
          t = cc / (-hb + sg * sq);
        else
          t = (-hb - sg * sq) / a;
      } else {
        t = cc / (4.f * f * uz);
      }
      break;
    }
    case OTX_SAG_CYLINDER: {
      const float R = s.sag_radius;
      const float a = fmaf(ux, ux, uz * uz);
      const float hb = fmaf(ux, oxf, uz * (ozf - R));
      const float cc = fmaf(oxf, oxf, ozf * (ozf - 2.f * R));
      const float disc = fmaf(hb, hb, -a * cc);
      if (disc > 0.f) {
        const float q = sqrtf(disc);
        const float sg = sgnf(R * uz);
        // chosen root (-hb - sg q) / a ; the other (-hb + sg q) / a ;
        // their product cc / a
        if (sg != 0.f && sgnf(-hb) == sg)
          t = cc / (-hb + sg * q);
        else
          t = (-hb - sg * q) / a;
      } else {
        t = -ozf / uz;
        polish = false;  // the reference keeps the vertex-plane point
      }
      break;
    }
    default:  // toroid: start from the vertex plane
      t = -ozf / uz;
      break;
  }
  // point on the ray, small coordinates: (o_hi + t u) + (o_lo + t u_lo)
  x = fmaf(t, ux, ox) + fmaf(t, lx, lo[0]);
  y = fmaf(t, uy, oy) + fmaf(t, ly, lo[1]);
  z = fmaf(t, uz, oz) + fmaf(t, lz, lo[2]);
  tl = 0.f;
  if (sag_type == OTX_SAG_TOROID) {
    const int iters = newton_max > 0 ? newton_max : 12;
    bool conv = false;
    for (int i = 0; i < iters; ++i) {
      const float dt = newton_step(sag_type, s, x, y, z, ux, uy, uz);
      float ts, te;
      two_sum(t, -dt, ts, te);
      t = ts;
      tl += te;
      if (fabsf(dt) <= 1e-7f * (1.f + fabsf(t))) {
        conv = true;
        break;
      }
    }
    if (!conv) {
      x = y = z = NAN;
    }
  } else if (polish && isfinite(t)) {
    tl = -newton_step(sag_type, s, x, y, z, ux, uy, uz);
  }
  return t;
}

// Surface normal at a point of the sag (z < 0 convention).
//   flat     optika/sags/_flat.py:41-45
//   sphere   optika/sags/_spherical.py:125-146
//   conic    optika/sags/_conic.py:50-75
//   parabola optika/sags/_parabolic.py:40-63 (equal to the k = -1 conic)
//   toroid   optika/sags/_toroidal.py:59-88
//   cylinder optika/sags/_cylindrical.py:93-113 (x / R, 0, -sqrt(1 - (x/R)^2))
//
// v receives a vector parallel to the normal that is exact up to the
// rounding of its components (the unnormalised gradient (g_x, g_y, -1), or
// for the sphere the normal itself); curved mirrors reflect off v.
__device__ __forceinline__ void normal(int sag_type, const otx_surface& s, float x, float y,
                                       float& nx, float& ny, float& nz, float v[3]) {
  switch (sag_type) {
    case OTX_SAG_SPHERE: {
      const float c = s.sag_curvature;
      nx = c * x;
      ny = c * y;
      nz = -sqrtf(1.f - nx * nx - ny * ny);
      v[0] = nx;
      v[1] = ny;
      v[2] = nz;
      return;
    }
    case OTX_SAG_CYLINDER: {
      nx = s.sag_curvature * x;
      ny = 0.f;
      nz = -sqrtf(1.f - nx * nx);
      v[0] = nx;
      v[1] = ny;
      v[2] = nz;
      return;
    }
    case OTX_SAG_CONIC:
    case OTX_SAG_PARABOLA:
    case OTX_SAG_TOROID: {
      float gx, gy;
      sag_eval(sag_type, s, x, y, gx, gy);
      // 1 / |(gx, gy, -1)|: the hardware estimate refined by one Newton step
      const float q = fmaf(gx, gx, fmaf(gy, gy, 1.f));
      float inv = rsqrtf(q);
      inv = fmaf(0.5f * inv, fmaf(-q * inv, inv, 1.f), inv);
      nx = gx * inv;
      ny = gy * inv;
      nz = -inv;
      v[0] = gx;
      v[1] = gy;
      v[2] = -1.f;
      return;
    }
    default:
      nx = 0.f;
      ny = 0.f;
      nz = -1.f;
      v[0] = 0.f;
      v[1] = 0.f;
      v[2] = -1.f;
      return;
  }
}

// ---------------------------------------------------------------- Snell

// Compensated dot product a.u (Ogita-Rump-Oishi Dot2: products split
// exactly by FMA, sums by TwoSum); accurate to ~1 ulp of the result.
__device__ __forceinline__ float dot3_compensated(float ax, float ay, float az, float ux,
                                                  float uy, float uz) {
  const float p1 = az * uz, e1 = fmaf(az, uz, -p1);
  const float p2 = ay * uy, e2 = fmaf(ay, uy, -p2);
  const float p3 = ax * ux, e3 = fmaf(ax, ux, -p3);
  float s, t1, s2, t2;
  two_sum(p1, p2, s, t1);
  two_sum(s, p3, s2, t2);
  return s2 + ((t1 + t2) + (e1 + e2 + e3));
}

// Scale a (near-)unit float-float vector to unit length when its length
// differs from 1 by more than FP32 rounding (reciprocal square root refined
// by one Newton step); a vector already unit to rounding is left as is.
__device__ __forceinline__ void normalize3(float& x, float& y, float& z, float& lx, float& ly,
                                           float& lz) {
  float e = fmaf(x, x, -1.f);
  e = fmaf(y, y, e);
  e = fmaf(z, z, e);
  e += 2.f * fmaf(x, lx, fmaf(y, ly, z * lz));
  if (fabsf(e) < 3e-7f) return;
  const float q = 1.f + e;
  float inv = rsqrtf(q);
  inv = fmaf(0.5f * inv, fmaf(-q * inv, inv, 1.f), inv);
  x *= inv;
  y *= inv;
  z *= inv;
  lx *= inv;
  ly *= inv;
  lz *= inv;
}

// Vector Snell's law, optika/materials/_snells_law.py:341-366:
//   d = -a.u + sgn (2 m - 1) sqrt(1/r^2 + (a.u)^2 - |a|^2),  b = r (a + d u)
// with sgn = -copysign(1, a.u).  The radicand's (1/r^2 - |a|^2) is formed
// as ((n2/n1)^2 - 1) - (|a|^2 - 1) with fused multiply-adds, and a.u is a
// compensated dot product: a rounding error in a.u would otherwise leave
// the reflected direction off unit length along the normal, and the next
// surface would turn that into a transverse error.  A direction whose
// |a|^2 differs from 1 by less than 1e-6 is unit up to FP32 rounding (the
// reference's float64 directions are unit to 1e-16): that residue is
// dropped instead of being folded into the normal component, and a unit
// ray crossing equal indices without reflection leaves unchanged (the
// formula's d is then 0).  Effective grating directions (|a|^2 - 1 ~ 1e-2)
// keep their residue.  Equal indices skip the divisions (r = 1).
__device__ __forceinline__ void snell(float& ax, float& ay, float& az, float& lx, float& ly,
                                      float& lz, float n1, float n2, bool mirror, float ux,
                                      float uy, float uz) {
  float e = fmaf(ax, ax, -1.f);
  e = fmaf(ay, ay, e);
  e = fmaf(az, az, e);
  const bool unit = fabsf(e) < 1e-6f;
  if (unit) {
    if (!mirror && n1 == n2) return;
    e = 0.f;
  }
  const float au = dot3_compensated(ax, ay, az, ux, uy, uz);
  const float lu = fmaf(lx, ux, fmaf(ly, uy, lz * uz));  // a_lo . u
  const float sgn = -copysignf(1.f, au);
  float r = 1.f, q2m1 = 0.f;
  if (n1 != n2) {
    r = n1 / n2;
    const float q = n2 / n1;
    q2m1 = (q - 1.f) * (q + 1.f);
  }
  float d, dd;  // d and its first-order change from the low parts
  if (mirror && unit && n1 == n2) {
    d = -2.f * au;  // sqrt((a.u)^2) = |a.u| and sgn |a.u| = -a.u
    dd = -2.f * lu;
  } else {
    const float rad = fmaf(au, au, q2m1 - e);
    const float sq = sqrtf(rad);
    const float sig = sgn * (mirror ? 1.f : -1.f);
    d = -au + sig * sq;
    // d(rad) = 2 (a.u) d(a.u) - 2 a.d(a); d(sq) = d(rad) / (2 sq)
    const float al = fmaf(ax, lx, fmaf(ay, ly, az * lz));
    dd = -lu + sig * (au * lu - al) / sq;
  }
  const float bx = fmaf(d, ux, ax), by = fmaf(d, uy, ay), bz = fmaf(d, uz, az);
  lx = r * fmaf(dd, ux, lx);
  ly = r * fmaf(dd, uy, ly);
  lz = r * fmaf(dd, uz, lz);
  ax = r * bx;
  ay = r * by;
  az = r * bz;
  // The formula's b is unit in exact arithmetic for any a (|b|^2 =
  // r^2 (|a|^2 + 2 d a.u + d^2) = 1); renormalising removes a residue
  // along the normal beyond FP32 rounding, and the low parts then take
  // up what FP32 rounding left (the mirror path with a unit direction and
  // a flat sag's exact normal preserves the norm and skips this).
  normalize3(ax, ay, az, lx, ly, lz);
  if (!(mirror && unit && n1 == n2)) unit_ff(ax, ay, az, lx, ly, lz);
}

// Reflection off a curved mirror, b = a - 2 (a.v) v / (v.v), with v parallel
// to the normal but not normalised: the scale k = 2 (a.v) / (v.v) is formed
// in float-float (compensated dot products and a corrected quotient), so the
// transverse components of b carry only the rounding of v's components.
// Equal to the reference's mirror case of Snell's law for unit a.
__device__ __forceinline__ void reflect_curved(float& ax, float& ay, float& az, float& lx,
                                               float& ly, float& lz, const float v[3]) {
  // numerator a.v and denominator v.v as float-float pairs
  float n_hi, n_lo, d_hi, d_lo;
  {
    const float p1 = az * v[2], e1 = fmaf(az, v[2], -p1);
    const float p2 = ay * v[1], e2 = fmaf(ay, v[1], -p2);
    const float p3 = ax * v[0], e3 = fmaf(ax, v[0], -p3);
    float t1, s2, t2, s;
    two_sum(p1, p2, s, t1);
    two_sum(s, p3, s2, t2);
    float lo = (t1 + t2) + (e1 + e2 + e3);
    lo = fmaf(lx, v[0], fmaf(ly, v[1], fmaf(lz, v[2], lo)));  // + a_lo . v
    n_hi = s2 + lo;
    n_lo = lo - (n_hi - s2);
  }
  {
    const float p1 = v[2] * v[2], e1 = fmaf(v[2], v[2], -p1);
    const float p2 = v[1] * v[1], e2 = fmaf(v[1], v[1], -p2);
    const float p3 = v[0] * v[0], e3 = fmaf(v[0], v[0], -p3);
    float t1, s2, t2, s;
    two_sum(p1, p2, s, t1);
    two_sum(s, p3, s2, t2);
    const float lo = (t1 + t2) + (e1 + e2 + e3);
    d_hi = s2 + lo;
    d_lo = lo - (d_hi - s2);
  }
  // q = n / d in float-float: q_hi = n_hi / d_hi, then one correction
  const float q_hi = n_hi / d_hi;
  const float rem = (fmaf(-q_hi, d_hi, n_hi) + n_lo) - q_hi * d_lo;
  const float q_lo = rem / d_hi;
  const float k_hi = 2.f * q_hi, k_lo = 2.f * q_lo;
  // b = a - k v, each component as a float-float pair
  float b[3], bl[3];
  const float a[3] = {ax, ay, az}, al[3] = {lx, ly, lz};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float p = k_hi * v[i];
    const float pe = fmaf(k_hi, v[i], -p);
    float s, e;
    two_sum(a[i], -p, s, e);
    b[i] = s;
    bl[i] = e + (al[i] - pe - k_lo * v[i]);
  }
  ax = b[0];
  ay = b[1];
  az = b[2];
  lx = bl[0];
  ly = bl[1];
  lz = bl[2];
  normalize3(ax, ay, az, lx, ly, lz);
}

// Reflection off a curved mirror whose normal is parallel to the gradient
// form v = (gx, gy, -1) (conic, paraboloid, toroid): reflect_curved with
// v.v = 1 + (gx^2 + gy^2) and a.v = -a_z + (a_x gx + a_y gy) each formed as
// a float-float pair around their dominant exact term, and the quotient
// from one reciprocal with a float-float correction.
__device__ __forceinline__ void reflect_gradient(float& ax, float& ay, float& az, float& lx,
                                                 float& ly, float& lz, float gx, float gy) {
  // a.v
  float n_hi, n_lo;
  two_sum(-az, fmaf(ax, gx, ay * gy), n_hi, n_lo);
  n_lo += fmaf(lx, gx, fmaf(ly, gy, -lz));
  // v.v = 1 + q, q = gx^2 + gy^2 with the products' errors
  const float p1 = gx * gx, e1 = fmaf(gx, gx, -p1);
  const float p2 = gy * gy, e2 = fmaf(gy, gy, -p2);
  float q, eq;
  two_sum(p1, p2, q, eq);
  float d_hi, d_lo;
  two_sum(1.f, q, d_hi, d_lo);
  d_lo += eq + (e1 + e2);
  // k = 2 (a.v) / (v.v) as a float-float pair; the correction term cancels
  // the approximate reciprocal's error to second order
  const float inv = __fdividef(1.f, d_hi);
  const float q_hi = n_hi * inv;
  const float rem = (fmaf(-q_hi, d_hi, n_hi) + n_lo) - q_hi * d_lo;
  const float k_hi = 2.f * q_hi, k_lo = 2.f * (rem * inv);
  // b = a - k v: x and y subtract k g, z adds k
  float s, e;
  {
    const float p = k_hi * gx, pe = fmaf(k_hi, gx, -p);
    two_sum(ax, -p, s, e);
    ax = s;
    lx = e + (lx - pe - k_lo * gx);
  }
  {
    const float p = k_hi * gy, pe = fmaf(k_hi, gy, -p);
    two_sum(ay, -p, s, e);
    ay = s;
    ly = e + (ly - pe - k_lo * gy);
  }
  two_sum(az, k_hi, s, e);
  az = s;
  lz = e + (lz + k_lo);
  normalize3(ax, ay, az, lx, ly, lz);
}

// ---------------------------------------------------------------- rulings

// Spacing vector kappa (length d, along the ruling-plane normal).
//   constant     optika/rulings/_spacing.py:69-74
//   polynomial   optika/rulings/_spacing.py:109-128
//   holographic  optika/rulings/_spacing.py:295-328
__device__ __forceinline__ void ruling_kappa(int rule_type, const otx_surface& s, float x,
                                             float y, float z, float nx,
                                             float ny, float nz, float& kx,
                                             float& ky, float& kz) {
  switch (rule_type) {
    case OTX_RULE_CONSTANT: {
      const float d = s.rule_coef[0];
      kx = d * s.rule_normal[0];
      ky = d * s.rule_normal[1];
      kz = d * s.rule_normal[2];
      return;
    }
    case OTX_RULE_POLY1D: {
      float px = x, py = y, pz = z;
      affine_point_folded(s.rule_xform, px, py, pz);
      const float xs = fmaf(px, s.rule_normal[0],
                            fmaf(py, s.rule_normal[1], pz * s.rule_normal[2]));
      float d = 0.f;  // Horner over the dense coefficient table
      const int nt = min(max(s.rule_num_terms, 0), OTX_MAX_POLY_TERMS);
      for (int k = nt - 1; k >= 0; --k) d = fmaf(d, xs, s.rule_coef[k]);
      kx = d * s.rule_normal[0];
      ky = d * s.rule_normal[1];
      kz = d * s.rule_normal[2];
      return;
    }
    case OTX_RULE_HOLOGRAPHIC: {
      float r1x = x - s.holo_x1[0], r1y = y - s.holo_x1[1], r1z = z - s.holo_x1[2];
      float r2x = x - s.holo_x2[0], r2y = y - s.holo_x2[1], r2z = z - s.holo_x2[2];
      const float i1 = s.holo_d1 * rsqrtf(r1x * r1x + r1y * r1y + r1z * r1z);
      const float i2 = s.holo_d2 * rsqrtf(r2x * r2x + r2y * r2y + r2z * r2z);
      const float drx = r1x * i1 - r2x * i2;
      const float dry = r1y * i1 - r2y * i2;
      const float drz = r1z * i1 - r2z * i2;
      // aq = n x dr ; a = |aq| ; q = aq / a ; d = lambda / a ; kappa = d q x n
      const float aqx = ny * drz - nz * dry;
      const float aqy = nz * drx - nx * drz;
      const float aqz = nx * dry - ny * drx;
      const float a2 = aqx * aqx + aqy * aqy + aqz * aqz;
      const float sc = s.holo_wavelength / a2;  // (lambda / a) / a
      kx = sc * (aqy * nz - aqz * ny);
      ky = sc * (aqz * nx - aqx * nz);
      kz = sc * (aqx * ny - aqy * nx);
      return;
    }
    default:
      kx = ky = kz = 0.f;
      return;
  }
}

// Effective incident direction, optika/rulings/_rulings.py:124-126:
//   a + sign(a.n) m lambda g / (n d),  g = kappa / d.
__device__ __forceinline__ void incident_effective(int rule_type, const otx_surface& s,
                                                   Ray& r, float nx, float ny,
                                                   float nz) {
  float kx, ky, kz;
  ruling_kappa(rule_type, s, r.px, r.py, r.pz, nx, ny, nz, kx, ky, kz);
  const float d2 = kx * kx + ky * ky + kz * kz;
  const float an = r.dx * nx + r.dy * ny + r.dz * nz;
  const float w_mm = r.wl * 1e-6f;
  const float f = sgnf(an) * s.rule_order * w_mm / (r.n * d2);
  r.dx = fmaf(f, kx, r.dx);
  r.dy = fmaf(f, ky, r.dy);
  r.dz = fmaf(f, kz, r.dz);
}

// Bessel function of the first kind J_m(x) for an integer order m (any
// sign) and a real argument of any sign, from CUDA's jnf of order |m| at
// |x|: J_-m(x) = (-1)^m J_m(x) and J_m(-x) = (-1)^m J_m(x).
__device__ __forceinline__ float bessel_j(float order, float x) {
  const int m = (int)order;
  const int am = m < 0 ? -m : m;
  float j = jnf(am, fabsf(x));
  if ((am & 1) && ((m < 0) != (x < 0.f))) j = -j;
  return j;
}

// Python's i % 2 == 0 for a float order (floored modulo).
__device__ __forceinline__ bool order_even(float m) {
  return m - 2.f * floorf(0.5f * m) == 0.f;
}

// numpy.interp of the second column of a [x(n), y(n), -] table (clamped to
// the end values outside the table).
__device__ __forceinline__ float table_interp(const otx_system& sys, int table, float x) {
  const otx_table T = sys.tables[table];
  const float* xs = reinterpret_cast<const float*>(sys.table_data) + T.offset;
  const float* ys = xs + T.count;
  const int cnt = T.count;
  if (!(x > xs[0])) return ys[0];
  if (!(x < xs[cnt - 1])) return ys[cnt - 1];
  int lo = 0, hi = cnt - 1;  // xs[lo] < x < xs[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xs[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  const float w = (x - xs[lo]) / (xs[hi] - xs[lo]);
  return fmaf(w, ys[hi] - ys[lo], ys[lo]);
}

// table_interp behind the checks of the table index the host also makes
// (NaN for an unusable table).
__device__ __forceinline__ float table_value(const otx_system& sys, int table, float x) {
  if (table < 0 || table >= OTX_MAX_STACKS * 4 || sys.tables[table].count < 1 ||
      sys.table_data == 0)
    return NAN;
  return table_interp(sys, table, x);
}

// Groove efficiency of the ruling models, on the rays after
// incident_effective (optika/surfaces.py:182-184) at the intercept point
// (px, py, pz) with effective direction a = (dx, dy, dz) and sag normal n:
//   measured     optika/rulings/_rulings.py:287-314 (interp on wavelength)
//   sinusoidal   :404-457   J_m(2 gamma)
//   square       :548-614   cos^2(pi g / 2) (m = 0), 0 (m even),
//                           (2 sin(pi g / 2) / (m pi))^2 (m odd)
//   sawtooth     :705-758   (sin(pi g) / (pi (g + m)))^2
//   triangular   :849-911   (g / ((pi g / 2)^2 + m^2))^2 times
//                           sin^2 (m even) or cos^2 (m odd) of pi^2 g / 4
//   rectangular  :1008-1073 b = sin^2(pi g / sqrt(2 (1 - cos a))),
//                           1 - (2 a / pi - (a / pi)^2) b (m = 0),
//                           2 (1 - cos(m a)) b / (m pi)^2 otherwise
// with, as in the reference, q = normalize(n x kappa), s = a.q,
// cos_theta = -(a - s).n where the scalar s is subtracted from every
// component of a, and g = pi depth / (lambda cos_theta), depth being the
// groove depth over the model's amplitude (folded in by the host).
static __device__ __noinline__ float ruling_efficiency_call(const otx_system& sys,
                                                            const otx_surface& s, int rule_type,
                                                            float px, float py, float pz,
                                                            float dx, float dy, float dz,
                                                            float wl, float nx, float ny,
                                                            float nz) {
  const int model = s.rule_eff_type;
  if (model == OTX_RULE_EFF_MEASURED) return table_value(sys, s.rule_table, wl);
  float kx, ky, kz;
  ruling_kappa(rule_type, s, px, py, pz, nx, ny, nz, kx, ky, kz);
  float qx = ny * kz - nz * ky;
  float qy = nz * kx - nx * kz;
  float qz = nx * ky - ny * kx;
  const float qi = 1.f / sqrtf(qx * qx + qy * qy + qz * qz);
  qx *= qi;
  qy *= qi;
  qz *= qi;
  const float sp = dx * qx + dy * qy + dz * qz;
  const float cos_t = -((dx - sp) * nx + (dy - sp) * ny + (dz - sp) * nz);
  const float pi = 3.14159265358979f;
  const float g = pi * s.rule_depth / (wl * cos_t);
  const float m = s.rule_order;
  switch (model) {
    case OTX_RULE_EFF_SINUSOIDAL:
      return bessel_j(m, 2.f * g);
    // sin(pi x) and cos(pi x) as sinpif / cospif: no rounding of pi x
    case OTX_RULE_EFF_SQUARE: {
      if (m == 0.f) {
        const float c = cospif(0.5f * g);
        return c * c;
      }
      if (order_even(m)) return 0.f;
      const float v = 2.f * sinpif(0.5f * g) / (m * pi);
      return v * v;
    }
    case OTX_RULE_EFF_SAWTOOTH: {
      const float u = g + m;
      float v;
      if (m == rintf(m)) {
        // sin(pi g) = (-1)^m sin(pi u): sinc^2(u), well conditioned near
        // the blaze u -> 0 where the quotient tends to 1
        v = (u == 0.f) ? 1.f : sinpif(u) / (pi * u);
      } else {
        v = sinpif(g) / (pi * u);
      }
      return v * v;
    }
    case OTX_RULE_EFF_TRIANGULAR: {
      const float h = 0.5f * pi * g;
      const float a = g / fmaf(h, h, m * m);
      const float ph = 0.25f * pi * g;  // (pi^2 g / 4) / pi
      const float v = a * (order_even(m) ? sinpif(ph) : cospif(ph));
      return v * v;
    }
    case OTX_RULE_EFF_RECTANGULAR: {
      const float a = s.rule_duty;
      const float b0 = sinpif(g / sqrtf(2.f * (1.f - cosf(a))));
      const float b = b0 * b0;
      if (m == 0.f) return 1.f - (2.f * a / pi - (a / pi) * (a / pi)) * b;
      const float mp = m * pi;
      return 2.f / (mp * mp) * (1.f - cosf(m * a)) * b;
    }
    default:
      return s.rule_efficiency;
  }
}

// ---------------------------------------------------------------- apertures

// optika/apertures/_apertures.py: circular :292-314, sector :438-480,
// elliptical :640-663, polygonal :739-778, rectangular :941-968.
// Comparisons are inclusive (<=) as in the reference; NaN coordinates test
// false before inversion.
__device__ __forceinline__ bool aperture_inside(int aper_type, const otx_system& sys,
                                                const otx_surface& s, float x,
                                                float y, float z) {
  const int flags = s.aper_flags;
  if (!(flags & OTX_APER_FLAG_ACTIVE)) return true;
  if (flags & OTX_APER_FLAG_TRANSFORM) affine_point_folded(s.aper_to_local, x, y, z);
  bool m;
  switch (aper_type) {
    case OTX_APER_CIRCULAR:
      m = sqrtf(fmaf(x, x, y * y)) <= s.aper_p[0];
      break;
    case OTX_APER_RECTANGULAR:
      m = (-s.aper_p[0] <= x) && (x <= s.aper_p[0]) && (-s.aper_p[1] <= y) &&
          (y <= s.aper_p[1]);
      break;
    case OTX_APER_ELLIPTICAL: {
      const float a = x / s.aper_p[0], b = y / s.aper_p[1];
      m = (a * a + b * b) <= 1.f;
      break;
    }
    case OTX_APER_SECTOR: {
      const bool mr = sqrtf(fmaf(x, x, y * y)) <= s.aper_p[0];
      const float ang = atan2f(y, x);
      const float twopi = 6.283185307179586f;
      const float ap = (ang < 0.f) ? ang + twopi : ang;
      const float an = (ang > 0.f) ? ang - twopi : ang;
      const float a0 = s.aper_p[1], a1 = s.aper_p[2];
      const bool ma = ((a0 < ap) && (ap < a1)) || ((a0 < an) && (an < a1));
      m = mr && ma;
      break;
    }
    case OTX_APER_POLYGON: {
      // even-odd crossing test over the vertex loop
      bool inside = false;
      const int b = s.aper_vertex_begin;
      const int cnt = (b >= 0 && s.aper_vertex_count >= 3 &&
                       b + s.aper_vertex_count <= OTX_MAX_VERTICES)
                          ? s.aper_vertex_count
                          : 0;
      for (int i = 0, j = cnt - 1; i < cnt; j = i++) {
        const float xi = sys.vertices[2 * (b + i)], yi = sys.vertices[2 * (b + i) + 1];
        const float xj = sys.vertices[2 * (b + j)], yj = sys.vertices[2 * (b + j) + 1];
        if (((yi > y) != (yj > y)) && (x < (xj - xi) * (y - yi) / (yj - yi) + xi))
          inside = !inside;
      }
      m = inside;
      break;
    }
    default:
      m = true;
      break;
  }
  if (flags & OTX_APER_FLAG_INVERTED) m = !m;
  return m;
}

// ---------------------------------------------------------------- complex

struct cf {
  float re, im;
};
__device__ __forceinline__ cf cadd(cf a, cf b) { return cf{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf csub(cf a, cf b) { return cf{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cf cmul(cf a, cf b) {
  return cf{fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re)};
}
__device__ __forceinline__ cf cscale(cf a, float s) { return cf{a.re * s, a.im * s}; }
__device__ __forceinline__ cf cconj(cf a) { return cf{a.re, -a.im}; }
__device__ __forceinline__ float cabs2(cf a) { return fmaf(a.re, a.re, a.im * a.im); }
// a / b for b of moderate magnitude (indices, cosines): conj(b) / |b|^2.
__device__ __forceinline__ cf cdiv(cf a, cf b) {
  return cscale(cmul(a, cconj(b)), 1.f / cabs2(b));
}
// Principal square root (branch cut on the negative real axis, as numpy),
// for arguments of moderate magnitude.
__device__ __forceinline__ cf csqrt(cf z) {
  const float m = sqrtf(cabs2(z));
  const float h = 0.5f * (m + fabsf(z.re));
  if (h == 0.f) return cf{0.f, z.im};
  const float rs = rsqrtf(h);
  const float t = h * rs;                   // sqrt(h)
  const float u = 0.5f * fabsf(z.im) * rs;  // |im| / (2 sqrt(h))
  if (z.re >= 0.f) return cf{t, copysignf(u, z.im)};
  return cf{u, copysignf(t, z.im)};
}

struct cm2 {
  cf a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ cm2 cm_mul(const cm2& x, const cm2& y) {
  return cm2{cadd(cmul(x.a, y.a), cmul(x.b, y.c)), cadd(cmul(x.a, y.b), cmul(x.b, y.d)),
             cadd(cmul(x.c, y.a), cmul(x.d, y.c)), cadd(cmul(x.c, y.b), cmul(x.d, y.d))};
}

// Exact power-of-two rescaling of a transfer matrix so that its largest
// component is O(1); the exponent is accumulated separately.
__device__ __forceinline__ void cm_normalize(cm2& m, int& exp2) {
  const float mx = fmaxf(fmaxf(fmaxf(fabsf(m.a.re), fabsf(m.a.im)),
                               fmaxf(fabsf(m.b.re), fabsf(m.b.im))),
                         fmaxf(fmaxf(fabsf(m.c.re), fabsf(m.c.im)),
                               fmaxf(fabsf(m.d.re), fabsf(m.d.im))));
  if (!(mx > 0.f) || !isfinite(mx)) return;
  const int e = ilogbf(mx);
  const float s = ldexpf(1.f, -e);
  m.a = cscale(m.a, s);
  m.b = cscale(m.b, s);
  m.c = cscale(m.c, s);
  m.d = cscale(m.d, s);
  exp2 += e;
}

// Complex index of a layer at a vacuum wavelength (nm).  FAST takes the
// interpolation weight from an approximate quotient (2 ulp).
template <bool FAST = false>
__device__ __forceinline__ cf layer_n(const otx_system& sys, const otx_layer& L,
                                      float wl) {
  if (L.table < 0) return cf{L.n_re, L.n_im};
  const otx_table T = sys.tables[L.table];
  const float* base = reinterpret_cast<const float*>(sys.table_data) + T.offset;
  const float* xs = base;
  const float* ns = base + T.count;
  const float* ks = base + 2 * T.count;
  const int cnt = T.count;
  if (!(wl > xs[0])) return cf{ns[0], ks[0]};
  if (!(wl < xs[cnt - 1])) return cf{ns[cnt - 1], ks[cnt - 1]};
  int lo = 0, hi = cnt - 1;  // xs[lo] < wl < xs[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xs[mid] <= wl)
      lo = mid;
    else
      hi = mid;
  }
  const float w = FAST ? __fdividef(wl - xs[lo], xs[hi] - xs[lo])
                       : (wl - xs[lo]) / (xs[hi] - xs[lo]);
  return cf{fmaf(w, ns[hi] - ns[lo], ns[lo]), fmaf(w, ks[hi] - ks[lo], ks[lo])};
}

// Fourier transform of the derivative of an interface profile at the
// wavenumber s (1/nm), the factor on r_ij (Stearns 1989):
//   erf          exp(-(s w)^2 / 2)             optika/materials/profiles.py:221-223
//   exponential  1 / (1 + (s w)^2 / 2)                                    :320-326
//   linear       sin(x) / x, x = sqrt(3) w s                              :424-431
//   sinusoidal   pi (sin(x - pi/2) / (x - pi/2) + sin(x + pi/2) / (x + pi/2)) / 4,
//                x = a w s, a = pi / (pi^2 - 8)                          :532-541
__device__ __forceinline__ float interface_factor(int type, float width, float s) {
  switch (type) {
    case OTX_PROFILE_ERF: {
      const float x = s * width;
      return expf(-0.5f * x * x);
    }
    case OTX_PROFILE_EXPONENTIAL: {
      const float x = s * width;
      return 1.f / fmaf(0.5f * x, x, 1.f);
    }
    case OTX_PROFILE_LINEAR: {
      const float x = 1.7320508075688772f * width * s;
      return sinf(x) / x;
    }
    case OTX_PROFILE_SINUSOIDAL: {
      const float pi = 3.14159265358979f;
      const float x = (pi / (pi * pi - 8.f)) * width * s;
      const float x1 = x - 0.5f * pi, x2 = x + 0.5f * pi;
      return 0.25f * pi * (sinf(x1) / x1 + sinf(x2) / x2);
    }
    default:
      return 1.f;
  }
}

// Running state of the transfer-matrix product for one polarisation.
//
// The reference's refraction matrix W = [[1, r], [r, 1]] / t
// (optika/materials/matrices.py:127-161) equals W' / (2 q_i) with
// W' = [[q_i + q_j, q_i - q_j], [q_i - q_j, q_i + q_j]].  The state keeps
// the product of the W' (times the propagation matrices U) and, when
// transmission is wanted, the product of |2 q_i|^2 separately:
// r = M21 / M11 is unchanged and |t|^2 = prod |2 q_i|^2 / |M'11|^2, so no
// complex division is needed.  Both products carry power-of-two exponents.
// q is n cos for s and conj(cos) / n = conj(n cos) / |n|^2 for p.
struct MLState {
  cm2 m;      // unnormalised product
  int e;      // its exponent
  bool first; // product still the identity
  float t;    // prod |2 q_i|^2 mantissa
  int te;     // and its exponent
  cf q;       // q of the current medium
  cf n;       // index of the current medium
  cf inv0;    // (n0 sin0)^2, Snell invariant
  bool where;
};

// q of the medium of index nj, from the Snell invariant:
// cos_j = sqrt(1 - (n0 sin0)^2 / n_j^2) equals the reference's chained
// optika/materials/_snells_law.py:13-38.
template <bool FAST = false>
__device__ __forceinline__ cf medium_q(const cf& inv0, const cf& nj, bool pol_p) {
  const cf nj2 = cmul(nj, nj);
  const float r = FAST ? __fdividef(1.f, cabs2(nj2)) : 1.f / cabs2(nj2);
  const cf ratio = cscale(cmul(inv0, cconj(nj2)), r);
  const cf cj = csqrt(cf{1.f - ratio.re, -ratio.im});
  const cf w = cmul(nj, cj);
  return pol_p ? cscale(cconj(w), 1.f / cabs2(nj)) : w;
}

__device__ __forceinline__ void ml_times(MLState& st, const cm2& t, int te) {
  if (st.first) {
    st.m = t;
    st.e = te;
    st.first = false;
  } else {
    st.m = cm_mul(st.m, t);
    st.e += te;
  }
  cm_normalize(st.m, st.e);
}

// Wavenumber of an interface profile's factor from the incident medium
// (optika/materials/profiles.py:103-128): s = Re(4 pi n_i d_i / lambda) with
// d_i = cos_i for s and conj(cos_i) for p, i.e. 4 pi Re(q) / lambda for s
// and 4 pi Re(q n_i^2) / lambda for p (q = conj(n cos) / |n|^2).
__device__ __forceinline__ float interface_wavenumber(const cf& q, const cf& n, float wl,
                                                      bool pol_p) {
  const float re = pol_p ? cmul(q, cmul(n, n)).re : q.re;
  return 12.566370614359172f * re / wl;
}

// Multiply the running product by one layer's W' (and its propagation U),
// optika/materials/_layers.py:229-277; thickness 0 is the substrate.  An
// interface profile on the layer's left side scales r_ij, i.e. the
// off-diagonal q_i - q_j of W' (optika/materials/matrices.py:147-152).
template <bool NEED_T>
__device__ __forceinline__ void layer_step(MLState& st, cf nj, float thickness, float wl,
                                           bool pol_p, int iface = OTX_PROFILE_NONE,
                                           float iface_width = 0.f) {
  const cf qj = medium_q(st.inv0, nj, pol_p);
  const cf a = cadd(st.q, qj);
  cf b = csub(st.q, qj);
  if (iface != OTX_PROFILE_NONE)
    b = cscale(b, interface_factor(iface, iface_width,
                                   interface_wavenumber(st.q, st.n, wl, pol_p)));
  // U = diag(exp(-i beta), exp(i beta)), beta = 2 pi h n cos / lambda
  bool wprop = true;
  cm2 tm = cm2{a, b, b, a};
  if (thickness != 0.f) {
    const cf ncos = pol_p ? cscale(cconj(qj), cabs2(nj)) : qj;  // n cos
    const cf beta = cscale(ncos, 6.283185307179586f * thickness / wl);
    float sn, cs;
    sincosf(beta.re, &sn, &cs);
    const float g = expf(beta.im);  // |exp(-i beta)|
    wprop = g < 1e10f;
    if (wprop) {
      const cf em{g * cs, -g * sn};
      const float gi = 1.f / g;
      const cf ep{gi * cs, gi * sn};
      tm = cm2{cmul(a, em), cmul(b, ep), cmul(b, em), cmul(a, ep)};
    }
  }
  if (st.where) {
    ml_times(st, tm, 0);
    if (NEED_T) {
      int e;
      st.t = frexpf(st.t * 4.f * cabs2(st.q), &e);
      st.te += e;
    }
  }
  st.where = st.where && wprop;
  st.q = qj;
  st.n = nj;
}

__device__ __forceinline__ void cm_pow(cm2 base, int bexp, int e, cm2& acc, int& aexp) {
  bool first = true;
  while (e > 0) {
    if (e & 1) {
      if (first) {
        acc = base;
        aexp = bexp;
        first = false;
      } else {
        acc = cm_mul(acc, base);
        aexp += bexp;
        cm_normalize(acc, aexp);
      }
    }
    e >>= 1;
    if (e) {
      base = cm_mul(base, base);
      bexp *= 2;
      cm_normalize(base, bexp);
    }
  }
}

template <bool NEED_T>
__device__ __forceinline__ void run_layers(MLState& st, const otx_system& sys, int begin,
                                           int count, float wl, bool pol_p) {
  for (int i = 0; i < count; ++i) {
    const otx_layer& L = sys.layers[begin + i];
    layer_step<NEED_T>(st, layer_n(sys, L, wl), L.thickness, wl, pol_p, L.interface_type,
                       L.interface_width);
  }
}

// Reflectivity and transmissivity of one polarisation of a stack,
// optika/materials/_multilayers.py:187-237 (coefficients) and :485-532
// (R = |r|^2, T = |t|^2 Re(q_sub / q_amb)).  A periodic block is its first
// period times the period matrix to the power num_periods - 1
// (optika/materials/_layers.py:611-645), by repeated squaring.
template <bool NEED_T>
__device__ __forceinline__ void multilayer_pol(const otx_system& sys, const otx_stack& K,
                                               float wl, float cos0, cf n0, bool pol_p,
                                               float& R, float& T) {
  MLState st;
  st.e = 0;
  st.first = true;
  st.t = 1.f;
  st.te = 0;
  st.inv0 = cscale(cmul(n0, n0), fmaf(-cos0, cos0, 1.f));
  st.q = pol_p ? cscale(cconj(n0), cos0 / cabs2(n0)) : cscale(n0, cos0);
  st.n = n0;
  const cf q0 = st.q;
  st.where = true;
  run_layers<NEED_T>(st, sys, K.pre_begin, K.pre_count, wl, pol_p);
  if (K.per_count > 0 && K.num_periods > 0) {
    // first period from the current medium
    run_layers<NEED_T>(st, sys, K.per_begin, K.per_count, wl, pol_p);
    // one period from the period's own last medium, to num_periods - 1
    MLState per = st;
    per.first = true;
    per.e = 0;
    per.t = 1.f;
    per.te = 0;
    run_layers<NEED_T>(per, sys, K.per_begin, K.per_count, wl, pol_p);
    const int reps = K.num_periods - 1;
    if (!per.first && reps > 0) {
      cm2 pm;
      int pe = 0;
      cm_pow(per.m, per.e, reps, pm, pe);
      ml_times(st, pm, pe);
      if (NEED_T) {
        for (int i = 0; i < reps; ++i) {
          int e;
          st.t = frexpf(st.t * per.t, &e);
          st.te += per.te + e;
        }
      }
    }
    st.where = per.where;
    st.q = per.q;
    st.n = per.n;
  }
  run_layers<NEED_T>(st, sys, K.post_begin, K.post_count, wl, pol_p);
  cf nsub{1.f, 0.f};
  int sub_iface = OTX_PROFILE_NONE;
  float sub_width = 0.f;
  if (K.substrate >= 0) {
    const otx_layer& L = sys.layers[K.substrate];
    nsub = layer_n(sys, L, wl);
    sub_iface = L.interface_type;
    sub_width = L.interface_width;
  }
  layer_step<NEED_T>(st, nsub, 0.f, wl, pol_p, sub_iface, sub_width);
  // R = |M21|^2 / |M11|^2 (exponents cancel)
  const float m11 = cabs2(st.m.a);
  R = cabs2(st.m.c) / m11;
  T = 0.f;
  if (NEED_T && st.where) {
    // |t|^2 = prod |2q|^2 / |M'11|^2 ; T = |t|^2 Re(q_sub / q_amb)
    T = ldexpf(st.t / m11, st.te - 2 * st.e) * cdiv(st.q, q0).re;
  }
}

// Both polarisations, for the standalone multilayer kernel.
__device__ __forceinline__ void multilayer(const otx_system& sys, const otx_stack& K,
                                           float wl, float cos0, cf n0, float& Rs,
                                           float& Rp, float& Ts, float& Tp) {
  multilayer_pol<true>(sys, K, wl, cos0, n0, false, Rs, Ts);
  multilayer_pol<true>(sys, K, wl, cos0, n0, true, Rp, Tp);
}

__device__ __forceinline__ bool stack_has_layers(const otx_stack& K) {
  return K.pre_count > 0 || (K.per_count > 0 && K.num_periods > 0) || K.post_count > 0;
}

// Substrate-only stack with a smooth substrate (a bare coating, or a film of
// no layers): the multilayer product reduces to one interface, r = (q0 - q1) / (q0 + q1),
// t = 2 q0 / (q0 + q1); returns the s/p average of R (mirror) or T.
//
// For a mirror both polarisations share n1 cos1 = n1 sqrt(1 - (n0 sin0)^2 /
// n1^2) (one complex square root): with q0 = n0 cos0 and w = n1 cos1,
//   R_s = |q0 - w|^2 / |q0 + w|^2,
//   R_p = |q0 |n1|^2 - w |n0|^2|^2 / |q0 |n1|^2 + w |n0|^2|^2
// (the p admittances conj(n cos) / |n|^2 scaled by |n0|^2 |n1|^2 and
// conjugated), and the average (R_s + R_p) / 2 takes one division.
__device__ __forceinline__ float fresnel_efficiency(const otx_system& sys, const otx_stack& K,
                                                    bool mirror, float wl, float cos0, cf n0) {
  cf n1{1.f, 0.f};
  if (K.substrate >= 0) n1 = mirror ? layer_n<true>(sys, sys.layers[K.substrate], wl)
                                    : layer_n(sys, sys.layers[K.substrate], wl);
  const cf inv0 = cscale(cmul(n0, n0), fmaf(-cos0, cos0, 1.f));
  if (mirror) {
    // approximate quotients: R is wanted to ~1e-6, each adds ~2e-7
    const cf w = medium_q<true>(inv0, n1, false);
    const cf q0 = cscale(n0, cos0);
    const float ns = cabs2(csub(q0, w)), ds = cabs2(cadd(q0, w));
    const cf a = cscale(q0, cabs2(n1)), b = cscale(w, cabs2(n0));
    const float np = cabs2(csub(a, b)), dp = cabs2(cadd(a, b));
    const float den = ds * dp;
    if (den > 1e-30f && den < 1e30f) return 0.5f * __fdividef(fmaf(ns, dp, np * ds), den);
    return 0.5f * (ns / ds + np / dp);
  }
  float acc = 0.f;
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const bool pol_p = p == 1;
    const cf q0 = pol_p ? cscale(cconj(n0), cos0 / cabs2(n0)) : cscale(n0, cos0);
    const cf q1 = medium_q(inv0, n1, pol_p);
    const float den = cabs2(cadd(q0, q1));
    acc += 4.f * cabs2(q0) / den * cdiv(q1, q0).re;
  }
  return 0.5f * acc;
}

// Out-of-line efficiency of a layered stack for the trace kernel (systems
// without layered coatings never call it): the s/p average of R or T.
static __device__ __noinline__ float multilayer_efficiency_call(const otx_system& sys,
                                                                int stack, bool mirror,
                                                                float wl, float cos0,
                                                                float n_re, float n_im) {
  const otx_stack& K = sys.stacks[stack];
  float acc = 0.f;
  for (int p = 0; p < 2; ++p) {
    float R, T;
    if (mirror) {
      multilayer_pol<false>(sys, K, wl, cos0, cf{n_re, n_im}, p == 1, R, T);
      acc += R;
    } else {
      multilayer_pol<true>(sys, K, wl, cos0, cf{n_re, n_im}, p == 1, R, T);
      acc += T;
    }
  }
  return 0.5f * acc;
}

// ---------------------------------------------------------------- surface

// Compile-time description of one surface: each tag is an OTX_* type, or
// -1 to read the type from the descriptor at run time.  MAT may also be
// OTX_MAT_FRESNEL_MIRROR: a multilayer mirror whose stack is a bare
// substrate.
#define OTX_MAT_FRESNEL_MIRROR 100
template <int SAG, int MAT, int APER, int RULE>
struct Kind {
  static constexpr int sag = SAG, mat = MAT, aper = APER, rule = RULE;
};
using AnyKind = Kind<-1, -1, -1, -1>;

// One surface of optika/surfaces.py:123-198 for a ray already expressed in
// the previous frame.  Returns with the ray in this surface's frame.  ML
// selects the variant that can evaluate layered multilayer stacks (chosen
// by the host when the system has one).
template <class K, bool ML>
__device__ __forceinline__ void propagate_surface(const otx_system& sys,
                                                  const otx_surface& s,
                                                  Ray& r) {
  const int sag_type = K::sag >= 0 ? K::sag : s.sag_type;
  const int mat_type = K::mat >= 0 ? K::mat : s.mat_type;
  const int aper_type = K::aper >= 0 ? K::aper : s.aper_type;
  const int rule_type = K::rule >= 0 ? K::rule : s.rule_type;

  // transformation.inverse (surfaces.py:141-142), float-float translation
  // and compensated rotation
  float lo[3];
  frame_change(s.to_local, r, lo);
  const float ox = r.px, oy = r.py, oz = r.pz;

  // sag.propagate_rays (sags/_abc.py:109-122)
  float x, y, z, tl;
  const float t = intercept(sag_type, s, sys.newton_iterations, ox, oy, oz, lo, r.dx,
                            r.dy, r.dz, r.lx, r.ly, r.lz, x, y, z, tl);
  r.px = x;
  r.py = y;
  r.pz = z;
  if (r.att != 0.f) {
    const float len = fabsf(t) * sqrtf(r.dx * r.dx + r.dy * r.dy + r.dz * r.dz);
    r.inten *= expf(-r.att * len);
  }
  // (t + tl) is the segment's geometric length: directions are unit to
  // float-float accuracy (unit_ff at their creation and after refraction;
  // rotations and reflections preserve the norm).
  opl_add(r, r.n, t, tl);

  float nx, ny, nz, v[3];
  normal(sag_type, s, x, y, nx, ny, nz, v);

  if (rule_type != OTX_RULE_NONE) incident_effective(rule_type, s, r, nx, ny, nz);

  // material (surfaces.py:160-181)
  const float n1 = r.n;
  float n2 = n1;
  float att2 = r.att;
  float eff = 1.f;
  bool mirror = false;
  switch (mat_type) {
    case OTX_MAT_VACUUM:
      n2 = 1.f;
      att2 = 0.f;
      break;
    case OTX_MAT_MIRROR:
      mirror = true;
      break;
    case OTX_MAT_MEASURED_MIRROR:
      // optika/materials/_materials.py:279-306: reflectivity interpolated in
      // the wavelength of the incident rays; n and attenuation unchanged
      mirror = true;
      eff = table_value(sys, s.mat_table, r.wl);
      break;
    case OTX_MAT_GLASS: {
      // Sellmeier, optika/materials/_materials.py:428-438
      const float w2 = r.wl * r.wl;
      float s2 = 1.f;
      for (int i = 0; i < 3; ++i) s2 += s.sellmeier_b[i] * w2 / (w2 - s.sellmeier_c[i]);
      n2 = sqrtf(s2);
      att2 = 0.f;
      break;
    }
    case OTX_MAT_FRESNEL_MIRROR:
    case OTX_MAT_MULTILAYER_MIRROR:
    case OTX_MAT_MULTILAYER_FILM: {
      mirror = (mat_type != OTX_MAT_MULTILAYER_FILM);
      // n = n_ray + i att lambda / (4 pi), cos = -a.n (_multilayers.py:924-932)
      const float k = r.att * (r.wl * 1e-6f) * 0.07957747154594767f;
      const float cos0 = -(r.dx * nx + r.dy * ny + r.dz * nz);
      const int ks = min(max(s.mat_stack, 0), OTX_MAX_STACKS - 1);
      const otx_stack& K2 = sys.stacks[ks];
      if (mat_type != OTX_MAT_FRESNEL_MIRROR && ML && stack_needs_product(sys, K2))
        eff = multilayer_efficiency_call(sys, ks, mirror, r.wl, cos0, n1, k);
      else
        eff = fresnel_efficiency(sys, K2, mirror, r.wl, cos0, cf{n1, k});
      break;
    }
    default:
      break;
  }
  if (rule_type != OTX_RULE_NONE)
    eff *= (s.rule_eff_type == OTX_RULE_EFF_IDEAL)
               ? s.rule_efficiency
               : ruling_efficiency_call(sys, s, rule_type, r.px, r.py, r.pz, r.dx, r.dy, r.dz,
                                        r.wl, nx, ny, nz);
  // wavelength_2 = wavelength_1 / (n1 / n2)   (surfaces.py:162-165)
  if (n2 != n1) r.wl = r.wl / (n1 / n2);
  const bool unit_mirror =
      mirror && rule_type == OTX_RULE_NONE &&
      fabsf(fmaf(r.dx, r.dx, fmaf(r.dy, r.dy, fmaf(r.dz, r.dz, -1.f)))) < 1e-6f;
  if (unit_mirror && sag_type == OTX_SAG_FLAT) {
    // the flat's normal is exactly (0, 0, -1): Snell's mirror case reduces
    // to negating the z component (the same values, without the dot product)
    r.dz = -r.dz;
    r.lz = -r.lz;
  } else if (unit_mirror && (sag_type == OTX_SAG_CONIC || sag_type == OTX_SAG_PARABOLA ||
                             sag_type == OTX_SAG_TOROID)) {
    reflect_gradient(r.dx, r.dy, r.dz, r.lx, r.ly, r.lz, v[0], v[1]);
  } else if (unit_mirror) {
    reflect_curved(r.dx, r.dy, r.dz, r.lx, r.ly, r.lz, v);
  } else {
    snell(r.dx, r.dy, r.dz, r.lx, r.ly, r.lz, n1, n2, mirror, nx, ny, nz);
  }
  r.inten *= eff;
  r.att = att2;
  r.n = n2;

  // aperture.clip_rays (apertures/_apertures.py:82-102)
  if (aper_type != OTX_APER_NONE) {
    const bool on_dir = (s.aper_flags & OTX_APER_FLAG_DIRECTION) != 0;
    const bool m = on_dir ? aperture_inside(aper_type, sys, s, r.dx, r.dy, r.dz)
                          : aperture_inside(aper_type, sys, s, r.px, r.py, r.pz);
    r.ok = r.ok && m;
  }
}

}  // namespace otx
