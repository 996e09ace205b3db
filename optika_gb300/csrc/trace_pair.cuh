// Two rays per thread on packed FP32 instructions.
//
// GB300 issues an FP32 add, multiply or fused multiply-add on a pair of
// values (add/mul/fma.rn.f32x2) as one instruction.  The shape-specialised
// trace is bound by instruction issue, so this variant carries two rays per
// thread in float2 registers and runs the arithmetic of the Newtonian
// telescope's surface kinds (flat and conic sags; vacuum, mirror and
// bare-coating Fresnel mirror materials; any aperture; no rulings) on both
// at once.  Square roots, quotients, table lookups, aperture tests, stores
// and binning stay per lane and call the scalar device functions; so do the
// paths that are rare here (rotations about other axes than y, directions
// off unit length, attenuating media), which fall back to the scalar step
// for each lane.  Each packed step performs, lane by lane, the same
// rounded operations as its scalar counterpart in trace_device.cuh, up to
// the contraction the compiler applies to the scalar source, so the two
// kernels agree to FP32 rounding.
#pragma once

#include "trace_kernel.cuh"

namespace otx {

using f2 = float2;

__device__ __forceinline__ f2 P2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 padd(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 pneg(f2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ f2 psub(f2 a, f2 b) { return __fadd2_rn(a, pneg(b)); }
__device__ __forceinline__ f2 pmul(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 pfma(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 pdivf(f2 a, f2 b) {
  return make_float2(__fdividef(a.x, b.x), __fdividef(a.y, b.y));
}
__device__ __forceinline__ f2 pdiv(f2 a, f2 b) { return make_float2(a.x / b.x, a.y / b.y); }
__device__ __forceinline__ f2 psqrt(f2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ f2 pabs(f2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ f2 psel(bool cx, bool cy, f2 a, f2 b) {
  return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}
__device__ __forceinline__ float lane(f2 v, int k) { return k ? v.y : v.x; }
__device__ __forceinline__ void set_lane(f2& v, int k, float s) {
  if (k)
    v.y = s;
  else
    v.x = s;
}

// Knuth's TwoSum on both lanes.
__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
  s = padd(a, b);
  const f2 bb = psub(s, a);
  e = padd(psub(a, psub(s, bb)), psub(b, bb));
}

struct Ray2 {
  f2 px, py, pz, dx, dy, dz, lx, ly, lz, wl, inten, att, n, opl_hi, opl_lo;
  bool ok[2];
};

__device__ __forceinline__ Ray get_ray(const Ray2& r, int k) {
  Ray s;
  s.px = lane(r.px, k);
  s.py = lane(r.py, k);
  s.pz = lane(r.pz, k);
  s.dx = lane(r.dx, k);
  s.dy = lane(r.dy, k);
  s.dz = lane(r.dz, k);
  s.lx = lane(r.lx, k);
  s.ly = lane(r.ly, k);
  s.lz = lane(r.lz, k);
  s.wl = lane(r.wl, k);
  s.inten = lane(r.inten, k);
  s.att = lane(r.att, k);
  s.n = lane(r.n, k);
  s.opl_hi = lane(r.opl_hi, k);
  s.opl_lo = lane(r.opl_lo, k);
  s.ok = r.ok[k];
  return s;
}

__device__ __forceinline__ void put_ray(Ray2& r, int k, const Ray& s) {
  set_lane(r.px, k, s.px);
  set_lane(r.py, k, s.py);
  set_lane(r.pz, k, s.pz);
  set_lane(r.dx, k, s.dx);
  set_lane(r.dy, k, s.dy);
  set_lane(r.dz, k, s.dz);
  set_lane(r.lx, k, s.lx);
  set_lane(r.ly, k, s.ly);
  set_lane(r.lz, k, s.lz);
  set_lane(r.wl, k, s.wl);
  set_lane(r.inten, k, s.inten);
  set_lane(r.att, k, s.att);
  set_lane(r.n, k, s.n);
  set_lane(r.opl_hi, k, s.opl_hi);
  set_lane(r.opl_lo, k, s.opl_lo);
  r.ok[k] = s.ok;
}

// ---------------------------------------------------------------- steps

// a x + b z in float-float on both lanes (rot2_ff).
__device__ __forceinline__ void rot2_ff2(float ah, float al, float bh, float bl, f2 x, f2 z,
                                         f2 xl, f2 zl, f2& hi, f2& lo) {
  const f2 A = P2(ah), B = P2(bh);
  const f2 p1 = pmul(A, x), e1 = pfma(A, x, pneg(p1));
  const f2 p2 = pmul(B, z), e2 = pfma(B, z, pneg(p2));
  f2 s, t;
  two_sum2(p1, p2, s, t);
  f2 l = padd(t, padd(e1, e2));
  l = pfma(P2(al), x, pfma(P2(bl), z, l));
  l = pfma(A, xl, pfma(B, zl, l));
  hi = padd(s, l);
  lo = psub(l, psub(hi, s));
}

// frame_change on both lanes: translations and rotations about y packed,
// other rotations lane by lane.
__device__ __forceinline__ void frame_change2(const otx_affine& f, Ray2& r, f2 lo[3]) {
  f2 rh[3], rl[3];
  if (f.flags & OTX_AFFINE_ROT_IDENTITY) {
    rh[0] = r.px;
    rh[1] = r.py;
    rh[2] = r.pz;
    rl[0] = rl[1] = rl[2] = P2(0.f);
  } else if (f.flags & OTX_AFFINE_ROT_Y) {
    rot2_ff2(f.m[0], f.m_lo[0], f.m[2], f.m_lo[2], r.px, r.pz, P2(0.f), P2(0.f), rh[0], rl[0]);
    rot2_ff2(f.m[6], f.m_lo[6], f.m[8], f.m_lo[8], r.px, r.pz, P2(0.f), P2(0.f), rh[2], rl[2]);
    rh[1] = r.py;
    rl[1] = P2(0.f);
    f2 dxh, dxl, dzh, dzl;
    rot2_ff2(f.m[0], f.m_lo[0], f.m[2], f.m_lo[2], r.dx, r.dz, r.lx, r.lz, dxh, dxl);
    rot2_ff2(f.m[6], f.m_lo[6], f.m[8], f.m_lo[8], r.dx, r.dz, r.lx, r.lz, dzh, dzl);
    r.dx = dxh;
    r.lx = dxl;
    r.dz = dzh;
    r.lz = dzl;
  } else {
    for (int k = 0; k < 2; ++k) {
      Ray s = get_ray(r, k);
      float l[3];
      frame_change(f, s, l);
      put_ray(r, k, s);
      set_lane(lo[0], k, l[0]);
      set_lane(lo[1], k, l[1]);
      set_lane(lo[2], k, l[2]);
    }
    return;
  }
  f2 e;
  two_sum2(rh[0], P2(f.t_hi[0]), r.px, e);
  lo[0] = padd(e, padd(rl[0], P2(f.t_lo[0])));
  two_sum2(rh[1], P2(f.t_hi[1]), r.py, e);
  lo[1] = padd(e, padd(rl[1], P2(f.t_lo[1])));
  two_sum2(rh[2], P2(f.t_hi[2]), r.pz, e);
  lo[2] = padd(e, padd(rl[2], P2(f.t_lo[2])));
}

// The conic's sag and gradient (sag_eval) on both lanes.
__device__ __forceinline__ f2 conic_sag2(const otx_surface& s, f2 x, f2 y, f2& gx, f2& gy) {
  const float c = s.sag_curvature;
  const float kp1 = 1.f + s.sag_conic;
  const f2 C = P2(c);
  const f2 r2 = pfma(x, x, pmul(y, y));
  if (kp1 == 0.f) {
    gx = pmul(C, x);
    gy = pmul(C, y);
    return pmul(P2(0.5f), pmul(C, r2));
  }
  const f2 g = psqrt(psub(P2(1.f), pmul(pmul(pmul(P2(kp1), C), C), r2)));
  const f2 cg = pdiv(C, g);
  gx = pmul(cg, x);
  gy = pmul(cg, y);
  return pdiv(pmul(C, r2), padd(P2(1.f), g));
}

// One Newton step on z - sag(x, y) from the current point (newton_step).
__device__ __forceinline__ f2 conic_newton2(const otx_surface& s, f2& x, f2& y, f2& z, f2 ux,
                                            f2 uy, f2 uz) {
  f2 gx, gy;
  const f2 zs = conic_sag2(s, x, y, gx, gy);
  const f2 f = psub(z, zs);
  const f2 fp = psub(uz, padd(pmul(gx, ux), pmul(gy, uy)));
  const f2 dt = pdivf(f, fp);
  x = pfma(pneg(dt), ux, x);
  y = pfma(pneg(dt), uy, y);
  z = pfma(pneg(dt), uz, z);
  return dt;
}

// Intercept with a flat or conic sag (intercept), t + tl as float-float.
template <int SAG>
__device__ __forceinline__ f2 intercept2(const otx_surface& s, f2 ox, f2 oy, f2 oz,
                                         const f2 lo[3], f2 ux, f2 uy, f2 uz, f2 lx, f2 ly,
                                         f2 lz, f2& x, f2& y, f2& z, f2& tl) {
  const f2 oxf = padd(ox, lo[0]), oyf = padd(oy, lo[1]), ozf = padd(oz, lo[2]);
  if constexpr (SAG == OTX_SAG_FLAT) {
    const f2 inv = pdivf(P2(1.f), uz);
    const f2 t0 = pmul(pneg(ozf), inv);
    const f2 t = psub(t0, pmul(pmul(t0, lz), inv));
    x = padd(pfma(t, ux, ox), pfma(t, lx, lo[0]));
    y = padd(pfma(t, uy, oy), pfma(t, ly, lo[1]));
    z = padd(pfma(t, uz, oz), pfma(t, lz, lo[2]));
    const f2 dt = pmul(z, inv);
    x = pfma(pneg(dt), ux, x);
    y = pfma(pneg(dt), uy, y);
    z = P2(0.f);
    tl = pneg(dt);
    return t;
  } else {
    const float c = s.sag_curvature;
    const f2 C = P2(c), K = P2(1.f + s.sag_conic);
    const f2 A = pmul(C, pfma(ux, ux, pfma(uy, uy, pmul(K, pmul(uz, uz)))));
    const f2 B = pmul(P2(2.f), psub(pmul(C, pfma(oxf, ux, pfma(oyf, uy, pmul(K, pmul(ozf, uz))))), uz));
    const f2 Cc = pfma(C, pfma(oxf, oxf, pfma(oyf, oyf, pmul(K, pmul(ozf, ozf)))), pmul(P2(-2.f), ozf));
    const f2 disc = pfma(B, B, pmul(P2(-4.f), pmul(A, Cc)));
    f2 t;
    for (int k = 0; k < 2; ++k) {
      const float a_ = lane(A, k), b_ = lane(B, k), c_ = lane(Cc, k), d_ = lane(disc, k);
      const bool real = d_ >= 0.f;
      const float sq = sqrtf(real ? d_ : 0.f);
      float ta, tb;
      if (fabsf(a_) < 1e-12f) {
        ta = -c_ / b_;
        tb = ta;
      } else {
        const float qq = -0.5f * (b_ + copysignf(sq, b_));
        const float r1 = __fdividef(qq, a_), r2 = __fdividef(c_, qq);
        ta = b_ >= 0.f ? r1 : r2;
        tb = b_ >= 0.f ? r2 : r1;
      }
      const float oxk = lane(oxf, k), oyk = lane(oyf, k), ozk = lane(ozf, k);
      const float uxk = lane(ux, k), uyk = lane(uy, k), uzk = lane(uz, k);
      const float za = fmaf(ta, uzk, ozk), xa = fmaf(ta, uxk, oxk), ya = fmaf(ta, uyk, oyk);
      const float zb = fmaf(tb, uzk, ozk), xb = fmaf(tb, uxk, oxk), yb = fmaf(tb, uyk, oyk);
      const bool va = real && (za * (c * fmaf(xa, xa, ya * ya) - za) >= 0.f);
      const bool vb = real && (zb * (c * fmaf(xb, xb, yb * yb) - zb) >= 0.f);
      ta = va ? ta : INFINITY;
      tb = vb ? tb : INFINITY;
      set_lane(t, k, (fabsf(ta) <= fabsf(tb)) ? ta : tb);
    }
    x = padd(pfma(t, ux, ox), pfma(t, lx, lo[0]));
    y = padd(pfma(t, uy, oy), pfma(t, ly, lo[1]));
    z = padd(pfma(t, uz, oz), pfma(t, lz, lo[2]));
    f2 xn = x, yn = y, zn = z;
    const f2 dt = conic_newton2(s, xn, yn, zn, ux, uy, uz);
    const bool fx = isfinite(t.x), fy = isfinite(t.y);
    x = psel(fx, fy, xn, x);
    y = psel(fx, fy, yn, y);
    z = psel(fx, fy, zn, z);
    tl = psel(fx, fy, pneg(dt), P2(0.f));
    return t;
  }
}

// opl += n (t + tl) on both lanes (opl_add).
__device__ __forceinline__ void opl_add2(Ray2& r, f2 n, f2 t, f2 tl) {
  const f2 p = pmul(n, t);
  const f2 pe = pfma(n, t, pneg(p));
  f2 s, e;
  two_sum2(r.opl_hi, p, s, e);
  r.opl_hi = s;
  r.opl_lo = padd(r.opl_lo, pfma(n, tl, padd(e, pe)));
}

// reflect_gradient on both lanes.
__device__ __forceinline__ void reflect_gradient2(Ray2& r, f2 gx, f2 gy) {
  f2 n_hi, n_lo;
  two_sum2(pneg(r.dz), pfma(r.dx, gx, pmul(r.dy, gy)), n_hi, n_lo);
  n_lo = padd(n_lo, pfma(r.lx, gx, pfma(r.ly, gy, pneg(r.lz))));
  const f2 p1 = pmul(gx, gx), e1 = pfma(gx, gx, pneg(p1));
  const f2 p2 = pmul(gy, gy), e2 = pfma(gy, gy, pneg(p2));
  f2 q, eq, d_hi, d_lo;
  two_sum2(p1, p2, q, eq);
  two_sum2(P2(1.f), q, d_hi, d_lo);
  d_lo = padd(d_lo, padd(eq, padd(e1, e2)));
  const f2 inv = pdivf(P2(1.f), d_hi);
  const f2 q_hi = pmul(n_hi, inv);
  const f2 rem = psub(padd(pfma(pneg(q_hi), d_hi, n_hi), n_lo), pmul(q_hi, d_lo));
  const f2 k_hi = pmul(P2(2.f), q_hi), k_lo = pmul(P2(2.f), pmul(rem, inv));
  f2 s, e;
  {
    const f2 p = pmul(k_hi, gx), pe = pfma(k_hi, gx, pneg(p));
    two_sum2(r.dx, pneg(p), s, e);
    r.dx = s;
    r.lx = padd(e, psub(psub(r.lx, pe), pmul(k_lo, gx)));
  }
  {
    const f2 p = pmul(k_hi, gy), pe = pfma(k_hi, gy, pneg(p));
    two_sum2(r.dy, pneg(p), s, e);
    r.dy = s;
    r.ly = padd(e, psub(psub(r.ly, pe), pmul(k_lo, gy)));
  }
  two_sum2(r.dz, k_hi, s, e);
  r.dz = s;
  r.lz = padd(e, padd(r.lz, k_lo));
  for (int k = 0; k < 2; ++k) {
    float ax = lane(r.dx, k), ay = lane(r.dy, k), az = lane(r.dz, k);
    float lx = lane(r.lx, k), ly = lane(r.ly, k), lz = lane(r.lz, k);
    normalize3(ax, ay, az, lx, ly, lz);
    set_lane(r.dx, k, ax);
    set_lane(r.dy, k, ay);
    set_lane(r.dz, k, az);
    set_lane(r.lx, k, lx);
    set_lane(r.ly, k, ly);
    set_lane(r.lz, k, lz);
  }
}

// Complex values on both lanes.
struct cf2 {
  f2 re, im;
};
__device__ __forceinline__ cf2 c2add(cf2 a, cf2 b) { return cf2{padd(a.re, b.re), padd(a.im, b.im)}; }
__device__ __forceinline__ cf2 c2sub(cf2 a, cf2 b) { return cf2{psub(a.re, b.re), psub(a.im, b.im)}; }
__device__ __forceinline__ cf2 c2mul(cf2 a, cf2 b) {
  return cf2{pfma(a.re, b.re, pneg(pmul(a.im, b.im))), pfma(a.re, b.im, pmul(a.im, b.re))};
}
__device__ __forceinline__ cf2 c2scale(cf2 a, f2 s) { return cf2{pmul(a.re, s), pmul(a.im, s)}; }
__device__ __forceinline__ cf2 c2conj(cf2 a) { return cf2{a.re, pneg(a.im)}; }
__device__ __forceinline__ f2 c2abs2(cf2 a) { return pfma(a.re, a.re, pmul(a.im, a.im)); }

// The bare-coating Fresnel mirror (fresnel_efficiency, mirror case) on both
// lanes: the table lookups and square roots per lane, the complex
// arithmetic packed.
__device__ __forceinline__ f2 fresnel_mirror2(const otx_system& sys, const otx_stack& K, f2 wl,
                                              f2 cos0, cf2 n0) {
  cf2 n1{P2(1.f), P2(0.f)};
  if (K.substrate >= 0) {
    const otx_layer& L = sys.layers[K.substrate];
    const cf a = layer_n<true>(sys, L, wl.x), b = layer_n<true>(sys, L, wl.y);
    n1 = cf2{make_float2(a.re, b.re), make_float2(a.im, b.im)};
  }
  const cf2 inv0 = c2scale(c2mul(n0, n0), pfma(pneg(cos0), cos0, P2(1.f)));
  // w = n1 sqrt(1 - inv0 / n1^2) (medium_q<true>, s)
  const cf2 nj2 = c2mul(n1, n1);
  const f2 rr = pdivf(P2(1.f), c2abs2(nj2));
  const cf2 ratio = c2scale(c2mul(inv0, c2conj(nj2)), rr);
  cf2 cj;
  for (int k = 0; k < 2; ++k) {
    const cf z = csqrt(cf{1.f - lane(ratio.re, k), -lane(ratio.im, k)});
    set_lane(cj.re, k, z.re);
    set_lane(cj.im, k, z.im);
  }
  const cf2 w = c2mul(n1, cj);
  const cf2 q0 = c2scale(n0, cos0);
  const f2 ns = c2abs2(c2sub(q0, w)), ds = c2abs2(c2add(q0, w));
  const cf2 a = c2scale(q0, c2abs2(n1)), b = c2scale(w, c2abs2(n0));
  const f2 np = c2abs2(c2sub(a, b)), dp = c2abs2(c2add(a, b));
  const f2 den = pmul(ds, dp);
  const f2 num = pfma(ns, dp, pmul(np, ds));
  f2 eff;
  for (int k = 0; k < 2; ++k) {
    const float d = lane(den, k);
    set_lane(eff, k,
             (d > 1e-30f && d < 1e30f)
                 ? 0.5f * __fdividef(lane(num, k), d)
                 : 0.5f * (lane(ns, k) / lane(ds, k) + lane(np, k) / lane(dp, k)));
  }
  return eff;
}

// One surface of the Newtonian kinds on both lanes (propagate_surface).
template <class K>
__device__ __forceinline__ void propagate2(const otx_system& sys, const otx_surface& s, Ray2& r) {
  static_assert(K::sag == OTX_SAG_FLAT || K::sag == OTX_SAG_CONIC, "packed sags: flat, conic");
  static_assert(K::rule == OTX_RULE_NONE, "packed surfaces have no rulings");
  f2 lo[3];
  frame_change2(s.to_local, r, lo);
  const f2 ox = r.px, oy = r.py, oz = r.pz;
  f2 x, y, z, tl;
  const f2 t = intercept2<K::sag>(s, ox, oy, oz, lo, r.dx, r.dy, r.dz, r.lx, r.ly, r.lz, x, y,
                                  z, tl);
  r.px = x;
  r.py = y;
  r.pz = z;
  if (r.att.x != 0.f || r.att.y != 0.f) {
    const f2 len = pmul(pabs(t), psqrt(pfma(r.dx, r.dx, pfma(r.dy, r.dy, pmul(r.dz, r.dz)))));
    r.inten = make_float2(r.inten.x * expf(-r.att.x * len.x), r.inten.y * expf(-r.att.y * len.y));
  }
  opl_add2(r, r.n, t, tl);

  // normal: the flat's (0, 0, -1); the conic's gradient form
  f2 nx, ny, nz, gx = P2(0.f), gy = P2(0.f);
  if constexpr (K::sag == OTX_SAG_FLAT) {
    nx = ny = P2(0.f);
    nz = P2(-1.f);
  } else {
    conic_sag2(s, x, y, gx, gy);
    const f2 q = pfma(gx, gx, pfma(gy, gy, P2(1.f)));
    f2 inv = make_float2(rsqrtf(q.x), rsqrtf(q.y));
    inv = pfma(pmul(P2(0.5f), inv), pfma(pneg(pmul(q, inv)), inv, P2(1.f)), inv);
    nx = pmul(gx, inv);
    ny = pmul(gy, inv);
    nz = pneg(inv);
  }

  const f2 n1 = r.n;
  f2 n2 = n1, att2 = r.att, eff = P2(1.f);
  bool mirror = false;
  if constexpr (K::mat == OTX_MAT_VACUUM) {
    n2 = P2(1.f);
    att2 = P2(0.f);
  } else if constexpr (K::mat == OTX_MAT_MIRROR) {
    mirror = true;
  } else if constexpr (K::mat == OTX_MAT_FRESNEL_MIRROR) {
    mirror = true;
    const f2 kk = pmul(pmul(r.att, pmul(r.wl, P2(1e-6f))), P2(0.07957747154594767f));
    const f2 cos0 = pneg(pfma(r.dx, nx, pfma(r.dy, ny, pmul(r.dz, nz))));
    const int ks = min(max(s.mat_stack, 0), OTX_MAX_STACKS - 1);
    eff = fresnel_mirror2(sys, sys.stacks[ks], r.wl, cos0, cf2{n1, kk});
  } else {
    static_assert(K::mat == OTX_MAT_VACUUM, "packed materials: vacuum, mirror, Fresnel mirror");
  }
  if (n2.x != n1.x || n2.y != n1.y)
    r.wl = make_float2(n2.x != n1.x ? r.wl.x / (n1.x / n2.x) : r.wl.x,
                       n2.y != n1.y ? r.wl.y / (n1.y / n2.y) : r.wl.y);
  // |a|^2 - 1 of both directions: unit ones take the packed reflection
  f2 e = pfma(r.dx, r.dx, P2(-1.f));
  e = pfma(r.dy, r.dy, e);
  e = pfma(r.dz, r.dz, e);
  const bool unit = fabsf(e.x) < 1e-6f && fabsf(e.y) < 1e-6f;
  if (mirror && unit && K::sag == OTX_SAG_FLAT) {
    r.dz = pneg(r.dz);
    r.lz = pneg(r.lz);
  } else if (mirror && unit) {
    reflect_gradient2(r, gx, gy);
  } else if (!mirror && unit && n1.x == n2.x && n1.y == n2.y) {
    // equal indices, unit directions: Snell's step leaves them unchanged
  } else {
    for (int k = 0; k < 2; ++k) {
      Ray q = get_ray(r, k);
      const float nk1 = lane(n1, k), nk2 = lane(n2, k);
      // the scalar step's choices (propagate_surface)
      const bool um = mirror && fabsf(fmaf(q.dx, q.dx, fmaf(q.dy, q.dy, fmaf(q.dz, q.dz, -1.f)))) < 1e-6f;
      if (um && K::sag == OTX_SAG_FLAT) {
        q.dz = -q.dz;
        q.lz = -q.lz;
      } else if (um) {
        reflect_gradient(q.dx, q.dy, q.dz, q.lx, q.ly, q.lz, lane(gx, k), lane(gy, k));
      } else {
        snell(q.dx, q.dy, q.dz, q.lx, q.ly, q.lz, nk1, nk2, mirror, lane(nx, k), lane(ny, k),
              lane(nz, k));
      }
      put_ray(r, k, q);
    }
  }
  r.inten = pmul(r.inten, eff);
  r.att = att2;
  r.n = n2;

  if constexpr (K::aper != OTX_APER_NONE) {
    const bool on_dir = (s.aper_flags & OTX_APER_FLAG_DIRECTION) != 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const bool m = on_dir ? aperture_inside(K::aper, sys, s, lane(r.dx, k), lane(r.dy, k),
                                              lane(r.dz, k))
                            : aperture_inside(K::aper, sys, s, lane(r.px, k), lane(r.py, k),
                                              lane(r.pz, k));
      r.ok[k] = r.ok[k] && m;
    }
  }
}

template <int I, class K, class... Rest>
__device__ __forceinline__ void propagate_pair(const otx_system& sys, Ray2& r) {
  propagate2<K>(sys, sys.surfaces[I], r);
  if constexpr (sizeof...(Rest) > 0) propagate_pair<I + 1, Rest...>(sys, r);
}

// Input rays of the grid at infinity for both lanes (load_ray): the
// direction series packed when both lanes' angles are small.
__device__ __forceinline__ void load_pair(const TraceArgs& a, int64_t i0, int64_t i1, Ray2& r) {
  const otx_grid& g = a.grid;
  const float* W = reinterpret_cast<const float*>(g.wavelength);
  const float* FX = reinterpret_cast<const float*>(g.field_x);
  const float* FY = reinterpret_cast<const float*>(g.field_y);
  const float* QX = reinterpret_cast<const float*>(g.pupil_x);
  const float* QY = reinterpret_cast<const float*>(g.pupil_y);
  r.wl = make_float2(W[i0 * g.stride_wavelength], W[i1 * g.stride_wavelength]);
  const f2 fx = make_float2(FX[i0 * g.stride_field], FX[i1 * g.stride_field]);
  const f2 fy = make_float2(FY[i0 * g.stride_field], FY[i1 * g.stride_field]);
  r.px = make_float2(QX[i0 * g.stride_pupil], QX[i1 * g.stride_pupil]);
  r.py = make_float2(QY[i0 * g.stride_pupil], QY[i1 * g.stride_pupil]);
  r.pz = P2(0.f);
  if (g.intensity) {
    const float* I = reinterpret_cast<const float*>(g.intensity);
    r.inten = make_float2(I[i0 * g.stride_intensity], I[i1 * g.stride_intensity]);
  } else {
    r.inten = P2(1.f);
  }
  r.att = P2(0.f);
  r.n = P2(1.f);
  r.opl_hi = r.opl_lo = P2(0.f);
  r.ok[0] = r.ok[1] = true;
  const float amax = fmaxf(fmaxf(fabsf(fx.x), fabsf(fy.x)), fmaxf(fabsf(fx.y), fabsf(fy.y)));
  if (amax <= 0.0625f) {
    // sin_cosm1_small and direction_from_angles on both lanes
    f2 sxh, sxl, cmx, syh, syl, cmy;
    {
      const f2 a2 = pmul(fx, fx);
      const f2 p = pmul(a2, pfma(a2, pfma(a2, P2(-1.f / 5040.f), P2(1.f / 120.f)), P2(-1.f / 6.f)));
      sxh = pfma(fx, p, fx);
      sxl = pfma(fx, p, psub(fx, sxh));
      cmx = pmul(a2, pfma(a2, pfma(a2, pfma(a2, P2(1.f / 40320.f), P2(-1.f / 720.f)), P2(1.f / 24.f)),
                          P2(-0.5f)));
    }
    {
      const f2 a2 = pmul(fy, fy);
      const f2 p = pmul(a2, pfma(a2, pfma(a2, P2(-1.f / 5040.f), P2(1.f / 120.f)), P2(-1.f / 6.f)));
      syh = pfma(fy, p, fy);
      syl = pfma(fy, p, psub(fy, syh));
      cmy = pmul(a2, pfma(a2, pfma(a2, pfma(a2, P2(1.f / 40320.f), P2(-1.f / 720.f)), P2(1.f / 24.f)),
                          P2(-0.5f)));
    }
    const f2 xh = pfma(cmy, sxh, sxh);
    const f2 xl = padd(pfma(cmy, sxh, psub(sxh, xh)), pfma(cmy, sxl, sxl));
    r.dx = pneg(xh);
    r.lx = pneg(xl);
    r.dy = pneg(syh);
    r.ly = pneg(syl);
    const f2 sz = pfma(cmx, cmy, padd(cmx, cmy));
    r.dz = padd(P2(1.f), sz);
    r.lz = psub(sz, psub(r.dz, P2(1.f)));
  } else {
    for (int k = 0; k < 2; ++k) {
      float dx, dy, dz, lx, ly, lz;
      direction_from_angles(lane(fx, k), lane(fy, k), dx, dy, dz, lx, ly, lz);
      set_lane(r.dx, k, dx);
      set_lane(r.dy, k, dy);
      set_lane(r.dz, k, dz);
      set_lane(r.lx, k, lx);
      set_lane(r.ly, k, ly);
      set_lane(r.lz, k, lz);
    }
  }
}

// The shape-specialised trace with two rays per thread: ray i and ray
// i + blockDim.x of each 2 * blockDim.x block of rays (both loads and stores
// coalesced).  Grid input with the object at infinity; 4 CTAs of 256
// threads per SM (64 registers per thread, a few bytes spilled).
//
// Measured on the precision workload (1e8 rays, one GB300): 21 % fewer
// issued instructions than the one-ray kernel, but 4.68 ms against its
// 4.63 ms (4.89 ms at 3 CTAs per SM, 5.48 ms at 2): the packed
// instructions' latency with fewer rays in flight per register, and the
// lane moves around the per-lane steps, take back what the pairing saves.
// The library therefore runs the one-ray kernel unless a caller asks for
// two rays per thread (otx_launch.rays_per_thread = 2).
#ifndef OTX_PAIR_MIN_BLOCKS
#define OTX_PAIR_MIN_BLOCKS 4
#endif
template <class K0, class... Ks>
__global__ void __launch_bounds__(256, OTX_PAIR_MIN_BLOCKS)
    k_trace_pair(const __grid_constant__ otx_system sys, const __grid_constant__ TraceArgs a) {
  const int64_t n = a.count;
  const int64_t step = (int64_t)gridDim.x * blockDim.x * 2;
  const bool bin = image_any(a.img);
  const bool final_identity = (sys.flags & OTX_SYS_FLAG_FINAL_IDENTITY) != 0;
  const bool skip0 = first_is_noop<OTX_INPUT_GRID_INFINITY, K0>(sys);
  int bin_skip = 0;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x * 2 + threadIdx.x; i0 < n; i0 += step) {
    const int64_t i1 = i0 + blockDim.x;
    const bool has1 = i1 < n;
    Ray2 r;
    load_pair(a, i0, has1 ? i1 : i0, r);
    if (!skip0) propagate2<K0>(sys, sys.surfaces[0], r);
    if constexpr (sizeof...(Ks) > 0) propagate_pair<1, Ks...>(sys, r);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k == 1 && !has1) break;
      const Ray q = get_ray(r, k);
      const int64_t i = k ? i1 : i0;
      if (bin) bin_ray_warp(sys.sensor, a.img, q, bin_skip);
      if (final_identity)
        store_ray<true>(a.out, i, sys.final_to_output, q);
      else
        store_ray<false>(a.out, i, sys.final_to_output, q);
    }
  }
}

}  // namespace otx
