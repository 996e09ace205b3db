// Multilayer reflectivity / transmissivity in float-float arithmetic.
//
// Same formulation as the FP32 evaluator of trace_device.cuh (unnormalised
// Yeh transfer matrices, optika/materials/_layers.py:229-277 and
// optika/materials/_multilayers.py:187-237, 485-532), carried in
// float-float: the period matrix of a periodic stack is raised to the power
// N - 1, which multiplies its rounding error by ~N, so FP32 products and
// FP32 phases leave T ~1e-5 off complex128 for 40 periods; float-float
// keeps it ~1e-7.  The layer phases use float-float exp / sin / cos built
// from argument reduction and Taylor series (no FP32 transcendental
// enters the phase).
#pragma once

#include "ff.cuh"
#include "trace_device.cuh"

namespace otx {

// 2 pi, pi / 2, ln 2 as float-float constants (hi + lo).
__device__ __forceinline__ ff ff_2pi() { return ff{6.28318548202514648f, -1.74845553e-07f}; }
__device__ __forceinline__ ff ff_pio2() { return ff{1.57079637050628662f, -4.37113883e-08f}; }
__device__ __forceinline__ ff ff_ln2() { return ff{0.693147182464599609f, -1.90465421e-09f}; }

// Taylor coefficients as float-float pairs (hi + lo): 1/i! for exp,
// (-1)^k/(2k+1)! for sin, (-1)^k/(2k)! for cos, each exact to ~2^-72.
__device__ __forceinline__ ff ffc(float hi, float lo) { return ff{hi, lo}; }

// Horner step p r + c in float-float.
__device__ __forceinline__ ff ff_horner(ff p, ff r, ff c) { return ff_add(ff_mul(p, r), c); }

// exp(x) for a float-float x: x = k ln2 + r, |r| <= ln2 / 2, exp(r) by its
// Taylor series to r^13 / 13! (Horner), then scaled by 2^k.  The terms from
// r^8 on are below 2^-25 of the sum, so their part of the Horner scheme
// runs in FP32; the rest runs in float-float.
__device__ __forceinline__ ff ff_exp(ff x) {
  if (x.hi > 88.f) return ff{INFINITY, 0.f};
  if (x.hi < -103.f) return ff{0.f, 0.f};
  const float k = rintf(x.hi * 1.44269504088896341f);
  const ff r = ff_sub(x, ff_mulf(ff_ln2(), k));
  const float rf = r.hi;
  float t = fmaf(0x1.612462p-33f, rf, 0x1.1eed8ep-29f);  // 1/13!, 1/12!
  t = fmaf(t, rf, 0x1.ae6456p-26f);                      // 1/11!
  t = fmaf(t, rf, 0x1.27e4fcp-22f);                      // 1/10!
  t = fmaf(t, rf, 0x1.71de3ap-19f);                      // 1/9!
  t = fmaf(t, rf, 0x1.a01a02p-16f);                      // 1/8!
  ff p = ff_add(ff_mul(ff_of(t), r), ffc(0x1.a01a02p-13f, -0x1.7f97fap-39f));  // 1/7!
  p = ff_horner(p, r, ffc(0x1.6c16c2p-10f, -0x1.27d27ep-35f));                 // 1/6!
  p = ff_horner(p, r, ffc(0x1.111112p-7f, -0x1.dddddep-32f));                  // 1/5!
  p = ff_horner(p, r, ffc(0x1.555556p-5f, -0x1.555556p-30f));                  // 1/4!
  p = ff_horner(p, r, ffc(0x1.555556p-3f, -0x1.555556p-28f));                  // 1/3!
  p = ff_horner(p, r, ff_of(0.5f));
  p = ff_horner(p, r, ff_of(1.f));
  p = ff_horner(p, r, ff_of(1.f));
  return ff_scale2(p, ldexpf(1.f, (int)k));
}

// sin and cos of a float-float x: x = k pi/2 + r, |r| <= pi/4, Taylor
// series of sin(r) to r^17 and cos(r) to r^16 (Horner in r^2), then the
// quadrant of k.  The terms from r^10 (cos) and r^11 (sin) on are below
// 2^-25 of the sum and run in FP32.
__device__ __forceinline__ void ff_sincos(ff x, ff& s, ff& c) {
  const float k = rintf(x.hi * 0.636619772367581343f);
  const ff r = ff_sub(x, ff_mulf(ff_pio2(), k));
  const ff r2 = ff_mul(r, r);
  const float q = r2.hi;
  float ts = fmaf(0x1.952c78p-49f, q, -0x1.ae7f3ep-41f);  // 1/17!, -1/15!
  ts = fmaf(ts, q, 0x1.612462p-33f);                       // 1/13!
  ts = fmaf(ts, q, -0x1.ae6456p-26f);                      // -1/11!
  float tc = fmaf(0x1.ae7f3ep-45f, q, -0x1.93974ap-37f);  // 1/16!, -1/14!
  tc = fmaf(tc, q, 0x1.1eed8ep-29f);                       // 1/12!
  tc = fmaf(tc, q, -0x1.27e4fcp-22f);                      // -1/10!
  ff ps = ff_add(ff_mul(ff_of(ts), r2), ffc(0x1.71de3ap-19f, 0x1.55b1ccp-45f));  // 1/9!
  ff pc = ff_add(ff_mul(ff_of(tc), r2), ffc(0x1.a01a02p-16f, -0x1.7f97fap-42f));  // 1/8!
  ps = ff_horner(ps, r2, ffc(-0x1.a01a02p-13f, 0x1.7f97fap-39f));  // -1/7!
  pc = ff_horner(pc, r2, ffc(-0x1.6c16c2p-10f, 0x1.27d27ep-35f));  // -1/6!
  ps = ff_horner(ps, r2, ffc(0x1.111112p-7f, -0x1.dddddep-32f));   // 1/5!
  pc = ff_horner(pc, r2, ffc(0x1.555556p-5f, -0x1.555556p-30f));   // 1/4!
  ps = ff_horner(ps, r2, ffc(-0x1.555556p-3f, 0x1.555556p-28f));   // -1/3!
  pc = ff_horner(pc, r2, ff_of(-0.5f));
  ps = ff_horner(ps, r2, ff_of(1.f));
  pc = ff_horner(pc, r2, ff_of(1.f));
  const ff sr = ff_mul(r, ps);
  const ff cr = pc;
  const int qd = ((int)k) & 3;
  switch (qd) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = ff_neg(sr); break;
    case 2: s = ff_neg(sr); c = ff_neg(cr); break;
    default: s = ff_neg(cr); c = sr; break;
  }
}

// Transfer-matrix state of one polarisation (see MLState in
// trace_device.cuh): unnormalised product with its exponent and, for T,
// the product of |2 q_i|^2.
struct MLff {
  cmff m;
  int e;
  bool first;
  ff t;
  int te;
  cff q;
  cf n;  // index of the current medium (interface-profile factors)
  cff inv0;
  bool where;
};

__device__ __forceinline__ cff medium_q_ff(const cff& inv0, cf nj_f, bool pol_p) {
  const cff nj = cff_of(nj_f.re, nj_f.im);
  const cff nj2 = cff_mul(nj, nj);
  const cff ratio = cff_div(inv0, nj2);
  const cff cj = cff_sqrt(cff_sub(cff_of(1.f, 0.f), ratio));
  const cff w = cff_mul(nj, cj);
  if (!pol_p) return w;
  return cff_scale(cff_conj(w), ff_div(ff_of(1.f), cff_abs2(nj)));
}

__device__ __forceinline__ void mlff_times(MLff& st, const cmff& t, int te) {
  if (st.first) {
    st.m = t;
    st.e = te;
    st.first = false;
  } else {
    st.m = cmff_mul(st.m, t);
    st.e += te;
  }
  cmff_normalize(st.m, st.e);
}

__device__ __forceinline__ void ff_normalize_scalar(ff& t, int& te) {
  if (!(t.hi > 0.f) || !isfinite(t.hi)) return;
  const int e = ilogbf(t.hi);
  t = ff_scale2(t, ldexpf(1.f, -e));
  te += e;
}

// An interface profile on the layer's left side scales r_ij, the
// off-diagonal q_i - q_j (see layer_step in trace_device.cuh); its factor is
// real, near 1 and evaluated in single precision.
template <bool NEED_T>
__device__ __forceinline__ void layer_step_ff(MLff& st, cf nj, float thickness, float wl,
                                              bool pol_p, int iface = OTX_PROFILE_NONE,
                                              float iface_width = 0.f) {
  const cff qj = medium_q_ff(st.inv0, nj, pol_p);
  const cff a = cff_add(st.q, qj);
  cff b = cff_sub(st.q, qj);
  if (iface != OTX_PROFILE_NONE) {
    const cf qi{st.q.re.hi, st.q.im.hi};
    b = cff_scale(b, ff_of(interface_factor(iface, iface_width,
                                            interface_wavenumber(qi, st.n, wl, pol_p))));
  }
  bool wprop = true;
  cmff tm{a, b, b, a};
  if (thickness != 0.f) {
    // beta = 2 pi h (n cos) / lambda ; n cos = q_s, or conj(q_p) |n|^2
    cff ncos = qj;
    if (pol_p) {
      const cff njc = cff_of(nj.re, nj.im);
      ncos = cff_scale(cff_conj(qj), cff_abs2(njc));
    }
    const ff k = ff_div(ff_mulf(ff_2pi(), thickness), ff_of(wl));
    const cff beta = cff_scale(ncos, k);
    ff sn, cs;
    ff_sincos(beta.re, sn, cs);
    const ff g = ff_exp(beta.im);  // |exp(-i beta)|
    wprop = g.hi < 1e10f;
    if (wprop) {
      const ff gi = ff_div(ff_of(1.f), g);
      const cff em{ff_mul(g, cs), ff_neg(ff_mul(g, sn))};
      const cff ep{ff_mul(gi, cs), ff_mul(gi, sn)};
      tm = cmff{cff_mul(a, em), cff_mul(b, ep), cff_mul(b, em), cff_mul(a, ep)};
    }
  }
  if (st.where) {
    mlff_times(st, tm, 0);
    if (NEED_T) {
      st.t = ff_mul(st.t, ff_scale2(cff_abs2(st.q), 4.f));
      ff_normalize_scalar(st.t, st.te);
    }
  }
  st.where = st.where && wprop;
  st.q = qj;
  st.n = nj;
}

__device__ __forceinline__ void cmff_pow(cmff base, int bexp, int e, cmff& acc, int& aexp) {
  bool first = true;
  while (e > 0) {
    if (e & 1) {
      if (first) {
        acc = base;
        aexp = bexp;
        first = false;
      } else {
        acc = cmff_mul(acc, base);
        aexp += bexp;
        cmff_normalize(acc, aexp);
      }
    }
    e >>= 1;
    if (e) {
      base = cmff_sqr(base);
      bexp *= 2;
      cmff_normalize(base, bexp);
    }
  }
}

// A stack as seen by the evaluator: pre layers, a periodic block, post
// layers and a substrate, each layer an index (at this wavelength) and a
// thickness.
struct SysStackSource {
  const otx_system& sys;
  const otx_stack& K;
  __device__ int count(int section) const {
    return section == 0 ? K.pre_count : (section == 1 ? K.per_count : K.post_count);
  }
  __device__ int periods() const { return K.num_periods; }
  __device__ const otx_layer& lay(int section, int i) const {
    const int b = section == 0 ? K.pre_begin : (section == 1 ? K.per_begin : K.post_begin);
    return sys.layers[b + i];
  }
  __device__ cf n(int section, int i, float wl) const { return layer_n(sys, lay(section, i), wl); }
  __device__ float h(int section, int i) const { return lay(section, i).thickness; }
  __device__ cf n_sub(float wl) const {
    return K.substrate >= 0 ? layer_n(sys, sys.layers[K.substrate], wl) : cf{1.f, 0.f};
  }
  __device__ int iface(int section, int i) const { return lay(section, i).interface_type; }
  __device__ float iface_width(int section, int i) const {
    return lay(section, i).interface_width;
  }
  __device__ int sub_iface() const {
    return K.substrate >= 0 ? sys.layers[K.substrate].interface_type : OTX_PROFILE_NONE;
  }
  __device__ float sub_iface_width() const {
    return K.substrate >= 0 ? sys.layers[K.substrate].interface_width : 0.f;
  }
};

struct PeriodicSource {
  const otx_periodic_stack& P;
  __device__ int count(int section) const { return section == 1 ? 2 : 0; }
  __device__ int periods() const { return P.num_periods; }
  __device__ cf n(int, int i, float) const {
    return i == 0 ? cf{P.n_a_re, P.n_a_im} : cf{P.n_b_re, P.n_b_im};
  }
  __device__ float h(int, int i) const { return i == 0 ? P.thickness_a : P.thickness_b; }
  __device__ cf n_sub(float) const { return cf{P.n_sub_re, P.n_sub_im}; }
  __device__ int iface(int, int) const { return OTX_PROFILE_NONE; }
  __device__ float iface_width(int, int) const { return 0.f; }
  __device__ int sub_iface() const { return OTX_PROFILE_NONE; }
  __device__ float sub_iface_width() const { return 0.f; }
};

template <bool NEED_T, class S>
__device__ __forceinline__ void run_section_ff(MLff& st, const S& src, int section, float wl,
                                               bool pol_p) {
  const int n = src.count(section);
  for (int i = 0; i < n; ++i)
    layer_step_ff<NEED_T>(st, src.n(section, i, wl), src.h(section, i), wl, pol_p,
                          src.iface(section, i), src.iface_width(section, i));
}

// Reflectivity and transmissivity of one polarisation (float-float), the
// same algorithm as multilayer_pol in trace_device.cuh.
template <bool NEED_T, class S>
__device__ __forceinline__ void multilayer_pol_ff(const S& src, float wl, float cos0, cf n0,
                                                  bool pol_p, float& R, float& T) {
  MLff st;
  st.e = 0;
  st.first = true;
  st.t = ff_of(1.f);
  st.te = 0;
  const cff n0c = cff_of(n0.re, n0.im);
  // (n0 sin0)^2 = n0^2 (1 - cos0^2)
  const ff one_m_c2 = ff_sub(ff_of(1.f), ff_mul(ff_of(cos0), ff_of(cos0)));
  st.inv0 = cff_scale(cff_mul(n0c, n0c), one_m_c2);
  if (pol_p)
    st.q = cff_scale(cff_conj(n0c), ff_div(ff_of(cos0), cff_abs2(n0c)));
  else
    st.q = cff_scale(n0c, ff_of(cos0));
  st.n = n0;
  const cff q0 = st.q;
  st.where = true;
  run_section_ff<NEED_T>(st, src, 0, wl, pol_p);
  if (src.count(1) > 0 && src.periods() > 0) {
    run_section_ff<NEED_T>(st, src, 1, wl, pol_p);  // first period
    MLff per = st;
    per.first = true;
    per.e = 0;
    per.t = ff_of(1.f);
    per.te = 0;
    run_section_ff<NEED_T>(per, src, 1, wl, pol_p);  // period from its own last medium
    const int reps = src.periods() - 1;
    if (!per.first && reps > 0) {
      cmff pm;
      int pe = 0;
      cmff_pow(per.m, per.e, reps, pm, pe);
      mlff_times(st, pm, pe);
      if (NEED_T) {
        for (int i = 0; i < reps; ++i) {
          st.t = ff_mul(st.t, per.t);
          st.te += per.te;
          ff_normalize_scalar(st.t, st.te);
        }
      }
    }
    st.where = per.where;
    st.q = per.q;
    st.n = per.n;
  }
  run_section_ff<NEED_T>(st, src, 2, wl, pol_p);
  layer_step_ff<NEED_T>(st, src.n_sub(wl), 0.f, wl, pol_p, src.sub_iface(),
                        src.sub_iface_width());
  const ff m11 = cff_abs2(st.m.a);
  R = ff_to_f(ff_div(cff_abs2(st.m.c), m11));
  T = 0.f;
  if (NEED_T && st.where) {
    const ff ratio = cff_div(st.q, q0).re;
    const ff tt = ff_mul(ff_div(st.t, m11), ratio);
    T = ldexpf(ff_to_f(tt), st.te - 2 * st.e);
  }
}

// ---------------------------------------------------------------- bilayer mirrors

// The propagation factors exp(-i beta), exp(+i beta) of one layer, beta =
// 2 pi h (n cos) / lambda, and whether the layer is transparent enough to
// enter the product (|exp(-i beta)| < 1e10).  n cos is the same for s and
// p (the p-medium factor conj(q_p) |n|^2 equals q_s), so one evaluation
// serves both polarisations and every period.
struct LayerPhase {
  cff em, ep;
  bool prop;
};

__device__ __forceinline__ LayerPhase layer_phase_ff(const cff& w, float thickness, float wl) {
  const ff k = ff_div(ff_mulf(ff_2pi(), thickness), ff_of(wl));
  const cff beta = cff_scale(w, k);
  ff sn, cs;
  ff_sincos(beta.re, sn, cs);
  const ff g = ff_exp(beta.im);
  LayerPhase L;
  L.prop = g.hi < 1e10f;
  L.em = cff{ff_mul(g, cs), ff_neg(ff_mul(g, sn))};
  const ff gi = ff_div(ff_of(1.f), g);
  L.ep = cff{ff_mul(gi, cs), ff_mul(gi, sn)};
  return L;
}

// t^e (e >= 1) for a normalised positive scalar, exponent tracked in te.
__device__ __forceinline__ void ff_pow_scalar(ff t, int te, int e, ff& out, int& oute) {
  bool first = true;
  while (e > 0) {
    if (e & 1) {
      if (first) {
        out = t;
        oute = te;
        first = false;
      } else {
        out = ff_mul(out, t);
        oute += te;
        ff_normalize_scalar(out, oute);
      }
    }
    e >>= 1;
    if (e) {
      t = ff_mul(t, t);
      te *= 2;
      ff_normalize_scalar(t, te);
    }
  }
}

// The step matrix from the medium of factor q into qj through a layer of
// phase ph (as layer_step_ff): [[a em, b ep], [b em, a ep]], a = q + qj,
// b = q - qj.
__device__ __forceinline__ cmff step_matrix(const cff& q, const cff& qj, const LayerPhase& ph) {
  const cff a = cff_add(q, qj), b = cff_sub(q, qj);
  return cmff{cff_mul(a, ph.em), cff_mul(b, ph.ep), cff_mul(b, ph.em), cff_mul(a, ph.ep)};
}

// The same step matrix applied to a column vector.
__device__ __forceinline__ cvff step_apply(const cff& q, const cff& qj, const LayerPhase& ph,
                                           const cvff& v) {
  const cff a = cff_add(q, qj), b = cff_sub(q, qj);
  const cff x = cff_mul(ph.em, v.x), y = cff_mul(ph.ep, v.y);
  return cvff{cff_dot2(a, x, b, y), cff_dot2(b, x, a, y)};
}

// First column of the step matrix of an interface alone: (q + qj, q - qj).
__device__ __forceinline__ cvff step_column(const cff& q, const cff& qj) {
  return cvff{cff_add(q, qj), cff_sub(q, qj)};
}

// The transmission factor's term 4 |q|^2 of a step out of the medium q.
__device__ __forceinline__ void t_step(ff& t, int& te, const cff& q) {
  t = ff_mul(t, ff_scale2(cff_abs2(q), 4.f));
  ff_normalize_scalar(t, te);
}

// R and T of one polarisation of [A, B] x periods on a substrate, given the
// media factors q0 (ambient), qa, qb, qs and the two layers' phases.  The
// product of the step matrices, M = T1 T2 (T3 T4)^(periods - 1) Ts (first
// period from the ambient, the repeated period from its own last medium,
// then the substrate: multilayer_pol_ff's order), enters R = |M10 / M00|^2
// and T only through its first column M e1, so it is evaluated from the
// right as matrix-vector products: only the period matrix P = T3 T4 is
// formed, and P^(periods - 1) is applied by squaring P.  A layer too opaque
// to propagate through (|exp(-i beta)| >= 1e10) ends the product at its
// interface and the stack transmits nothing, as in the sequential form.
__device__ __forceinline__ void bilayer_pol_ff(const cff& q0, const cff& qa, const cff& qb,
                                               const cff& qs, const LayerPhase& A,
                                               const LayerPhase& B, int periods, float& R,
                                               float& T) {
  cvff u;
  int ue = 0;
  ff t = ff_of(1.f);
  int te = 0;
  bool where = true;
  if (periods <= 0) {
    u = step_column(q0, qs);
    t_step(t, te, q0);
  } else if (!A.prop) {
    u = step_column(q0, qa);
    where = false;
  } else if (!B.prop) {
    u = step_apply(q0, qa, A, step_column(qa, qb));
    where = false;
  } else {
    u = step_column(qb, qs);  // Ts e1
    const int reps = periods - 1;
    if (reps > 0) {
      cmff P = cmff_mul(step_matrix(qb, qa, A), step_matrix(qa, qb, B));
      int pe = 0;
      cmff_normalize(P, pe);
      for (int e = reps;;) {
        if (e & 1) {
          u = cmff_apply(P, u);
          ue += pe;
          cvff_normalize(u, ue);
        }
        e >>= 1;
        if (!e) break;
        P = cmff_sqr(P);
        pe *= 2;
        cmff_normalize(P, pe);
      }
      ff pt = ff_of(1.f);
      int pte = 0;
      t_step(pt, pte, qb);
      t_step(pt, pte, qa);
      ff_pow_scalar(pt, pte, reps, t, te);
    }
    u = step_apply(qa, qb, B, u);
    cvff_normalize(u, ue);
    u = step_apply(q0, qa, A, u);
    cvff_normalize(u, ue);
    t_step(t, te, q0);  // first period and substrate steps
    t_step(t, te, qa);
    t_step(t, te, qb);
  }
  const ff m11 = cff_abs2(u.x);
  R = ff_to_f(ff_div(cff_abs2(u.y), m11));
  T = 0.f;
  if (where) {
    const ff ratio = cff_div(qs, q0).re;
    const ff tt = ff_mul(ff_div(t, m11), ratio);
    T = ldexpf(ff_to_f(tt), te - 2 * ue);
  }
}

// Medium factor n cos of the medium of index nj for the ambient's
// invariant inv0 = (n0 sin0)^2 (the s factor q_s).
__device__ __forceinline__ cff medium_w_ff(const cff& inv0, cf nj_f) {
  const cff nj = cff_of(nj_f.re, nj_f.im);
  const cff cj = cff_sqrt(cff_sub(cff_of(1.f, 0.f), cff_div(inv0, cff_mul(nj, nj))));
  return cff_mul(nj, cj);
}

// p factor conj(q_s) / |n|^2 from the s factor.
__device__ __forceinline__ cff p_factor(const cff& w, cf nj_f) {
  return cff_scale(cff_conj(w), ff_div(ff_of(1.f), cff_abs2(cff_of(nj_f.re, nj_f.im))));
}

// R and T of one polarisation of a periodic bilayer mirror, two lanes per
// sample: the even lane of a lane pair takes s, the odd lane p.  The even
// lane evaluates layer A's medium factor and phase, the odd lane layer B's,
// and the pair exchanges them by shuffles (both lanes of a pair always run
// together); each lane then forms its own polarisation's product: half the
// state of one thread evaluating both polarisations, twice the threads.
__device__ __forceinline__ void periodic_bilayer_lane_ff(const otx_periodic_stack& P, float wl,
                                                         float cos0, cf n0, float& R, float& T) {
  const int lane = threadIdx.x & 31;
  const bool odd = lane & 1;
  const unsigned pair = 3u << (lane & ~1);
  const cff n0c = cff_of(n0.re, n0.im);
  const ff one_m_c2 = ff_sub(ff_of(1.f), ff_mul(ff_of(cos0), ff_of(cos0)));
  const cff inv0 = cff_scale(cff_mul(n0c, n0c), one_m_c2);
  const cf na{P.n_a_re, P.n_a_im}, nb{P.n_b_re, P.n_b_im}, ns{P.n_sub_re, P.n_sub_im};
  // this lane's layer: A on even lanes, B on odd lanes
  const cf nl = odd ? nb : na;
  const cff wl_mine = medium_w_ff(inv0, nl);
  const LayerPhase ph = layer_phase_ff(wl_mine, odd ? P.thickness_b : P.thickness_a, wl);
  const cff ws = medium_w_ff(inv0, ns);
  auto xch = [&](float v) { return __shfl_xor_sync(pair, v, 1); };
  const cff w_other{{xch(wl_mine.re.hi), xch(wl_mine.re.lo)}, {xch(wl_mine.im.hi), xch(wl_mine.im.lo)}};
  LayerPhase po;
  po.em = cff{{xch(ph.em.re.hi), xch(ph.em.re.lo)}, {xch(ph.em.im.hi), xch(ph.em.im.lo)}};
  po.ep = cff{{xch(ph.ep.re.hi), xch(ph.ep.re.lo)}, {xch(ph.ep.im.hi), xch(ph.ep.im.lo)}};
  po.prop = __shfl_xor_sync(pair, (int)ph.prop, 1) != 0;
  const cff wa = odd ? w_other : wl_mine, wb = odd ? wl_mine : w_other;
  const LayerPhase& A = odd ? po : ph;
  const LayerPhase& B = odd ? ph : po;
  cff q0, qa, qb, qs;
  if (!odd) {
    q0 = cff_scale(n0c, ff_of(cos0));
    qa = wa;
    qb = wb;
    qs = ws;
  } else {
    q0 = cff_scale(cff_conj(n0c), ff_div(ff_of(cos0), cff_abs2(n0c)));
    qa = p_factor(wa, na);
    qb = p_factor(wb, nb);
    qs = p_factor(ws, ns);
  }
  bilayer_pol_ff(q0, qa, qb, qs, A, B, P.num_periods, R, T);
}

}  // namespace otx
