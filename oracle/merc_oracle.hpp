// merc_oracle.hpp - CPU oracle of the Mercurius step.  TEST INFRASTRUCTURE.
//
// This file is the checker, never the product: only tests, the smoke check
// and the CPU-baseline leg of bench.py load it (through liboracle.so).  The
// GPU library never links it and never falls back to it.
//
// It restates the reference step (at2005/p9-integrator, src/sim.cuh) in plain
// C++, templated on the real type R so that the same algorithm runs in binary64
// (parity oracle) and in long double (energy-error reference).  Every function
// cites the reference lines it follows.  Operation order and the explicit fma
// calls of the reference are kept, and the file is compiled with
// -ffp-contract=off, so that the double instantiation reproduces the
// reference arithmetic; where the reference is racy (its democratic-
// heliocentric conversion and its kicks read velocities that other threads
// are overwriting, sim.cuh:677,684-685,740-741,748) the oracle defines the
// race-free order "read every source, then write".
//
// The universal-variable drift (drift == 1) is the new formulation of the GPU
// library; it has no reference counterpart.  It is restated here with the same
// explicit-fma arithmetic as the CUDA kernel so both produce the same bits.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../p9-integrator_gb300/csrc/merc_math.h"

namespace oracle {

constexpr double kTwoPiD = 6.283185307179586476925286766559005768394338798750211641949;

struct Params {
  double dt = 0.8219;
  double softening2 = 1e-8;
  double hill_factor = 1.0;
  double kepler_tol = 1e-13;
  double eject_r = 0.0;
  int kepler_iters = 8;
  int bs_rows = 3;
  int compat_block = 0;
  int drift = 0;
  int kepler_max_iter = 30;
  int warm_start = 0;
};

template <class R> struct V3 { R x, y, z; };

// Math of the host C library, with the CUDA-only helpers the reference uses
// expressed in IEEE operations: rsqrt(x) = 1/sqrt(x), norm3d = sqrt of the fma
// chain.  Long double picks the long double overloads.
struct StdMath {
  template <class R> static R sqrt(R x) { return std::sqrt(x); }
  template <class R> static R rsqrt(R x) { return R(1) / std::sqrt(x); }
  template <class R> static R norm3d(R a, R b, R c) { return std::sqrt(std::fma(a, a, std::fma(b, b, c * c))); }
  template <class R> static void sincos(R x, R* s, R* c) { *s = std::sin(x); *c = std::cos(x); }
  template <class R> static R sin(R x) { return std::sin(x); }
  template <class R> static R cos(R x) { return std::cos(x); }
  template <class R> static R sinh(R x) { return std::sinh(x); }
  template <class R> static R cosh(R x) { return std::cosh(x); }
  template <class R> static R acos(R x) { return std::acos(x); }
  template <class R> static R atan2(R y, R x) { return std::atan2(y, x); }
  template <class R> static R log(R x) { return std::log(x); }
  template <class R> static R cbrt(R x) { return std::cbrt(x); }
};

// The elementary functions of the GPU library (merc_math.h: only IEEE
// operations, so host and device evaluate them to the same bits).  With this
// policy the double oracle and the CUDA kernels agree bit for bit; with
// StdMath it agrees bit for bit with the reference source compiled for the
// host.  Both are restatements of the same algorithm.
struct MercMath {
  static double sqrt(double x) { return std::sqrt(x); }
  static double rsqrt(double x) { return 1.0 / std::sqrt(x); }
  static double norm3d(double a, double b, double c) { return std::sqrt(std::fma(a, a, std::fma(b, b, c * c))); }
  static void sincos(double x, double* s, double* c) { mm::sincos(x, s, c); }
  static double sin(double x) { return mm::sin(x); }
  static double cos(double x) { return mm::cos(x); }
  static double sinh(double x) { return mm::sinh(x); }
  static double cosh(double x) { return mm::cosh(x); }
  static double acos(double x) { return mm::acos(x); }
  static double atan2(double y, double x) { return mm::atan2(y, x); }
  static double log(double x) { return mm::log(x); }
  static double cbrt(double x) { return mm::cbrt(x); }
};

template <class R> inline R two_pi() { return R(kTwoPiD); }
template <> inline long double two_pi<long double>() {
  return 6.283185307179586476925286766559005768394338798750211641949L;
}

// ---- helpers: reference src/sim.cuh:28-87 ------------------------------
template <class R> inline R mag2(const V3<R>& a) {  // sim.cuh:42-48
  return std::fma(a.x, a.x, std::fma(a.y, a.y, a.z * a.z));
}
template <class R> inline V3<R> cross(const V3<R>& a, const V3<R>& b) {  // sim.cuh:28-33
  return {std::fma(a.y, b.z, -a.z * b.y), std::fma(a.z, b.x, -a.x * b.z), std::fma(a.x, b.y, -a.y * b.x)};
}
template <class R, class M> inline R stable_sqrt(R x) { return M::sqrt(x * R(x >= R(0))); }  // :35-40
template <class R, class M> inline R stable_log(R x) {                                      // :57-62
  return M::log(x * R(x > R(0)) + R(x <= R(0)));
}
template <class R, class M> inline R stable_acos(R x) {  // :64-72
  R alto = R(std::fabs(x) <= R(1));
  return M::acos(std::fma(x, alto, std::copysign(R(1) - alto, x)));
}
template <class R> inline R stable_div(R x, R y) {  // :81-87
  R etz = R(y == R(0)), netz = R(y != R(0));
  return (netz * x) / (y + etz);
}

// ---- Kepler's equation, Danby/Burkardt, fixed iterations: sim.cuh:90-126 ----
template <class R, class M> R danby(R mean_anomaly, R e, int iters) {
  R E = mean_anomaly;
  for (int i = 0; i < iters; i++) {
    R s, c;
    M::sincos(E, &s, &c);
    R lt1 = R(e < R(1)), gt1 = R(e > R(1));
    // the reference evaluates both branches and blends them (sim.cuh:100-101)
    s = lt1 * s + gt1 * M::sinh(E);
    c = lt1 * c + gt1 * M::cosh(E);
    R esin = e * s;
    R sign = std::copysign(R(1), e - R(1));
    R f = (sign * mean_anomaly) - esin + E;
    R ecos = e * c;
    R fp = R(1) - ecos;
    R dE = -f / fp;
    if (i > iters - 2) {  // last iteration: cubic, quartic, quintic corrections (:112-121)
      dE = -f / (fp + dE * esin / R(2));
      dE = -f / ((fp + dE * esin / R(2)) + (dE * dE * ecos / R(6)));
      dE = -f / ((fp + dE * esin / R(2)) + (dE * dE * ecos / R(6)) - (dE * dE * dE * esin / R(24)));
    }
    E += dE;
  }
  return E;
}

template <class R> struct PV { V3<R> pos, vel; };

// ---- elements -> cartesian, mu = 1: sim.cuh:188-239 ----------------------
template <class R, class M>
PV<R> cart_from_elem(R inc, R node, R peri, R mean_anomaly, R e, R a, int iters) {
  R si, ci, so, co, sa, ca;
  M::sincos(inc, &si, &ci);
  M::sincos(node, &so, &co);
  M::sincos(peri, &sa, &ca);
  R z1 = ca * co, z2 = ca * so, z3 = sa * co, z4 = sa * so;
  R d11 = std::fma(-z4, ci, z1), d12 = std::fma(z3, ci, z2), d13 = sa * si;
  R d21 = std::fma(-z2, ci, -z3), d22 = std::fma(z1, ci, -z4), d23 = ca * si;
  R romes = stable_sqrt<R, M>(std::copysign(R(1), e - R(1)) * std::fma(e, e, R(-1)));
  R gt1 = R(e > R(1)), lt1 = R(e < R(1));
  R E = danby<R, M>(mean_anomaly, e, iters);
  R sE, cE;
  M::sincos(E, &sE, &cE);
  sE = std::fma(lt1, sE, gt1 * M::sinh(E));
  cE = std::fma(lt1, cE, gt1 * M::cosh(E));
  z1 = a * (cE - e);
  z2 = std::copysign(R(1), R(1) - e) * a * romes * sE;
  R q = stable_div(stable_sqrt<R, M>(stable_div(R(1), std::fabs(a))),
                   std::copysign(R(1), R(1) - e) * (std::fma(-e, cE, R(1))));
  z3 = -sE * q;
  z4 = romes * cE * q;
  PV<R> r;
  r.pos = {std::fma(d11, z1, d21 * z2), std::fma(d12, z1, d22 * z2), std::fma(d13, z1, d23 * z2)};
  r.vel = {std::fma(d11, z3, d21 * z4), std::fma(d12, z3, d22 * z4), std::fma(d13, z3, d23 * z4)};
  return r;
}

template <class R> struct Elem { R inc, node, peri, M, e, a; };

// ---- cartesian -> elements, mu = 1: sim.cuh:241-324 ----------------------
template <class R, class M> Elem<R> elem_from_cart(const V3<R>& p, const V3<R>& v) {
  const R tp = two_pi<R>();
  V3<R> h = cross(p, v);
  R h_sq = mag2(h) + R(1e-8);
  R inc = stable_acos<R, M>(h.z * M::rsqrt(h_sq));
  R node = M::atan2(h.x, -h.y);
  R r_v = std::fma(p.x, v.x, std::fma(p.y, v.y, (p.z * v.z)));
  R v_sq = mag2(v);
  R r = M::norm3d(p.x, p.y, p.z);
  R s = h_sq;
  R e = stable_sqrt<R, M>(std::fma(s, v_sq - (R(2) / r), R(1)));
  R q = s / (R(1) + e);
  R cos_i = M::cos(inc);
  R to = stable_div(-h.x, h.y);
  R temp = (R(1) - cos_i) * to;
  R etz = R(h.y == R(0)), netz = R(h.y != R(0));
  R temp2 = std::fma(netz, to * to, etz);
  R true_long = M::atan2((std::fma(p.y, std::fma(temp2, cos_i, (netz * R(1))), -p.x * temp)),
                         std::fma(p.x, std::fma(netz, cos_i, temp2), -p.y * temp));
  etz = R(e == R(0));
  netz = R(e != R(0));
  R cosE = stable_div(std::fma(v_sq, r, R(-1)), e);
  R E = stable_acos<R, M>(cosE);
  R rv_lt0 = R(r_v < R(0));
  E = std::fma(rv_lt0, tp, std::copysign(E, r_v));
  R Ma = netz * std::fma(-e, M::sin(E), E) + etz * true_long;
  R gt1 = R(e > R(1)), lt1 = R(e < R(1));
  E = std::fma(gt1, stable_log<R, M>(cosE + stable_sqrt<R, M>(std::fma(cosE, cosE, R(-1)))), lt1 * E);
  E = std::fma(gt1, std::copysign(E, r_v), lt1 * E);
  Ma = std::fma(gt1, std::fma(e, M::sinh(E), -E), lt1 * Ma);
  R cos_f = stable_div((s - r), (e * r));
  R f = stable_acos<R, M>(cos_f);
  f = std::fma(rv_lt0, tp, std::copysign(f, r_v));
  R pp = true_long - f;
  pp = netz * std::fmod(pp + tp + tp, tp);
  R M_lt0 = R(Ma < R(0));
  Ma = std::fma(M_lt0, tp, Ma);
  Ma = std::fmod(Ma, tp);
  Elem<R> out;
  out.inc = inc;
  out.node = node;
  out.peri = pp - node;
  out.M = Ma;
  out.e = e;
  out.a = q / (R(1) - e);
  return out;
}

// A gravitating source as seen by the kick: position, mass and changeover
// radius r_crit (computed once per phase from the source state).
template <class R> struct Src { V3<R> x; R m, rc; };

// ---- r_crit = hill_factor * a * cbrt(m/3), a from h and e: sim.cuh:133-164 ----
// (the shipped source calls an undefined magnitude(); its intent, sqrt of the
// squared magnitude, is used)
template <class R, class M> R rcrit(const V3<R>& r, const V3<R>& v, R m, R hill_factor) {
  V3<R> h = {std::fma(r.y, v.z, -r.z * v.y), std::fma(r.z, v.x, -r.x * v.z), std::fma(r.x, v.y, -r.y * v.x)};
  R h2 = mag2(h);
  R rmag = M::sqrt(mag2(r));
  R v2 = mag2(v);
  R rdv = std::fma(r.x, v.x, std::fma(r.y, v.y, r.z * v.z));
  R factor = v2 - R(1) / rmag;
  V3<R> ev = {std::fma(factor, r.x, -rdv * v.x), std::fma(factor, r.y, -rdv * v.y),
              std::fma(factor, r.z, -rdv * v.z)};
  R e2 = mag2(ev);
  R a = h2 / (R(1) - e2);
  return a * (M::cbrt(m / R(3)) * hill_factor);
}

// ---- K-weighted kick of one body: body_interaction_kick sim.cuh:327-382 with
// changeover sim.cuh:166-186.  `self` is the source index the body excludes
// (its own index, or threadIdx.x of the reference with compat_block). ----
template <class R, class M>
V3<R> kick(const V3<R>& pos, V3<R> vel, int self, const Src<R>* src, int nm, R dt, bool bs, R soft2) {
  V3<R> acc = {R(0), R(0), R(0)};
  for (int i = 0; i < nm; i++) {
    V3<R> d = {src[i].x.x - pos.x, src[i].x.y - pos.y, src[i].x.z - pos.z};
    R r_sq = mag2(d);
    R r = stable_sqrt<R, M>(r_sq);
    R rc = src[i].rc;
    R notself = R(self != i);
    R r_ij = notself * M::norm3d(d.x, d.y, d.z);
    R y = (r_ij - R(0.1) * rc) / (R(0.9) * rc);
    R K = y * y / (R(2) * y * y - R(2) * y + R(1));
    R gtz = R(y > R(0)), gto = R(y > R(1)), valid = R(y <= R(1) && y >= R(0));
    K = K * gtz * valid + gto;
    R w = K;
    if (bs) w = R(r <= rc) * (R(1) - K) + R(r > rc) * K;  // sim.cuh:357-361
    r_sq += notself * soft2;
    R denom = r_sq * r;
    R wa = w * stable_div(src[i].m, denom);
    acc.x = std::fma(wa, d.x, acc.x);
    acc.y = std::fma(wa, d.y, acc.y);
    acc.z = std::fma(wa, d.z, acc.z);
  }
  vel.x = std::fma(acc.x, dt, vel.x);
  vel.y = std::fma(acc.y, dt, vel.y);
  vel.z = std::fma(acc.z, dt, vel.z);
  return vel;
}

// ---- encounter sub-stepper: sim.cuh:410-551 ----------------------------
template <class R, class M>
V3<R> vel_total(const V3<R>& pos, const V3<R>& vel, int self, const Src<R>* src, int nm, R dt, R soft2) {
  V3<R> nv = kick<R, M>(pos, vel, self, src, nm, dt, true, soft2);  // :425
  R r_sq = mag2(pos);
  R r = stable_sqrt<R, M>(r_sq);
  r_sq += soft2;
  R denom = r_sq * r;
  V3<R> rv = {pos.x / denom, pos.y / denom, pos.z / denom};
  nv.x = std::fma(-rv.x, dt, nv.x);
  nv.y = std::fma(-rv.y, dt, nv.y);
  nv.z = std::fma(-rv.z, dt, nv.z);
  return nv;
}

template <class R, class M>
PV<R> mod_midpoint(PV<R> c, int self, const Src<R>* src, int nm, R dt, int N, R soft2) {  // :445-500
  R h = dt / R(N);
  V3<R> z1 = c.pos;
  z1.x = std::fma(c.vel.x, h, z1.x);
  z1.y = std::fma(c.vel.y, h, z1.y);
  z1.z = std::fma(c.vel.z, h, z1.z);
  R h2 = R(2) * h;
  V3<R> z0 = c.pos;
  c.pos = z1;
  c.vel = vel_total<R, M>(c.pos, c.vel, self, src, nm, h, soft2);
  for (int i = 1; i < N; i++) {
    V3<R> t = {std::fma(h2, c.vel.x, z0.x), std::fma(h2, c.vel.y, z0.y), std::fma(h2, c.vel.z, z0.z)};
    z0 = z1;
    z1 = t;
    c.pos = z1;
    c.vel = vel_total<R, M>(c.pos, c.vel, self, src, nm, h, soft2);
  }
  PV<R> res;
  res.pos = {R(0.5) * (z1.x + std::fma(c.vel.x, h, z0.x)), R(0.5) * (z1.y + std::fma(c.vel.y, h, z0.y)),
             R(0.5) * (z1.z + std::fma(c.vel.z, h, z0.z))};
  res.vel = c.vel;
  return res;
}

template <class R, class M>
PV<R> richardson(const PV<R>& c, int self, const Src<R>* src, int nm, R dt, int rows, R soft2) {  // :502-551
  PV<R> b[4][4];
  int N = 1;
  b[0][0] = mod_midpoint<R, M>(c, self, src, nm, dt, N, soft2);
  for (int i = 1; i < rows; i++) {
    N <<= 1;
    b[i][0] = mod_midpoint<R, M>(c, self, src, nm, dt, N, soft2);
    for (int j = 1; j <= i; j++) {
      R p4 = std::pow(R(4), R(j));
      R den = p4 - R(1);
      PV<R>& o = b[i][j];
      const PV<R>& a = b[i][j - 1];
      const PV<R>& q = b[i - 1][j - 1];
      o.pos = {std::fma(p4, a.pos.x, -q.pos.x) / den, std::fma(p4, a.pos.y, -q.pos.y) / den,
               std::fma(p4, a.pos.z, -q.pos.z) / den};
      o.vel = {std::fma(p4, a.vel.x, -q.vel.x) / den, std::fma(p4, a.vel.y, -q.vel.y) / den,
               std::fma(p4, a.vel.z, -q.vel.z) / den};
    }
  }
  return b[rows - 1][rows - 1];
}

// ---- universal-variable drift (new formulation; no reference counterpart) ----
// Stumpff functions c0..c3 of z by quartering z until |z| <= 0.1, a 7-term
// Taylor series (Horner) for c2 and c3 (3 terms in binary64 when |z| < 5e-5,
// where the z^3 terms are below 1e-17 relative), then the doubling identities
//   c0(4z) = 2 c0^2 - 1, c1(4z) = c0 c1, c2(4z) = c1^2 / 2, c3(4z) = (c2 + c0 c3) / 4
// (Stumpff; Danby, Fundamentals of Celestial Mechanics, 2nd ed., sec. 6.9).
// Shared bit for bit with the CUDA kernel: only +, *, fma and one division.
template <class R> inline void stumpff(R z, R* c0, R* c1, R* c2, R* c3) {
  // Taylor coefficients (-1)^k/(2k+3)! of c3 and (-1)^k/(2k+2)! of c2
  const R a0 = R(1) / R(6), a1 = R(-1) / R(120), a2 = R(1) / R(5040), a3 = R(-1) / R(362880),
          a4 = R(1) / R(39916800), a5 = R(-1) / R(6227020800.0), a6 = R(1) / R(1307674368000.0);
  const R b0 = R(1) / R(2), b1 = R(-1) / R(24), b2 = R(1) / R(720), b3 = R(-1) / R(40320),
          b4 = R(1) / R(3628800), b5 = R(-1) / R(479001600), b6 = R(1) / R(87178291200.0);
  int k = 0;
  while (std::fabs(z) > R(0.1) && k < 60) {
    z = z * R(0.25);
    k++;
  }
  R s3, s2;
  if (sizeof(R) == sizeof(double) && std::fabs(z) < R(5e-5)) {
    // binary64: the z^3 terms are below 1e-17 relative here
    s3 = std::fma(z, std::fma(z, a2, a1), a0);
    s2 = std::fma(z, std::fma(z, b2, b1), b0);
  } else {
    s3 = std::fma(z, std::fma(z, std::fma(z, std::fma(z, std::fma(z, std::fma(z, a6, a5), a4), a3), a2), a1), a0);
    s2 = std::fma(z, std::fma(z, std::fma(z, std::fma(z, std::fma(z, std::fma(z, b6, b5), b4), b3), b2), b1), b0);
  }
  R s1 = std::fma(-z, s3, R(1));
  R s0 = std::fma(-z, s2, R(1));
  for (; k > 0; k--) {
    R n3 = std::fma(s0, s3, s2) * R(0.25);
    R n2 = s1 * s1 * R(0.5);
    R n1 = s0 * s1;
    R n0 = std::fma(R(2) * s0, s0, R(-1));
    s0 = n0; s1 = n1; s2 = n2; s3 = n3;
  }
  *c0 = s0; *c1 = s1; *c2 = s2; *c3 = s3;
}

template <class R> struct UDrift { PV<R> out; int iters; bool converged; R s; };

// Universal-variable Kepler drift with mu = 1: solve
//   r0 s + eta G2(s) + zeta G3(s) = dt,  G_k = s^k c_k(alpha s^2),
// alpha = 2/r0 - v0^2, eta = x0.v0, zeta = 1 - alpha r0, by Newton from s0
// (Laguerre-Conway steps with n = 5 after 8 Newton steps without convergence:
// Newton can oscillate on drifts long against the pericentre passage).
// Stopping rule: after the update s += ds, the Newton error estimate of the
// new s is |f''/(2 f')| ds^2; stop when it is <= tol |s| (and |ds| <= 1e-3 |s|,
// so the estimate is only trusted in the quadratic regime).  The f and g
// functions are then evaluated at the final s.
template <class R>
UDrift<R> universal_drift(const V3<R>& x0, const V3<R>& v0, R dt, R s0, R tol, int max_iter) {
  constexpr int kNewtonIters = 8;
  R r0 = std::sqrt(mag2(x0));
  R ir0 = R(1) / r0;
  R eta = std::fma(x0.x, v0.x, std::fma(x0.y, v0.y, x0.z * v0.z));
  R v2 = mag2(v0);
  R alpha = std::fma(R(2), ir0, -v2);
  R zeta = std::fma(-alpha, r0, R(1));
  R s = s0;
  int it = 0;
  bool conv = false;
  R c0, c1, c2, c3;
  while (it < max_iter) {
    R s2 = s * s;
    stumpff(alpha * s2, &c0, &c1, &c2, &c3);
    R G1 = s * c1, G2 = s2 * c2, G3 = s2 * s * c3;
    R f = std::fma(r0, s, std::fma(eta, G2, std::fma(zeta, G3, -dt)));
    R fp = std::fma(eta, G1, std::fma(zeta, G2, r0));
    R fpp = std::fma(eta, c0, zeta * G1);
    R ds;
    if (it < kNewtonIters) {
      ds = -f / fp;
    } else {  // Laguerre-Conway step (n = 5) after kNewtonIters Newton steps
      const R h = std::fabs(std::fma(R(16) * fp, fp, -R(20) * f * fpp));
      ds = -R(5) * f / (fp + std::sqrt(h));
    }
    s = s + ds;
    it++;
    R as = std::fabs(s);
    if (std::fabs(ds) <= R(1e-3) * as && std::fabs(fpp * ds * ds) <= R(2) * tol * as * std::fabs(fp)) {
      conv = true;
      break;
    }
  }
  R s2 = s * s;
  stumpff(alpha * s2, &c0, &c1, &c2, &c3);
  R G1 = s * c1, G2 = s2 * c2, G3 = s2 * s * c3;
  R r = std::fma(eta, G1, std::fma(zeta, G2, r0));
  R ir = R(1) / r;
  R f = std::fma(-G2, ir0, R(1));
  R g = dt - G3;
  R fd = -G1 * ir0 * ir;
  R gd = std::fma(-G2, ir, R(1));
  UDrift<R> u;
  u.out.pos = {std::fma(f, x0.x, g * v0.x), std::fma(f, x0.y, g * v0.y), std::fma(f, x0.z, g * v0.z)};
  u.out.vel = {std::fma(fd, x0.x, gd * v0.x), std::fma(fd, x0.y, gd * v0.y), std::fma(fd, x0.z, gd * v0.z)};
  u.iters = it;
  u.converged = conv;
  u.s = s;
  return u;
}

// Plain initial guess of the universal solve: s0 = dt / r0.
template <class R> inline R plain_guess(const V3<R>& x0, R dt) { return dt / std::sqrt(mag2(x0)); }

// Series guess: the universal Kepler equation t = r0 s + eta s^2/2 + zeta s^3/6
// + O(s^4) inverted to third order in t,
//   s = s0 (1 - (eta / (2 r0)) s0 + ((3 eta^2 - r0 zeta) / (6 r0^2)) s0^2),  s0 = t / r0,
// (the second-order part is the usual small-dt guess of Wisdom-Holman codes);
// kept only when it lies within a factor 2 of s0.
template <class R> inline R series_guess(const V3<R>& x0, const V3<R>& v0, R dt) {
  R r0 = std::sqrt(mag2(x0));
  R ir0 = R(1) / r0;
  R eta = std::fma(x0.x, v0.x, std::fma(x0.y, v0.y, x0.z * v0.z));
  R v2 = mag2(v0);
  R zeta = std::fma(-std::fma(R(2), ir0, -v2), r0, R(1));
  R s0 = dt * ir0;
  R a1 = R(0.5) * eta * ir0;
  R a2 = std::fma(R(3) * eta, eta, -r0 * zeta) * (ir0 * ir0) * (R(1) / R(6));
  R g = s0 * std::fma(s0, std::fma(s0, a2, -a1), R(1));
  return (g > R(0.5) * s0 && g < R(2) * s0) ? g : s0;
}

}  // namespace oracle
