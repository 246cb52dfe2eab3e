// merc_device.cuh - per-body device physics of the Mercurius step.
//
// Each function is the GPU form of one stage of the reference step
// (at2005/p9-integrator src/sim.cuh); the cited lines give the formula.  The
// translation unit is compiled with -fmad=false so that a*b+c is never fused
// implicitly: the explicit fma() calls below are exactly those of the
// reference, and together with merc_math.h every stage evaluates to the same
// bits as the CPU check of the same algorithm.
#pragma once
#include <stdint.h>

#include "merc_math.h"

namespace merc {

struct d3 {
  double x, y, z;
};

__device__ __forceinline__ double mag2(const d3& a) { return fma(a.x, a.x, fma(a.y, a.y, a.z * a.z)); }
// The reference's guarded division and square root, (netz x) / (y + etz)
// and sqrt(x (x >= 0)).  Where the guard's factor is 1 and its addend 0 they
// change nothing (1 x = x and y + 0 = y exactly for y != 0, NaN kept), so
// those cases skip the two operations; the others keep them.
// The guards' tests on the bit patterns (integer operations; an FP64 compare
// takes a slot of the FP64 pipe on this GPU): y != 0 is "not +-0" (NaN
// included, as in the compare), x >= 0 is "+0..+inf or -0" (NaN excluded).
__device__ __forceinline__ double stable_div(double x, double y) {  // sim.cuh:81-87
  return (__double_as_longlong(y) << 1) != 0 ? x / y : (0.0 * x) / (y + 1.0);
}
__device__ __forceinline__ double stable_sqrt(double x) {  // :35-40
  const long long b = __double_as_longlong(x);
  const bool ge0 = (b >= 0 && b <= 0x7ff0000000000000LL) || b == (long long)0x8000000000000000ULL;
  return sqrt(ge0 ? x : x * 0.0);
}

// Unit constants read at run time (kernel parameters): fma(one, a, b) and
// fma(a, b, nz) with one = 1 and nz = -0 give exactly a + b and a * b (the
// negative zero keeps the sign of a zero product), and run at the FP64 FMA
// rate, which on this GPU is about 19% above that of DADD and DMUL (measured).
// A compile-time 1 or 0 would be folded back into DADD / DMUL.
struct FU {
  double one, nz;
};
__device__ __forceinline__ double fadd(const FU& U, double a, double b) { return fma(U.one, a, b); }
__device__ __forceinline__ double fsub(const FU& U, double a, double b) { return fma(U.one, a, -b); }
__device__ __forceinline__ double fmul(const FU& U, double a, double b) { return fma(a, b, U.nz); }

// 1 / N for N = 2^k (k < 1023), built from the exponent bits: x * inv_pow2(N)
// equals x / N bit for bit without a division.
__device__ __forceinline__ double inv_pow2(int N) { return __hiloint2double((1023 - (__ffs(N) - 1)) << 20, 0); }
__device__ __forceinline__ double stable_log(double x) {                                         // :57-62
  return mm::log(x * (double)(x > 0.0) + (double)(x <= 0.0));
}
__device__ __forceinline__ double stable_acos(double x) {  // :64-72
  double alto = (double)(fabs(x) <= 1.0);
  return mm::acos(fma(x, alto, copysign(1.0 - alto, x)));
}
__device__ __forceinline__ double rsqrt_ieee(double x) { return 1.0 / sqrt(x); }

// Changeover radius of a source: hill_factor x Hill radius, a from h and e
// (sim.cuh:133-164).
// r_crit = a * hc with hc = cbrt(m / 3) * hill_factor (a per-body constant)
__device__ __forceinline__ double rcrit_hc(const d3& r, const d3& v, double hc) {
  d3 h = {fma(r.y, v.z, -r.z * v.y), fma(r.z, v.x, -r.x * v.z), fma(r.x, v.y, -r.y * v.x)};
  double h2 = mag2(h);
  double rmag = sqrt(mag2(r));
  double v2 = mag2(v);
  double rdv = fma(r.x, v.x, fma(r.y, v.y, r.z * v.z));
  double factor = v2 - 1.0 / rmag;
  d3 ev = {fma(factor, r.x, -rdv * v.x), fma(factor, r.y, -rdv * v.y), fma(factor, r.z, -rdv * v.z)};
  double e2 = mag2(ev);
  double a = h2 / (1.0 - e2);
  return a * hc;
}

// Changeover weight K(y), y = (r_ij - 0.1 rc) / (0.9 rc) (sim.cuh:176-183),
// K = y^2 / ((2 y) y - 2 y + 1) with the reference's roundings, its additions
// and products as FMAs on the run-time unit constants (each the same single
// rounding).  The common cases y > 1 (K = 1) and y < 0 (K = 0) give the same
// bits as the branch-free formula, and so does K itself for y in [0, 1]
// (K gtz valid + gto with gtz = valid = 1, gto = 0; K = +0 at y = 0); the
// rest (infinite or NaN y) takes the formula.  (Products with 0/1 factors
// and their conversions each take an FP64 slot.)
// The range tests of K(y) on the bit patterns, the same decisions as the
// compares 1 < y < DBL_MAX, -DBL_MAX < y < 0 and 0 <= y <= 1 (NaN in none)
__device__ __forceinline__ bool y_above_one(double y) {
  const long long b = __double_as_longlong(y);
  return b > 0x3ff0000000000000LL && b < 0x7fefffffffffffffLL;
}
__device__ __forceinline__ bool y_below_zero(double y) {
  const long long b = __double_as_longlong(y), m = b & 0x7fffffffffffffffLL;
  return b < 0 && m != 0 && m < 0x7fefffffffffffffLL;
}
__device__ __forceinline__ bool y_in_unit(double y) {
  const long long b = __double_as_longlong(y);
  return (b >= 0 && b <= 0x3ff0000000000000LL) || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ double changeover_K(const FU& U, double y) {
  if (y_above_one(y)) return 1.0;
  if (y_below_zero(y)) return 0.0;
  const double y2 = fmul(U, fmul(U, 2.0, y), y), d = fadd(U, fsub(U, y2, fmul(U, 2.0, y)), 1.0);
  double K = fmul(U, y, y) / d;
  if (y_in_unit(y)) return K;
  double gtz = (double)(y > 0.0), gto = (double)(y > 1.0), valid = (double)(y <= 1.0 && y >= 0.0);
  return K * gtz * valid + gto;
}

// Sources of one system as seen by the kicks: positions, mass and the two
// changeover products 0.1 rc, 0.9 rc, plus rc itself.
struct SrcView {
  const double* x;
  const double* y;
  const double* z;
  const double* m;
  const double* rc;  // rc, 0.1 rc, 0.9 rc, fast-path threshold: rc[4*i + k]
  FU u;              // run-time unit constants of the exact term's additions and products
};

// K-weighted kick of one body over the system's sources in the reference's
// order (body_interaction_kick, sim.cuh:327-382).  BS selects the encounter
// weighting (1 - K inside r_crit, sim.cuh:357-361).
// Term of source i in kick_exact: the weighted factor wa and the separation
// d, accumulated as acc = fma(wa, d, acc) in source order.
template <bool BS>
__device__ __forceinline__ double exact_term(const d3& pos, int self, const SrcView& S, int i, double soft2,
                                             d3& d) {
  // additions and products as FMAs on the run-time unit constants (the same
  // single roundings, so the same bits; an FMA issues about 19% faster than
  // DADD and DMUL on this GPU)
  const FU& U = S.u;
  d = {fsub(U, S.x[i], pos.x), fsub(U, S.y[i], pos.y), fsub(U, S.z[i], pos.z)};
  double r_sq = fma(d.x, d.x, fma(d.y, d.y, fmul(U, d.z, d.z)));
  double r = stable_sqrt(r_sq);
  double rc = S.rc[4 * i], rc01 = S.rc[4 * i + 1], rc09 = S.rc[4 * i + 2];
  // notself * r and notself * soft2 of the reference as selects: the same
  // values for finite r (a non-finite r makes the term NaN either way)
  const bool other = self != i;
  double r_ij = other ? r : 0.0;  // norm3d of d is the same sqrt of the same fma chain
  // K = changeover_K(y), y = (r_ij - rc01) / rc09.  Without the division
  // where y is certainly in (1, DBL_MAX), i.e. K = 1, decided on the bit
  // patterns (no FP64 compares): b = rc09 positive, normal and >= 2^-1000; t
  // more than 4 ulps of b above b, so t >= b (1 + 2^-51) and t / b rounds to
  // a double >= 1 + 2^-52; t below 2^996 b and finite, so t / b stays finite.
  // Where the test fails the formula gives K = 1 for such pairs too: the same
  // bits either way.
  const double t = fsub(U, r_ij, rc01);
  double K;
  const long long tb = __double_as_longlong(t), bb = __double_as_longlong(rc09);
  if (bb >= 0x0170000000000000LL && bb < 0x7ff0000000000000LL && tb > bb + 4 && tb - bb < (996LL << 52) &&
      tb < 0x7ff0000000000000LL)
    K = 1.0;
  else
    K = changeover_K(U, t / rc09);
  double w = K;
  // (r <= rc) (1 - K) + (r > rc) K: the same value (NaN where K is)
  if (BS) w = r <= rc ? fsub(U, 1.0, K) : K;
  if (other) r_sq = fadd(U, r_sq, soft2);
  const double denom = fmul(U, r_sq, r);
  return fmul(U, w, stable_div(S.m[i], denom));
}

template <bool BS>
__device__ __forceinline__ d3 kick_exact(const d3& pos, d3 vel, int self, const SrcView& S, int nm, double dt,
                                         double soft2) {
  d3 acc = {0.0, 0.0, 0.0};
  for (int i = 0; i < nm; i++) {
    d3 d;
    const double wa = exact_term<BS>(pos, self, S, i, soft2, d);
    acc.x = fma(wa, d.x, acc.x);
    acc.y = fma(wa, d.y, acc.y);
    acc.z = fma(wa, d.z, acc.z);
  }
  vel.x = fma(acc.x, dt, vel.x);
  vel.y = fma(acc.y, dt, vel.y);
  vel.z = fma(acc.z, dt, vel.z);
  return vel;
}

// acc = fma(a[k], b[k], acc) for k = 0..cnt-1 in order (cnt <= NT); a full
// chunk in unrolled blocks, so the shared-memory loads run ahead of the fma
// chain
template <int NT>
__device__ __forceinline__ double chain_fma(const double* a, const double* b, int cnt, double acc) {
  if (cnt == NT) {
#pragma unroll 16
    for (int k = 0; k < NT; k++) acc = fma(a[k], b[k], acc);
  } else {
    for (int k = 0; k < cnt; k++) acc = fma(a[k], b[k], acc);
  }
  return acc;
}

// kick_exact by one warp (every lane calls it with the same arguments and
// gets the same result): the terms of 32 sources at a time on the 32 lanes,
// staged in shared memory (4 x 32 doubles per warp), then accumulated in
// source order by lanes 0-2, one component each, with the same fma chain,
// so the bits are those of kick_exact.
template <bool BS>
__device__ __forceinline__ d3 warp_kick_exact(const d3& pos, d3 vel, int self, const SrcView& S, int nm, double dt,
                                              double soft2, double* stage) {
  const int lane = (int)(threadIdx.x & 31);
  double acc = 0.0;  // lane c < 3: component c
  for (int base = 0; base < nm; base += 32) {
    const int i = base + lane;
    d3 d = {0.0, 0.0, 0.0};
    const double wa = i < nm ? exact_term<BS>(pos, self, S, i, soft2, d) : 0.0;
    stage[lane] = wa;
    stage[32 + lane] = d.x;
    stage[64 + lane] = d.y;
    stage[96 + lane] = d.z;
    __syncwarp();
    if (lane < 3) {
      const int cnt = min(32, nm - base);
      const double* dc = stage + 32 * (lane + 1);
      acc = chain_fma<32>(stage, dc, cnt, acc);
    }
    __syncwarp();
  }
  const double ax = __shfl_sync(0xffffffffu, acc, 0), ay = __shfl_sync(0xffffffffu, acc, 1),
               az = __shfl_sync(0xffffffffu, acc, 2);
  vel.x = fma(ax, dt, vel.x);
  vel.y = fma(ay, dt, vel.y);
  vel.z = fma(az, dt, vel.z);
  return vel;
}

// close_encounter_p, sim.cuh:589-613
__device__ __forceinline__ bool ce_pair(const d3& pos, int self, const SrcView& S, int i) {
  d3 d = {S.x[i] - pos.x, S.y[i] - pos.y, S.z[i] - pos.z};
  double mag = sqrt(mag2(d));
  return (mag < S.rc[4 * i]) && (self != i);
}
__device__ __forceinline__ bool close_encounter(const d3& pos, int self, const SrcView& S, int nm) {
  bool ce = false;
  for (int i = 0; i < nm; i++) ce = ce || ce_pair(pos, self, S, i);
  return ce;
}
// the same test by one warp (the sources split over the lanes; an OR does
// not depend on the order)
__device__ __forceinline__ bool warp_close_encounter(const d3& pos, int self, const SrcView& S, int nm) {
  bool ce = false;
  for (int i = (int)(threadIdx.x & 31); i < nm; i += 32) ce = ce || ce_pair(pos, self, S, i);
  return __any_sync(0xffffffffu, ce);
}

// ---- Kepler's equation, Danby/Burkardt, fixed iterations: sim.cuh:90-126 ----
__device__ __forceinline__ double danby(double M, double e, int iters) {
  double E = M;
  const double lt1 = (double)(e < 1.0), gt1 = (double)(e > 1.0);
  const double sign = copysign(1.0, e - 1.0);
  for (int i = 0; i < iters; i++) {
    double s, c;
    mm::sincos(E, &s, &c);
    // The reference blends both branches (sim.cuh:100-101).  For e < 1 and a
    // finite sinh the hyperbolic terms enter as exact zeros, so they are only
    // evaluated when they can matter.
    double sh = 0.0, ch = 0.0;
    if (gt1 != 0.0 || !(fabs(E) < 700.0)) {
      sh = mm::sinh(E);
      ch = mm::cosh(E);
    }
    s = lt1 * s + gt1 * sh;
    c = lt1 * c + gt1 * ch;
    double esin = e * s;
    double f = (sign * M) - esin + E;
    double ecos = e * c;
    double fp = 1.0 - ecos;
    double dE = -f / fp;
    if (i > iters - 2) {
      dE = -f / (fp + dE * esin / 2.0);
      dE = -f / ((fp + dE * esin / 2.0) + (dE * dE * ecos / 6.0));
      dE = -f / ((fp + dE * esin / 2.0) + (dE * dE * ecos / 6.0) - (dE * dE * dE * esin / 24.0));
    }
    E += dE;
  }
  return E;
}

struct PV {
  d3 pos, vel;
};

// ---- elements -> cartesian, mu = 1: sim.cuh:188-239 ----
__device__ __forceinline__ PV cart_from_elem(double inc, double node, double peri, double M, double e, double a,
                                             int iters) {
  double si, ci, so, co, sa, ca;
  mm::sincos(inc, &si, &ci);
  mm::sincos(node, &so, &co);
  mm::sincos(peri, &sa, &ca);
  double z1 = ca * co, z2 = ca * so, z3 = sa * co, z4 = sa * so;
  double d11 = fma(-z4, ci, z1), d12 = fma(z3, ci, z2), d13 = sa * si;
  double d21 = fma(-z2, ci, -z3), d22 = fma(z1, ci, -z4), d23 = ca * si;
  double romes = stable_sqrt(copysign(1.0, e - 1.0) * fma(e, e, -1.0));
  double gt1 = (double)(e > 1.0), lt1 = (double)(e < 1.0);
  double E = danby(M, e, iters);
  double sE, cE;
  mm::sincos(E, &sE, &cE);
  double shE = 0.0, chE = 0.0;
  if (gt1 != 0.0 || !(fabs(E) < 700.0)) {
    shE = mm::sinh(E);
    chE = mm::cosh(E);
  }
  sE = fma(lt1, sE, gt1 * shE);
  cE = fma(lt1, cE, gt1 * chE);
  z1 = a * (cE - e);
  z2 = copysign(1.0, 1.0 - e) * a * romes * sE;
  double q = stable_div(stable_sqrt(stable_div(1.0, fabs(a))), copysign(1.0, 1.0 - e) * (fma(-e, cE, 1.0)));
  z3 = -sE * q;
  z4 = romes * cE * q;
  PV r;
  r.pos = {fma(d11, z1, d21 * z2), fma(d12, z1, d22 * z2), fma(d13, z1, d23 * z2)};
  r.vel = {fma(d11, z3, d21 * z4), fma(d12, z3, d22 * z4), fma(d13, z3, d23 * z4)};
  return r;
}

struct Elem {
  double inc, node, peri, M, e, a;
};

// ---- cartesian -> elements, mu = 1: sim.cuh:241-324 ----
__device__ __forceinline__ Elem elem_from_cart(const d3& p, const d3& v) {
  const double tp = 6.283185307179586476925286766559005768394338798750211641949;
  d3 h = {fma(p.y, v.z, -p.z * v.y), fma(p.z, v.x, -p.x * v.z), fma(p.x, v.y, -p.y * v.x)};
  double h_sq = mag2(h) + 1e-8;
  double inc = stable_acos(h.z * rsqrt_ieee(h_sq));
  double node = mm::atan2(h.x, -h.y);
  double r_v = fma(p.x, v.x, fma(p.y, v.y, (p.z * v.z)));
  double v_sq = mag2(v);
  double r = sqrt(mag2(p));
  double s = h_sq;
  double e = stable_sqrt(fma(s, v_sq - (2.0 / r), 1.0));
  double q = s / (1.0 + e);
  double cos_i = mm::cos(inc);
  double to = stable_div(-h.x, h.y);
  double temp = (1.0 - cos_i) * to;
  double etz = (double)(h.y == 0.0), netz = (double)(h.y != 0.0);
  double temp2 = fma(netz, to * to, etz);
  double true_long = mm::atan2((fma(p.y, fma(temp2, cos_i, (netz * 1.0)), -p.x * temp)),
                               fma(p.x, fma(netz, cos_i, temp2), -p.y * temp));
  etz = (double)(e == 0.0);
  netz = (double)(e != 0.0);
  double cosE = stable_div(fma(v_sq, r, -1.0), e);
  double E = stable_acos(cosE);
  double rv_lt0 = (double)(r_v < 0.0);
  E = fma(rv_lt0, tp, copysign(E, r_v));
  double Ma = netz * fma(-e, mm::sin(E), E) + etz * true_long;
  double gt1 = (double)(e > 1.0), lt1 = (double)(e < 1.0);
  if (gt1 != 0.0 || !(e < 1.0)) {  // hyperbolic (or degenerate) branch of sim.cuh:297-299
    E = fma(gt1, stable_log(cosE + stable_sqrt(fma(cosE, cosE, -1.0))), lt1 * E);
    E = fma(gt1, copysign(E, r_v), lt1 * E);
    Ma = fma(gt1, fma(e, mm::sinh(E), -E), lt1 * Ma);
  }
  double cos_f = stable_div((s - r), (e * r));
  double f = stable_acos(cos_f);
  f = fma(rv_lt0, tp, copysign(f, r_v));
  double pp = true_long - f;
  pp = netz * fmod(pp + tp + tp, tp);
  double M_lt0 = (double)(Ma < 0.0);
  Ma = fma(M_lt0, tp, Ma);
  Ma = fmod(Ma, tp);
  Elem out;
  out.inc = inc;
  out.node = node;
  out.peri = pp - node;
  out.M = Ma;
  out.e = e;
  out.a = q / (1.0 - e);
  return out;
}

// ---- encounter sub-stepper: sim.cuh:410-551 ----
// The velocity update of one sub-step (update_my_velocity_total, sim.cuh:410-
// 443) is a functor so the same Richardson scheme runs with the exact pair
// sum of the reference order (ExactVelTotal) or with the parallel fast sums of
// the universal path.
// kick_exact by a group of NT threads (threads tid = 0..NT-1 of named barrier
// `bar`; every thread of the group calls it with the same arguments and gets
// the same result): the terms of NT sources at a time, staged in shared
// memory (2 x 4 x NT + 3 doubles, two buffers so that the next chunk's terms
// are computed while threads 0-2 add the current one in source order with
// the reference's fma chain, one component each).
__device__ __forceinline__ void group_sync(int bar, int nt) {
  asm volatile("bar.sync %0, %1;" : : "r"(bar), "r"(nt) : "memory");
}
template <bool BS, int NT>
__device__ __forceinline__ d3 group_kick_exact(const d3& pos, d3 vel, int self, const SrcView& S, int nm, double dt,
                                               double soft2, double* stage, int tid, int bar) {
  double acc = 0.0;  // thread c < 3: component c
  for (int base = 0, c = 0; base < nm; base += NT, c ^= 1) {
    double* buf = stage + 4 * NT * c;
    const int i = base + tid;
    d3 d = {0.0, 0.0, 0.0};
    const double wa = i < nm ? exact_term<BS>(pos, self, S, i, soft2, d) : 0.0;
    buf[tid] = wa;
    buf[NT + tid] = d.x;
    buf[2 * NT + tid] = d.y;
    buf[3 * NT + tid] = d.z;
    // this chunk's terms are visible, and the previous chunk's additions
    // (which read the other buffer) are done
    group_sync(bar, NT);
    if (tid < 3) acc = chain_fma<NT>(buf, buf + NT * (tid + 1), min(NT, nm - base), acc);
  }
  if (tid < 3) stage[8 * NT + tid] = acc;
  group_sync(bar, NT);
  vel.x = fma(stage[8 * NT], dt, vel.x);
  vel.y = fma(stage[8 * NT + 1], dt, vel.y);
  vel.z = fma(stage[8 * NT + 2], dt, vel.z);
  return vel;
}

// NT = 1: the source sum by one thread (kick_exact); NT > 1: by a group of
// NT threads (group_kick_exact; `stage` is its shared memory, tid the
// thread's index in the group, bar its named barrier)
template <int NT = 1>
struct ExactVelTotal {
  const SrcView* S;
  int nm, self;
  double soft2;
  double* stage = nullptr;
  int tid = 0, bar = 0;
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    d3 nv = NT > 1 ? group_kick_exact<true, (NT > 1 ? NT : 32)>(pos, vel, self, *S, nm, dt, soft2, stage, tid, bar)
                   : kick_exact<true>(pos, vel, self, *S, nm, dt, soft2);
    double r_sq = mag2(pos);
    double r = stable_sqrt(r_sq);
    r_sq += soft2;
    double denom = r_sq * r;
    d3 rv = {pos.x / denom, pos.y / denom, pos.z / denom};
    nv.x = fma(-rv.x, dt, nv.x);
    nv.y = fma(-rv.y, dt, nv.y);
    nv.z = fma(-rv.z, dt, nv.z);
    return nv;
  }
};

template <class VT>
__device__ __forceinline__ PV mod_midpoint(PV c, const VT& vt, double dt, int N) {
  double h = dt * inv_pow2(N);  // = dt / N exactly (N a power of two)
  d3 z1 = c.pos;
  z1.x = fma(c.vel.x, h, z1.x);
  z1.y = fma(c.vel.y, h, z1.y);
  z1.z = fma(c.vel.z, h, z1.z);
  double h2 = 2.0 * h;
  d3 z0 = c.pos;
  c.pos = z1;
  c.vel = vt(c.pos, c.vel, h);
  for (int i = 1; i < N; i++) {
    d3 t = {fma(h2, c.vel.x, z0.x), fma(h2, c.vel.y, z0.y), fma(h2, c.vel.z, z0.z)};
    z0 = z1;
    z1 = t;
    c.pos = z1;
    c.vel = vt(c.pos, c.vel, h);
  }
  PV res;
  res.pos = {0.5 * (z1.x + fma(c.vel.x, h, z0.x)), 0.5 * (z1.y + fma(c.vel.y, h, z0.y)),
             0.5 * (z1.z + fma(c.vel.z, h, z0.z))};
  res.vel = c.vel;
  return res;
}

// x / d bit for bit, for a divisor whose reciprocal y = RN(1 / d) lies below
// 1 / d by at most 2^-54 relative (d = 3, 15, 63: 2^-54, 2^-56, 2^-54).  Then
// q = RN(x y) is within one ulp of x / d, the remainder r = x - d q is exact in
// one fma, and RN(q + r y) is the correctly rounded quotient: Markstein's
// theorem on the FMA correction of a faithful quotient (P. W. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990).  The theorem needs x / d to
// be a normal number, so |x| outside 2^-1000 .. 2^1000 takes the division;
// r = 0 keeps q, so a zero quotient keeps the sign of x.  Three FP64
// instructions instead of the division's software sequence, whose dependent
// steps made the Richardson combination of an encounter body the longest
// serial part of the encounter sub-step on this GPU's FP64 units.
__device__ __forceinline__ double div_known(double x, double d, double y) {
  const int ex = (__double2hiint(x) >> 20) & 0x7ff;
  if (ex < 1023 - 1000 || ex > 1023 + 1000) return x / d;
  const double q = x * y;
  const double r = fma(-q, d, x);
  return r == 0.0 ? q : fma(r, y, q);
}

// RN(1 / den) for the Richardson denominators 4^j - 1 of up to four rows
// (0 for any other value: the caller divides)
__device__ __forceinline__ double rich_recip(double den) {
  return den == 3.0 ? 1.0 / 3.0 : (den == 15.0 ? 1.0 / 15.0 : (den == 63.0 ? 1.0 / 63.0 : 0.0));
}

// (p4 a - q) / (p4 - 1) for one component (sim.cuh:522-544), the quotient by
// div_known: the same bits as the division
__device__ __forceinline__ double rich_q(double a, double q, double p4) {
  const double den = p4 - 1.0, y = rich_recip(den), x = fma(p4, a, -q);
  return y != 0.0 ? div_known(x, den, y) : x / den;
}
__device__ __forceinline__ void rich_combine(PV& o, const PV& a, const PV& q, double p4) {
  o.pos = {rich_q(a.pos.x, q.pos.x, p4), rich_q(a.pos.y, q.pos.y, p4), rich_q(a.pos.z, q.pos.z, p4)};
  o.vel = {rich_q(a.vel.x, q.vel.x, p4), rich_q(a.vel.y, q.vel.y, p4), rich_q(a.vel.z, q.vel.z, p4)};
}

// The Richardson tableau of richardson() from its rows' modified-midpoint
// results (row i: N = 2^i), in the same order of operations.
__device__ __forceinline__ PV richardson_of_rows(const PV* row, int rows) {
  PV prev[4], cur[4];
  prev[0] = row[0];
  for (int i = 1; i < rows; i++) {
    cur[0] = row[i];
    double p4 = 1.0;
    for (int j = 1; j <= i; j++) {
      p4 *= 4.0;
      rich_combine(cur[j], cur[j - 1], prev[j - 1], p4);
    }
    for (int j = 0; j <= i; j++) prev[j] = cur[j];
  }
  return prev[rows - 1];
}

// Richardson extrapolation over modified-midpoint steps N = 1, 2, 4, ...
// (sim.cuh:502-551); rows <= 4.  The tableau is kept row by row.
template <class VT>
__device__ __forceinline__ PV richardson(const PV& c, const VT& vt, double dt, int rows) {
  PV prev[4], cur[4];
  int N = 1;
  prev[0] = mod_midpoint(c, vt, dt, N);
  for (int i = 1; i < rows; i++) {
    N <<= 1;
    cur[0] = mod_midpoint(c, vt, dt, N);
    double p4 = 1.0;
    for (int j = 1; j <= i; j++) {
      p4 *= 4.0;  // pow(4, j), exact
      rich_combine(cur[j], cur[j - 1], prev[j - 1], p4);
    }
    for (int j = 0; j <= i; j++) prev[j] = cur[j];
  }
  return prev[rows - 1];
}

// ---- universal-variable drift (new formulation, no reference counterpart) ----
// Stumpff functions by quartering and doubling, Horner-form Taylor series
// (three terms when |z| < 5e-5, seven otherwise).
// |z| > c and |z| < c for a positive normal c as integer compares of the bit
// patterns (positive doubles order like their bits; NaN is neither, as with
// the FP64 compares, which each take a slot of the FP64 pipe on this GPU)
__device__ __forceinline__ bool abs_gt(double z, double c) {
  const long long a = __double_as_longlong(z) & 0x7fffffffffffffffLL;
  return a > __double_as_longlong(c) && a <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool abs_lt(double z, double c) {
  return (__double_as_longlong(z) & 0x7fffffffffffffffLL) < __double_as_longlong(c);
}
__device__ __forceinline__ void stumpff(double z, double* c0, double* c1, double* c2, double* c3) {
  int k = 0;
  while (abs_gt(z, 0.1) && k < 60) {
    z = z * 0.25;
    k++;
  }
  double s3, s2;
  if (abs_lt(z, 5e-5)) {
    // the z^3 terms are below 1e-17 relative here
    s3 = fma(z, fma(z, 1.0 / 5040.0, -1.0 / 120.0), 1.0 / 6.0);
    s2 = fma(z, fma(z, 1.0 / 720.0, -1.0 / 24.0), 0.5);
  } else {
    s3 = fma(z, fma(z, fma(z, fma(z, fma(z, fma(z, 1.0 / 1307674368000.0, -1.0 / 6227020800.0),
                                           1.0 / 39916800.0), -1.0 / 362880.0), 1.0 / 5040.0),
                    -1.0 / 120.0), 1.0 / 6.0);
    s2 = fma(z, fma(z, fma(z, fma(z, fma(z, fma(z, 1.0 / 87178291200.0, -1.0 / 479001600.0),
                                           1.0 / 3628800.0), -1.0 / 40320.0), 1.0 / 720.0),
                    -1.0 / 24.0), 0.5);
  }
  double s1 = fma(-z, s3, 1.0);
  double s0 = fma(-z, s2, 1.0);
  for (; k > 0; k--) {
    double n3 = fma(s0, s3, s2) * 0.25;
    double n2 = s1 * s1 * 0.5;
    double n1 = s0 * s1;
    double n0 = fma(2.0 * s0, s0, -1.0);
    s0 = n0;
    s1 = n1;
    s2 = n2;
    s3 = n3;
  }
  *c0 = s0;
  *c1 = s1;
  *c2 = s2;
  *c3 = s3;
}

// 1 / sqrt(x) and 1 / x for positive doubles inside the FP32 normal range
// (about 1e-37 .. 1e37): an FP32 seed whose double <-> float moves are
// integer operations on the high word (exponent rebias 1023 - 127 = 896),
// refined by one Halley step (rsqrt: seed error 2^-22 -> 2^-66) or two Newton
// steps (rcp: 2^-23 -> 2^-92); the refinement costs 5 and 4 FP64 operations
// where sqrt and division cost about 10 each.  Within an ulp or two of the
// correctly rounded value; outside the range, sqrt and division themselves.
__device__ __forceinline__ bool seed_range_ok(double x) {
  const int h = __double2hiint(x);
  return h > 0x38300000 && h < 0x47C00000;
}
__device__ __forceinline__ double rsqrt_fast(const FU& U, double x) {
  if (!seed_range_ok(x)) return 1.0 / sqrt(x);
  const float xf = __int_as_float((__double2hiint(x) - 0x38000000) << 3);
  const int yb = __float_as_int(rsqrtf(xf));
  const double u = __hiloint2double((yb >> 3) + 0x38000000, yb << 29);
  const double t = fmul(U, x, u);
  const double e = fma(-t, u, 1.0);
  const double c = fma(0.375, e, 0.5);
  const double ue = fmul(U, u, e);
  return fma(ue, c, u);
}
__device__ __forceinline__ double rcp_fast(double x) {
  if (!seed_range_ok(x)) return 1.0 / x;
  const float xf = __int_as_float((__double2hiint(x) - 0x38000000) << 3);
  const int yb = __float_as_int(__frcp_rn(xf));
  double y = __hiloint2double((yb >> 3) + 0x38000000, yb << 29);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

struct UD {
  PV out;
  int iters;
  bool converged;
  double s;  // converged universal anomaly
};

// |x| as an FP32 number, from the high word by integer operations (the top 20
// bits of the mantissa): 0 below the FP32 normal range, 3e38 above it.
__device__ __forceinline__ float abs_f32_trunc(double x) {
  const int h = __double2hiint(x) & 0x7fffffff;
  if (h < 0x38100000) return 0.0f;
  if (h > 0x47E00000) return 3e38f;
  return __int_as_float((h - 0x38000000) << 3);
}

// Initial guesses of the universal anomaly (the s0 argument of universal_drift)
constexpr double kGuessPlain = 0.0;    // s0 = dt / r0
constexpr double kGuessSeries = -1.0;  // third-order series in dt (below)
constexpr double kGuessRel = -2.0;     // s0 = (dt / r0) (1 + rel), rel from the learned guess

// x as a double by integer operations on its bits (exact for normal floats
// and zero; a denormal gives zero; not for infinities or NaN), so that no
// conversion runs on the FP64 pipe
__device__ __forceinline__ double f64_of_f32(float x) {
  const int b = __float_as_int(x), m = b & 0x7fffffff;
  if (m < 0x00800000) return 0.0;
  return __hiloint2double((b & (int)0x80000000) | ((m >> 3) + 0x38000000), m << 29);
}

// Universal Kepler drift with mu = 1 from initial guess s0 (kGuessPlain: dt /
// r0; kGuessSeries: the universal Kepler equation t = r0 s + eta s^2/2 + zeta
// s^3/6 + O(s^4) inverted to third order, s = s0 (1 - (eta / 2 r0) s0 + ((3
// eta^2 - r0 zeta) / 6 r0^2) s0^2) with s0 = dt / r0, kept when within a factor
// 2 of s0; kGuessRel: s0 (1 + rel), kept within a factor 16): Newton on
// r0 s + eta G2 + zeta G3 = dt (Laguerre-Conway steps, n = 5, after
// kNewtonIters Newton steps without convergence); after each update the
// Newton error estimate |f''/(2 f')| ds^2 of the new s is compared with tol |s|
// (trusted once |ds| <= 1e-3 |s|), in FP32 on truncated copies (the decision
// needs no more than a factor of 2); f and g at the final s.
constexpr int kNewtonIters = 8;  // Newton steps before the Laguerre-Conway fallback
__device__ __forceinline__ UD universal_drift(const FU& U, const d3& x0, const d3& v0, double dt, double s0,
                                              double tol, int max_iter, float rel = 0.0f) {
  const double rr = fma(x0.x, x0.x, fma(x0.y, x0.y, fmul(U, x0.z, x0.z)));
  const double ir0 = rsqrt_fast(U, rr);
  const double r0 = fmul(U, rr, ir0);
  double eta = fma(x0.x, v0.x, fma(x0.y, v0.y, fmul(U, x0.z, v0.z)));
  double v2 = fma(v0.x, v0.x, fma(v0.y, v0.y, fmul(U, v0.z, v0.z)));
  double alpha = fma(2.0, ir0, -v2);
  double zeta = fma(-alpha, r0, 1.0);
  // (s0 > 0 and the factor-of-2 window of the series guess tested on the bit
  // patterns where that is exact: FP64 compares and products take FP64-pipe
  // slots on this GPU)
  const long long s0b = __double_as_longlong(s0);
  if (!(s0b > 0 && s0b <= 0x7ff0000000000000LL)) {
    const double p0 = fmul(U, dt, ir0);
    double g = p0;
    if (s0 == kGuessSeries) {
      const double a1 = fmul(U, fmul(U, 0.5, eta), ir0);
      const double a2 = fmul(U, fmul(U, fma(fmul(U, 3.0, eta), eta, -fmul(U, r0, zeta)), fmul(U, ir0, ir0)),
                             1.0 / 6.0);
      const double q = fmul(U, p0, fma(p0, fma(p0, a2, -a1), 1.0));
      // 0.5 p0 < q < 2 p0: for p0 in [2^-1020, 2^1022) the halving and the
      // doubling are exact exponent steps, so the window is pb - 2^52 < qb <
      // pb + 2^52 on the bits (q of another sign or NaN falls outside)
      const long long pb = __double_as_longlong(p0), qb = __double_as_longlong(q);
      if (pb >= 0x0030000000000000LL && pb < 0x7fd0000000000000LL) {
        if (qb > pb - (1LL << 52) && qb < pb + (1LL << 52)) g = q;
      } else if (q > 0.5 * p0 && q < 2.0 * p0) {
        g = q;
      }
    } else if (s0 == kGuessRel) {
      // the learned guess covers long drifts, where s/s0 spans ~0.1..4
      const double q = fma(p0, f64_of_f32(rel), p0);
      if (q > 0.0625 * p0 && q < 16.0 * p0) g = q;
    }
    s0 = g;
  }
  const float tol2f = abs_f32_trunc(2.0 * tol);
  double s = s0;
  int it = 0;
  bool conv = false;
  double c0, c1, c2, c3;
  while (it < max_iter) {
    double s2 = fmul(U, s, s);
    stumpff(fmul(U, alpha, s2), &c0, &c1, &c2, &c3);
    double G1 = fmul(U, s, c1), G2 = fmul(U, s2, c2), G3 = fmul(U, fmul(U, s2, s), c3);
    double f = fma(r0, s, fma(eta, G2, fma(zeta, G3, -dt)));
    double fp = fma(eta, G1, fma(zeta, G2, r0));
    double fpp = fma(eta, c0, fmul(U, zeta, G1));
    double ds;
    if (it < kNewtonIters) {
      ds = fmul(U, -f, rcp_fast(fp));
    } else {
      // Laguerre-Conway step (n = 5): converges where Newton oscillates on
      // long drifts (x1 = dt / r0^1.5 >> 1 near perihelion)
      const double h = fabs(fma(fmul(U, 16.0, fp), fp, -fmul(U, fmul(U, 20.0, f), fpp)));
      ds = fmul(U, fmul(U, -5.0, f), rcp_fast(fadd(U, fp, sqrt(h))));
    }
    s = fadd(U, s, ds);
    it++;
    const float dsf = abs_f32_trunc(ds), sf = abs_f32_trunc(s);
    if (dsf <= 1e-3f * sf && abs_f32_trunc(fpp) * dsf * dsf <= tol2f * sf * abs_f32_trunc(fp)) {
      conv = true;
      break;
    }
  }
  double s2 = fmul(U, s, s);
  stumpff(fmul(U, alpha, s2), &c0, &c1, &c2, &c3);
  double G1 = fmul(U, s, c1), G2 = fmul(U, s2, c2), G3 = fmul(U, fmul(U, s2, s), c3);
  double r = fma(eta, G1, fma(zeta, G2, r0));
  double ir = rcp_fast(r);
  double f = fma(-G2, ir0, 1.0);
  double g = fsub(U, dt, G3);
  double fd = fmul(U, fmul(U, -G1, ir0), ir);
  double gd = fma(-G2, ir, 1.0);
  UD u;
  u.out.pos = {fma(f, x0.x, fmul(U, g, v0.x)), fma(f, x0.y, fmul(U, g, v0.y)), fma(f, x0.z, fmul(U, g, v0.z))};
  u.out.vel = {fma(fd, x0.x, fmul(U, gd, v0.x)), fma(fd, x0.y, fmul(U, gd, v0.y)),
               fma(fd, x0.z, fmul(U, gd, v0.z))};
  u.iters = it;
  u.converged = conv;
  u.s = s;
  return u;
}

}  // namespace merc
