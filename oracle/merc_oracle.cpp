// merc_oracle.cpp - C ABI of the CPU oracle (liboracle.so).  TEST INFRASTRUCTURE.
//
// Only tests, the smoke check and the CPU-baseline leg of bench.py load this
// library, as the checker.  It runs the Mercurius step of the reference
// (src/sim.cuh:615-766) on host cores, OpenMP-parallel over systems (many
// systems) or over the bodies of each phase (few systems), in binary64
// (precision 0) or long double (precision 1).
//
// Layouts are those of include/merc.h: systems concatenated body-wise,
// positions/velocities component-major pos[c * n_total + j].
#include <omp.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <memory>

#include "../include/merc.h"
#include "merc_oracle.hpp"

namespace oracle {

static Params to_params(const merc_params* p) {
  Params q;
  q.dt = p->dt;
  q.softening2 = p->softening2;
  q.hill_factor = p->hill_factor;
  q.kepler_tol = p->kepler_tol;
  q.eject_r = p->eject_r;
  q.kepler_iters = p->kepler_iters;
  q.bs_rows = p->bs_rows;
  q.compat_block = p->compat_block;
  q.drift = p->drift;
  q.kepler_max_iter = p->kepler_max_iter;
  q.warm_start = p->warm_start;
  return q;
}

struct Counters {
  int64_t ce_body_steps = 0, kep_iters = 0, kep_solves = 0, nonconv = 0;
};

template <class R> struct Sys {
  int n = 0, nm = 0;
  std::vector<V3<R>> x, v;
  std::vector<R> m, alag;
  std::vector<uint32_t> flags;
  // physical collisions (empty: off): radii, steps since load, events
  // (step, survivor, absorbed; indices within the system)
  std::vector<double> rad;
  int64_t step = 0;
  std::vector<int64_t> ev;
};

// Index of the source a body excludes as "itself": its index in the system,
// or, reproducing the reference, threadIdx.x = index % blockDim.x
// (sim.cuh:172,335,598 with block size N/16, mercurius.cu:49).
static inline int self_index(int j, int compat_block) { return compat_block > 0 ? j % compat_block : j; }

template <class R, class M> static void build_sources(const Sys<R>& S, R hill, std::vector<Src<R>>& src) {
  src.resize(S.nm);
  for (int i = 0; i < S.nm; i++) {
    src[i].x = S.x[i];
    src[i].m = S.m[i];
    src[i].rc = rcrit<R, M>(S.x[i], S.v[i], S.m[i], hill);
  }
}

// main_body_kinetic: x += dt * sum_i m_i v_i, sim.cuh:384-406 (the sum is the
// same for every body; the reference recomputes it per thread in this order).
template <class R> static V3<R> momentum(const Sys<R>& S) {
  V3<R> p = {R(0), R(0), R(0)};
  for (int i = 0; i < S.nm; i++) {
    p.x = std::fma(S.m[i], S.v[i].x, p.x);
    p.y = std::fma(S.m[i], S.v[i].y, p.y);
    p.z = std::fma(S.m[i], S.v[i].z, p.z);
  }
  return p;
}

// democratic_heliocentric_conversion, sim.cuh:555-587, read-all-then-write.
template <class R> static void dh_convert(Sys<R>& S, bool reverse) {
  R total = R(0);
  V3<R> mw = {R(0), R(0), R(0)};
  R not_rev = R(!reverse);
  R sgn = reverse ? R(1) : R(-1);  // pow(-1, not_reverse)
  for (int i = 0; i < S.nm; i++) {
    total += S.m[i];
    mw.x = std::fma(S.m[i], S.v[i].x, mw.x);
    mw.y = std::fma(S.m[i], S.v[i].y, mw.y);
    mw.z = std::fma(S.m[i], S.v[i].z, mw.z);
  }
  R scale = R(1) / std::fma(not_rev, total, R(1));
  mw.x *= scale;
  mw.y *= scale;
  mw.z *= scale;
  for (int j = 0; j < S.n; j++) {
    S.v[j].x = std::fma(sgn, mw.x, S.v[j].x);
    S.v[j].y = std::fma(sgn, mw.y, S.v[j].y);
    S.v[j].z = std::fma(sgn, mw.z, S.v[j].z);
  }
}

// close_encounter_p, sim.cuh:589-613
template <class R, class M>
static bool close_encounter(const V3<R>& pos, int self, const Src<R>* src, int nm) {
  bool ce = false;
  for (int i = 0; i < nm; i++) {
    R mag = M::norm3d(src[i].x.x - pos.x, src[i].x.y - pos.y, src[i].x.z - pos.z);
    ce = ce || ((mag < src[i].rc) && (self != i));
  }
  return ce;
}

// Physical collisions after the drift (no reference counterpart; restates
// k_collide_find / k_collide_resolve of the GPU library, merc_collide.cuh):
// every body in encounter this step against the massive bodies of its system,
// |x_a - x_b| < R_a + R_b on the drift outputs; the pairs (a < b) merge in
// ascending order while both are unmerged: the heavier survives (the lower
// index on a tie) with the total mass and the mass-weighted mean position and
// velocity; the other body keeps MERC_MERGED_MASS if it was massive and is
// parked on a circular orbit at MERC_PARK_R + 64 x its index.
template <class R, class M> static void collide(Sys<R>& S, const std::vector<char>& ce, R hill) {
  S.step++;
  std::vector<std::pair<int, int>> pairs;
  for (int j = 0; j < S.n; j++) {
    if (!ce[j] || (S.flags[j] & MERC_FLAG_MERGED)) continue;
    for (int i = 0; i < S.nm; i++) {
      if (i == j || (S.flags[i] & MERC_FLAG_MERGED)) continue;
      const int a = std::min(i, j), b = std::max(i, j);
      const R dx = S.x[b].x - S.x[a].x, dy = S.x[b].y - S.x[a].y, dz = S.x[b].z - S.x[a].z;
      const R d2 = std::fma(dx, dx, std::fma(dy, dy, dz * dz));
      const R rs = R(S.rad[a]) + R(S.rad[b]);
      if (d2 < rs * rs) pairs.push_back({a, b});
    }
  }
  std::sort(pairs.begin(), pairs.end());
  pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
  for (const auto& pr : pairs) {
    const int a = pr.first, b = pr.second;
    if ((S.flags[a] | S.flags[b]) & MERC_FLAG_MERGED) continue;
    const int s = S.m[b] > S.m[a] ? b : a, o = s == a ? b : a;
    if (o < S.nm) {
      const R ms = S.m[s], mo = S.m[o], Mt = ms + mo;
      S.x[s] = {std::fma(ms, S.x[s].x, mo * S.x[o].x) / Mt, std::fma(ms, S.x[s].y, mo * S.x[o].y) / Mt,
                std::fma(ms, S.x[s].z, mo * S.x[o].z) / Mt};
      S.v[s] = {std::fma(ms, S.v[s].x, mo * S.v[o].x) / Mt, std::fma(ms, S.v[s].y, mo * S.v[o].y) / Mt,
                std::fma(ms, S.v[s].z, mo * S.v[o].z) / Mt};
      S.m[s] = Mt;
      S.m[o] = R(MERC_MERGED_MASS);
    }
    const R r = R(MERC_PARK_R) + R(64) * R(o);
    S.x[o] = {r, R(0), R(0)};
    S.v[o] = {R(0), R(1) / std::sqrt(r), R(0)};
    S.alag[o] = r;
    S.flags[s] |= MERC_FLAG_GREW;
    S.flags[o] |= MERC_FLAG_MERGED;
    S.ev.push_back(S.step);
    S.ev.push_back(s);
    S.ev.push_back(o);
  }
  (void)hill;
}

// One Mercurius step of one system: the loop body of mercurius_solver,
// sim.cuh:679-742.  `par` parallelises the body loops with OpenMP.
template <class R, class M> static void step_system(Sys<R>& S, const Params& P, bool par, Counters& cnt) {
  const R dt = R(P.dt), hdt = R(0.5) * dt, soft2 = R(P.softening2), hill = R(P.hill_factor);
  const int n = S.n, nm = S.nm;
  std::vector<Src<R>> src;
  std::vector<V3<R>> xn(n), vn(n);
  std::vector<char> ce(n, 0);
  std::vector<int> its(n, 0), ok(n, 1);

  // first half kick, sim.cuh:683-685
  build_sources<R, M>(S, hill, src);
#pragma omp parallel for schedule(static) if (par)
  for (int j = 0; j < n; j++)
    vn[j] = kick<R, M>(S.x[j], S.v[j], self_index(j, P.compat_block), src.data(), nm, hdt, false, soft2);
  S.v.swap(vn);
  // first solar jump, sim.cuh:687-689
  V3<R> p = momentum(S);
  for (int j = 0; j < n; j++) {
    S.x[j].x = std::fma(p.x, hdt, S.x[j].x);
    S.x[j].y = std::fma(p.y, hdt, S.x[j].y);
    S.x[j].z = std::fma(p.z, hdt, S.x[j].z);
  }
  // drift or encounter sub-step, sim.cuh:692-731
  build_sources<R, M>(S, hill, src);
  const R tp = two_pi<R>();
#pragma omp parallel for schedule(dynamic, 16) if (par)
  for (int j = 0; j < n; j++) {
    const int self = self_index(j, P.compat_block);
    const bool is_ce = close_encounter<R, M>(S.x[j], self, src.data(), nm);
    ce[j] = is_ce;
    PV<R> cur = {S.x[j], S.v[j]};
    PV<R> out;
    if (P.drift == MERC_DRIFT_ELEMENTS) {
      R a = S.alag[j];
      R nmot = M::rsqrt(a * a * a);  // mean motion from the previous elements, sim.cuh:692
      Elem<R> el = elem_from_cart<R, M>(cur.pos, cur.vel);
      S.alag[j] = el.a;
      R Mn = R(!is_ce) * std::fmod(std::fma(nmot, dt, el.M), tp) + R(is_ce) * el.M;  // :707
      PV<R> kep = cart_from_elem<R, M>(el.inc, el.node, el.peri, Mn, el.e, el.a, P.kepler_iters);
      if (is_ce) {
        // the unused Kepler branch still enters the blend (sim.cuh:718-730)
        PV<R> bs = richardson<R, M>(cur, self, src.data(), nm, dt, P.bs_rows, soft2);
        out.pos = {std::fma(R(0), kep.pos.x, bs.pos.x), std::fma(R(0), kep.pos.y, bs.pos.y),
                   std::fma(R(0), kep.pos.z, bs.pos.z)};
        out.vel = {std::fma(R(0), kep.vel.x, bs.vel.x), std::fma(R(0), kep.vel.y, bs.vel.y),
                   std::fma(R(0), kep.vel.z, bs.vel.z)};
      } else {
        out = kep;
      }
    } else {
      if (is_ce) {
        out = richardson<R, M>(cur, self, src.data(), nm, dt, P.bs_rows, soft2);
      } else {
        R s0 = P.warm_start == 2 ? series_guess(cur.pos, cur.vel, dt) : plain_guess(cur.pos, dt);
        UDrift<R> u = universal_drift(cur.pos, cur.vel, dt, s0, R(P.kepler_tol), P.kepler_max_iter);
        out = u.out;
        its[j] = u.iters;
        ok[j] = u.converged;
      }
    }
    xn[j] = out.pos;
    vn[j] = out.vel;
  }
  S.x.swap(xn);
  S.v.swap(vn);
  if (!S.rad.empty()) collide<R, M>(S, ce, hill);
  // second solar jump, sim.cuh:735-737
  p = momentum(S);
  for (int j = 0; j < n; j++) {
    S.x[j].x = std::fma(p.x, hdt, S.x[j].x);
    S.x[j].y = std::fma(p.y, hdt, S.x[j].y);
    S.x[j].z = std::fma(p.z, hdt, S.x[j].z);
  }
  // second half kick, sim.cuh:739-741
  build_sources<R, M>(S, hill, src);
#pragma omp parallel for schedule(static) if (par)
  for (int j = 0; j < n; j++)
    vn[j] = kick<R, M>(S.x[j], S.v[j], self_index(j, P.compat_block), src.data(), nm, hdt, false, soft2);
  S.v.swap(vn);

  const R ej2 = R(P.eject_r) * R(P.eject_r);
  for (int j = 0; j < n; j++) {
    uint32_t f = S.flags[j] & ~MERC_FLAG_CE_LAST;
    if (ce[j]) {
      f |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
      cnt.ce_body_steps++;
    }
    R r2 = mag2(S.x[j]);
    if (P.eject_r > 0 && r2 > ej2) f |= MERC_FLAG_EJECTED;
    bool fin = std::isfinite(S.x[j].x) && std::isfinite(S.x[j].y) && std::isfinite(S.x[j].z) &&
               std::isfinite(S.v[j].x) && std::isfinite(S.v[j].y) && std::isfinite(S.v[j].z);
    if (!fin) f |= MERC_FLAG_NONFINITE;
    S.flags[j] = f;
    if (P.drift == MERC_DRIFT_UNIVERSAL && !ce[j]) {
      cnt.kep_iters += its[j];
      cnt.kep_solves++;
      if (!ok[j]) cnt.nonconv++;
    }
  }
}

// elements -> heliocentric cartesian -> democratic heliocentric: the kernel
// prologue, sim.cuh:654-677.
template <class R, class M> static void from_elements(Sys<R>& S, const R* el6[6], int iters) {
  for (int j = 0; j < S.n; j++) {
    PV<R> pv = cart_from_elem<R, M>(el6[0][j], el6[1][j], el6[2][j], el6[3][j], el6[4][j], el6[5][j], iters);
    S.x[j] = pv.pos;
    S.v[j] = pv.vel;
    S.alag[j] = el6[5][j];
  }
  dh_convert(S, false);
}

// reverse conversion then cartesian -> elements: the kernel epilogue,
// sim.cuh:746-765.  Leaves S.v heliocentric.
template <class R, class M> static void to_elements(Sys<R>& S, std::vector<Elem<R>>& el) {
  dh_convert(S, true);
  el.resize(S.n);
  for (int j = 0; j < S.n; j++) el[j] = elem_from_cart<R, M>(S.x[j], S.v[j]);
}

// ---- marshalling between the flat C arrays and per-system structs ----
template <class R>
static void gather(Sys<R>& S, int64_t b0, int64_t n, int nm, int64_t ntot, const double* mass, const double* pos,
                   const double* vel, const double* alag, const uint32_t* flags) {
  S.n = (int)n;
  S.nm = nm;
  S.x.resize(n);
  S.v.resize(n);
  S.m.resize(n);
  S.alag.assign(n, R(0));
  S.flags.assign(n, 0u);
  for (int64_t j = 0; j < n; j++) {
    int64_t g = b0 + j;
    S.m[j] = R(mass[g]);
    if (pos) S.x[j] = {R(pos[g]), R(pos[ntot + g]), R(pos[2 * ntot + g])};
    if (vel) S.v[j] = {R(vel[g]), R(vel[ntot + g]), R(vel[2 * ntot + g])};
    if (alag) S.alag[j] = R(alag[g]);
    if (flags) S.flags[j] = flags[g];
  }
}

template <class R>
static void scatter(const Sys<R>& S, int64_t b0, int64_t ntot, double* pos, double* vel, double* alag,
                    uint32_t* flags) {
  for (int64_t j = 0; j < S.n; j++) {
    int64_t g = b0 + j;
    if (pos) {
      pos[g] = double(S.x[j].x);
      pos[ntot + g] = double(S.x[j].y);
      pos[2 * ntot + g] = double(S.x[j].z);
    }
    if (vel) {
      vel[g] = double(S.v[j].x);
      vel[ntot + g] = double(S.v[j].y);
      vel[2 * ntot + g] = double(S.v[j].z);
    }
    if (alag) alag[g] = double(S.alag[j]);
    if (flags) flags[g] = S.flags[j];
  }
}

static int check_layout(int n_sys, const int64_t* off, const int32_t* nm) {
  if (n_sys <= 0 || !off || !nm) return MERC_ERR_CONFIG;
  for (int s = 0; s < n_sys; s++) {
    int64_t n = off[s + 1] - off[s];
    if (n <= 0 || nm[s] < 0 || nm[s] > n) return MERC_ERR_CONFIG;
  }
  return MERC_OK;
}

// Collision arguments of run_impl: radii (NULL: off), masses written back,
// steps since load before the call, and the events (step, survivor, absorbed
// as global indices) in the order the GPU library logs them: by step, then
// by the pair (lower, higher index).
struct CollideIO {
  const double* radius = nullptr;
  double* mass_out = nullptr;
  int64_t step0 = 0;
  std::vector<int64_t> events;
};

template <class R, class M>
static int run_impl(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm, const double* mass,
                    double* pos, double* vel, double* alag, uint32_t* flags, int64_t n_steps, int64_t* stats,
                    CollideIO* col = nullptr) {
  Params P = to_params(mp);
  const int64_t ntot = off[n_sys];
  const int nthr = omp_get_max_threads();
  const bool by_system = n_sys >= 2 * nthr;
  std::vector<Counters> cnt(n_sys);
  std::vector<std::vector<int64_t>> ev(n_sys);
#pragma omp parallel for schedule(dynamic, 1) if (by_system)
  for (int s = 0; s < n_sys; s++) {
    Sys<R> S;
    gather(S, off[s], off[s + 1] - off[s], nm[s], ntot, mass, pos, vel, alag, flags);
    if (col && col->radius) {
      S.rad.assign(col->radius + off[s], col->radius + off[s + 1]);
      S.step = col->step0;
    }
    for (int64_t k = 0; k < n_steps; k++) step_system<R, M>(S, P, !by_system, cnt[s]);
    scatter(S, off[s], ntot, pos, vel, alag, flags);
    if (col && col->radius) {
      for (int j = 0; j < S.n; j++) col->mass_out[off[s] + j] = double(S.m[j]);
      for (size_t e = 0; e < S.ev.size(); e += 3)
        ev[s].insert(ev[s].end(), {S.ev[e], off[s] + S.ev[e + 1], off[s] + S.ev[e + 2]});
    }
  }
  if (col && col->radius) {
    std::vector<std::array<int64_t, 3>> all;
    for (int s = 0; s < n_sys; s++)
      for (size_t e = 0; e < ev[s].size(); e += 3) all.push_back({ev[s][e], ev[s][e + 1], ev[s][e + 2]});
    std::stable_sort(all.begin(), all.end(), [](const std::array<int64_t, 3>& x, const std::array<int64_t, 3>& y) {
      const int64_t xa = std::min(x[1], x[2]), ya = std::min(y[1], y[2]);
      const int64_t xb = std::max(x[1], x[2]), yb = std::max(y[1], y[2]);
      return x[0] != y[0] ? x[0] < y[0] : (xa != ya ? xa < ya : xb < yb);
    });
    for (const auto& e : all) col->events.insert(col->events.end(), e.begin(), e.end());
  }
  if (stats) {
    for (int s = 0; s < n_sys; s++) {
      stats[0] += cnt[s].ce_body_steps;
      stats[1] += cnt[s].kep_iters;
      stats[2] += cnt[s].kep_solves;
      stats[3] += cnt[s].nonconv;
    }
  }
  return MERC_OK;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_num_threads(void) { return omp_get_max_threads(); }
void oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

// Prologue: elements -> heliocentric positions, DH velocities, a_lag.
int oracle_load_elements(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm,
                         const double* mass, const double* elements, double* pos, double* vel, double* alag,
                         int precision) {
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  const int64_t ntot = off[n_sys];
  for (int s = 0; s < n_sys; s++) {
    Sys<double> S;
    gather<double>(S, off[s], off[s + 1] - off[s], nm[s], ntot, mass, nullptr, nullptr, nullptr, nullptr);
    const double* el6[6];
    for (int k = 0; k < 6; k++) el6[k] = elements + k * ntot + off[s];
    if (precision == 2)
      from_elements<double, MercMath>(S, el6, mp->kepler_iters);
    else
      from_elements<double, StdMath>(S, el6, mp->kepler_iters);
    scatter(S, off[s], ntot, pos, vel, alag, nullptr);
  }
  return MERC_OK;
}

// n_steps Mercurius steps.  precision 0: binary64 with the host C library,
// 1: long double, 2: binary64 with the GPU library's merc_math functions.
// stats (may be NULL): int64[4] accumulated: CE body-steps, universal
// iterations, universal solves, non-converged solves.
int oracle_run(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm, const double* mass,
               double* pos, double* vel, double* alag, uint32_t* flags, int64_t n_steps, int precision,
               int64_t* stats) {
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  if (mp->bs_rows < 1 || mp->bs_rows > 4 || mp->kepler_iters < 1 || mp->kepler_max_iter < 1) return MERC_ERR_CONFIG;
  if (precision == 1)
    return run_impl<long double, StdMath>(mp, n_sys, off, nm, mass, pos, vel, alag, flags, n_steps, stats);
  if (precision == 2)
    return run_impl<double, MercMath>(mp, n_sys, off, nm, mass, pos, vel, alag, flags, n_steps, stats);
  return run_impl<double, StdMath>(mp, n_sys, off, nm, mass, pos, vel, alag, flags, n_steps, stats);
}

// oracle_run with physical collisions: radius[n_total] (AU), mass in/out
// (merged masses written back), step0 = steps since load before the call.
// events: room for 3 x max_events int64 (step, survivor, absorbed), *n_events
// gets the total.
int oracle_run_collide(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm, double* mass,
                       const double* radius, double* pos, double* vel, double* alag, uint32_t* flags,
                       int64_t n_steps, int precision, int64_t* stats, int64_t step0, int64_t* events,
                       int64_t max_events, int64_t* n_events) {
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  if (!radius || !mass || !flags) return MERC_ERR_CONFIG;
  const int64_t ntot = off[n_sys];
  std::vector<double> m_in(mass, mass + ntot);
  CollideIO io;
  io.radius = radius;
  io.mass_out = mass;
  io.step0 = step0;
  if (precision == 1)
    st = run_impl<long double, StdMath>(mp, n_sys, off, nm, m_in.data(), pos, vel, alag, flags, n_steps, stats, &io);
  else if (precision == 2)
    st = run_impl<double, MercMath>(mp, n_sys, off, nm, m_in.data(), pos, vel, alag, flags, n_steps, stats, &io);
  else
    st = run_impl<double, StdMath>(mp, n_sys, off, nm, m_in.data(), pos, vel, alag, flags, n_steps, stats, &io);
  const int64_t ne = (int64_t)io.events.size() / 3;
  if (n_events) *n_events = ne;
  for (int64_t k = 0; k < std::min(ne, max_events); k++)
    for (int c = 0; c < 3; c++) events[3 * k + c] = io.events[3 * k + c];
  return st;
}

// Batch boundary: reverse DH, elements, cartesian, forward DH (sim.cuh:744-765,
// then :654-677 of the next launch).  Updates pos, vel, alag in place.
int oracle_roundtrip(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm, const double* mass,
                     double* pos, double* vel, double* alag, int precision) {
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  const int64_t ntot = off[n_sys];
  for (int s = 0; s < n_sys; s++) {
    Sys<double> S;
    gather<double>(S, off[s], off[s + 1] - off[s], nm[s], ntot, mass, pos, vel, nullptr, nullptr);
    std::vector<Elem<double>> el;
    if (precision == 2)
      to_elements<double, MercMath>(S, el);
    else
      to_elements<double, StdMath>(S, el);
    std::vector<double> e6(6 * (size_t)S.n);
    const double* el6[6];
    for (int j = 0; j < S.n; j++) {
      e6[0 * S.n + j] = el[j].inc;
      e6[1 * S.n + j] = el[j].node;
      e6[2 * S.n + j] = el[j].peri;
      e6[3 * S.n + j] = el[j].M;
      e6[4 * S.n + j] = el[j].e;
      e6[5 * S.n + j] = el[j].a;
    }
    for (int k = 0; k < 6; k++) el6[k] = e6.data() + k * S.n;
    if (precision == 2)
      from_elements<double, MercMath>(S, el6, mp->kepler_iters);
    else
      from_elements<double, StdMath>(S, el6, mp->kepler_iters);
    scatter(S, off[s], ntot, pos, vel, alag, nullptr);
  }
  return MERC_OK;
}

// Elements of the state (reverse DH + cartesian -> elements), 6 x n_total.
int oracle_to_elements(const merc_params* mp, int n_sys, const int64_t* off, const int32_t* nm, const double* mass,
                       const double* pos, const double* vel, double* elements, int precision) {
  (void)mp;
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  const int64_t ntot = off[n_sys];
  for (int s = 0; s < n_sys; s++) {
    Sys<double> S;
    gather<double>(S, off[s], off[s + 1] - off[s], nm[s], ntot, mass, pos, vel, nullptr, nullptr);
    std::vector<Elem<double>> el;
    if (precision == 2)
      to_elements<double, MercMath>(S, el);
    else
      to_elements<double, StdMath>(S, el);
    for (int j = 0; j < S.n; j++) {
      int64_t g = off[s] + j;
      elements[0 * ntot + g] = el[j].inc;
      elements[1 * ntot + g] = el[j].node;
      elements[2 * ntot + g] = el[j].peri;
      elements[3 * ntot + g] = el[j].M;
      elements[4 * ntot + g] = el[j].e;
      elements[5 * ntot + g] = el[j].a;
    }
  }
  return MERC_OK;
}

// Total energy of each system's massive bodies with the Sun (mass 1), in
// democratic-heliocentric variables, unsoftened:
//   sum m v^2/2 - sum m/r - sum_{i<k} m_i m_k/r_ik + |sum m v|^2/2.
int oracle_energy(int n_sys, const int64_t* off, const int32_t* nm, const double* mass, const double* pos,
                  const double* vel, double* energy, int precision) {
  int st = check_layout(n_sys, off, nm);
  if (st) return st;
  const int64_t ntot = off[n_sys];
  for (int s = 0; s < n_sys; s++) {
    long double E = 0, px = 0, py = 0, pz = 0;
    int64_t b = off[s];
    for (int i = 0; i < nm[s]; i++) {
      int64_t g = b + i;
      long double m = mass[g], x = pos[g], y = pos[ntot + g], z = pos[2 * ntot + g];
      long double vx = vel[g], vy = vel[ntot + g], vz = vel[2 * ntot + g];
      E += 0.5L * m * (vx * vx + vy * vy + vz * vz) - m / std::sqrt(x * x + y * y + z * z);
      px += m * vx;
      py += m * vy;
      pz += m * vz;
      for (int k = i + 1; k < nm[s]; k++) {
        int64_t h = b + k;
        long double dx = x - pos[h], dy = y - pos[ntot + h], dz = z - pos[2 * ntot + h];
        E -= m * (long double)mass[h] / std::sqrt(dx * dx + dy * dy + dz * dz);
      }
    }
    E += 0.5L * (px * px + py * py + pz * pz);
    energy[s] = precision == 1 ? (double)E : (double)E;
  }
  return MERC_OK;
}

// ---- unit-level entry points for golden vectors ----
void oracle_danby(int64_t n, const double* M, const double* e, int iters, double* E) {
  for (int64_t i = 0; i < n; i++) E[i] = danby<double, StdMath>(M[i], e[i], iters);
}

void oracle_cart_from_elem(int64_t n, const double* el, int iters, double* pos, double* vel) {
  for (int64_t j = 0; j < n; j++) {
    PV<double> pv = cart_from_elem<double, StdMath>(el[j], el[n + j], el[2 * n + j], el[3 * n + j], el[4 * n + j],
                                                    el[5 * n + j], iters);
    pos[j] = pv.pos.x; pos[n + j] = pv.pos.y; pos[2 * n + j] = pv.pos.z;
    vel[j] = pv.vel.x; vel[n + j] = pv.vel.y; vel[2 * n + j] = pv.vel.z;
  }
}

void oracle_elem_from_cart(int64_t n, const double* pos, const double* vel, double* el) {
  for (int64_t j = 0; j < n; j++) {
    V3<double> p = {pos[j], pos[n + j], pos[2 * n + j]}, v = {vel[j], vel[n + j], vel[2 * n + j]};
    Elem<double> e = elem_from_cart<double, StdMath>(p, v);
    el[j] = e.inc; el[n + j] = e.node; el[2 * n + j] = e.peri;
    el[3 * n + j] = e.M; el[4 * n + j] = e.e; el[5 * n + j] = e.a;
  }
}

// Universal-variable drift of n independent bodies from a given initial guess
// (s0 NULL: plain guess dt/r0).  Writes the converged s if s_out is given.
void oracle_universal(int64_t n, const double* pos, const double* vel, double dt, double tol, int max_iter,
                      const double* s0, double* pos_out, double* vel_out, int32_t* iters, int precision) {
  for (int64_t j = 0; j < n; j++) {
    if (precision == 1) {
      V3<long double> p = {pos[j], pos[n + j], pos[2 * n + j]}, v = {vel[j], vel[n + j], vel[2 * n + j]};
      long double g = s0 ? (long double)s0[j] : plain_guess(p, (long double)dt);
      UDrift<long double> u = universal_drift(p, v, (long double)dt, g, (long double)tol, max_iter);
      pos_out[j] = u.out.pos.x; pos_out[n + j] = u.out.pos.y; pos_out[2 * n + j] = u.out.pos.z;
      vel_out[j] = u.out.vel.x; vel_out[n + j] = u.out.vel.y; vel_out[2 * n + j] = u.out.vel.z;
      if (iters) iters[j] = u.iters;
    } else {
      V3<double> p = {pos[j], pos[n + j], pos[2 * n + j]}, v = {vel[j], vel[n + j], vel[2 * n + j]};
      double g = s0 ? s0[j] : plain_guess(p, dt);
      UDrift<double> u = universal_drift(p, v, dt, g, tol, max_iter);
      pos_out[j] = u.out.pos.x; pos_out[n + j] = u.out.pos.y; pos_out[2 * n + j] = u.out.pos.z;
      vel_out[j] = u.out.vel.x; vel_out[n + j] = u.out.vel.y; vel_out[2 * n + j] = u.out.vel.z;
      if (iters) iters[j] = u.iters;
    }
  }
}

// Evaluate one merc_math function on the host: fn 0 sin, 1 cos, 2 atan2(x, y),
// 3 acos, 4 log, 5 sinh, 6 cosh, 7 cbrt, 8 exp.
void oracle_mm_eval(int fn, int64_t n, const double* x, const double* y, double* out) {
  for (int64_t i = 0; i < n; i++) {
    double a = x[i];
    switch (fn) {
      case 0: out[i] = mm::sin(a); break;
      case 1: out[i] = mm::cos(a); break;
      case 2: out[i] = mm::atan2(a, y[i]); break;
      case 3: out[i] = mm::acos(a); break;
      case 4: out[i] = mm::log(a); break;
      case 5: out[i] = mm::sinh(a); break;
      case 6: out[i] = mm::cosh(a); break;
      case 7: out[i] = mm::cbrt(a); break;
      default: out[i] = mm::exp(a); break;
    }
  }
}

void oracle_stumpff(int64_t n, const double* z, double* c /* 4 x n */) {
  for (int64_t j = 0; j < n; j++) stumpff(z[j], &c[j], &c[n + j], &c[2 * n + j], &c[3 * n + j]);
}

}  // extern "C"
