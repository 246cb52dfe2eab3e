// merc_fast.cuh - pair arithmetic of the universal-drift path.
//
// FP64 is the bottleneck of this integrator on GB300 (one FP64 FMA per
// SM per clock cycle pair, 1/58 of the FP32 rate), so the pair kernels count
// FP64 instructions.  The common pair (source outside its changeover radius,
// K = 1, not the body itself) costs 18 FP64 operations:
//   d = x_i - x_j (3), r^2 (3), q = (r^2 + eps^2)^2 r^2 (3),
//   u = q^(-1/2) from an FP32 MUFU seed refined by one Halley step (5),
//   w = m u (1), acc += w d (3),
// i.e. u = 1 / ((r^2 + eps^2) r) to ~1 ulp.  Every other pair (inside the
// changeover radius, the body's own index, degenerate radii, distances
// outside the FP32 range of the seed) takes the reference formula
// (sim.cuh:339-375).  The decision "r > r_crit" is made on the high 32 bits of
// r^2 and r_crit^2 (integer compare on positive doubles), with a margin so
// that the fast branch is only taken where the reference's y > 1.
#pragma once
#include "merc_device.cuh"

namespace merc {

// A source of the fast path: position, mass, changeover radius and its
// products, and the high word threshold of r_crit^2 (INT_MAX when r_crit is
// not a positive finite number, which sends every pair to the exact branch).
struct FastSrc {
  double x, y, z, m, rc, rc01, rc09;
  int rc2_hi;
};

__device__ __forceinline__ int hi_word(double x) { return __double2hiint(x); }

// The fast-path threshold is stored in the fourth double of an r_crit table
// entry as integer bits, so that reading it back costs no double -> int
// conversion (which would occupy the FP64 pipe once per pair).
__device__ __forceinline__ double thr_pack(int t) { return __longlong_as_double((long long)t); }
__device__ __forceinline__ int thr_unpack(double d) { return (int)__double_as_longlong(d); }

// high-word threshold: r^2 hi word above this means r > r_crit with margin
// 0 < x < 1e150, on the bit pattern (positive doubles order like their bits;
// NaN, zeros and negatives fail as in the FP64 compares, which each take a
// slot of the FP64 pipe on this GPU)
__device__ __forceinline__ bool pos_below_1e150(double x) {
  const long long b = __double_as_longlong(x);
  return b > 0 && b < 0x5f138d352e5096afLL;  // the bits of 1e150
}
__device__ __forceinline__ int rc2_threshold(double rc) {
  if (!pos_below_1e150(rc)) return 0x7fffffff;
  return hi_word(rc * rc) + 1;
}

// 1 / ((r2 + eps2) sqrt(r2)) from an FP32 seed and one Halley step; valid
// when (r2 + eps2)^2 r2 is a normal FP32 number (checked by the caller).  The
// double <-> float moves of the seed are done on the integer pipes from the
// high word (exponent rebias by 1023 - 127 = 896), so the FP64 pipe only sees
// the 8 arithmetic operations (products as FMAs on the unit constants U).
__device__ __forceinline__ double inv_softened_r3(const FU& U, double r2, double s) {
  double q = fmul(U, s, s);
  q = fmul(U, q, r2);
  float qf = __int_as_float((__double2hiint(q) - 0x38000000) << 3);
  int yb = __float_as_int(rsqrtf(qf));
  double u = __hiloint2double((yb >> 3) + 0x38000000, yb << 29);
  double t = fmul(U, q, u);
  double e = fma(-t, u, 1.0);
  double c = fma(0.375, e, 0.5);
  double ue = fmul(U, u, e);
  return fma(ue, c, u);
}

// is q = (r2 + eps2)^2 r2 inside the FP32 normal range of the seed?  Checked
// on the high word of r2 (integer compare, positive doubles order like their
// bits): 2^-36 < r2 < 2^39 keeps q in [2^-108, 2^120] for eps2 <= 1.
__device__ __forceinline__ bool seed_in_range(double r2) {
  const int h = __double2hiint(r2);
  return h > 0x3DB00000 && h < 0x42600000;
}

// The reference's pair formula (sim.cuh:344-374): weight K or the encounter
// weighting, self exclusion, softening except for "self" -- for the
// universal-drift kernels, with the square root and the three divisions
// (r, the changeover argument y, K, and m / ((r^2 + eps^2) r)) by the
// FP32-seeded reciprocal square root and reciprocal, each within about an ulp
// of the IEEE operation (seed_range_ok; outside it, and for r^2 = 0, the IEEE
// forms).  On this GPU an FP64 square root or division costs about 8.5
// FP64-pipe slots, the seeded reciprocal 4.5 and reciprocal square root 5.8;
// the pair is on the chains of the kick reduce and inside the encounter
// sub-step's part sums.  The element drift keeps exact_term's IEEE form.
__device__ __forceinline__ double div_seeded(double x, double y) {
  return seed_range_ok(y) ? x * rcp_fast(y) : x / y;
}
// (inside [0, 1] the reference's K gtz valid + gto is K itself, and outside
// the finite range its form is kept; selects rather than products with 0/1
// factors, whose conversions and multiplications each take an FP64 slot)
__device__ __forceinline__ double changeover_K_seeded(double y) {
  if (y_above_one(y)) return 1.0;
  if (y_below_zero(y)) return 0.0;
  const double K = div_seeded(y * y, 2.0 * y * y - 2.0 * y + 1.0);
  if (y_in_unit(y)) return K;
  double gtz = (double)(y > 0.0), gto = (double)(y > 1.0), valid = (double)(y <= 1.0 && y >= 0.0);
  return K * gtz * valid + gto;
}
// The reference formula's factor wa and separation d of one pair
// (pair_exact adds wa d to its sum with three fmas)
template <bool BS>
__device__ __forceinline__ double pair_exact_w(const d3& pos, int self, int i, const FastSrc& S, double soft2,
                                               d3& d) {
  const FU U1 = {1.0, -0.0};
  d = {S.x - pos.x, S.y - pos.y, S.z - pos.z};
  double r_sq = mag2(d);
  double r = seed_range_ok(r_sq) ? r_sq * rsqrt_fast(U1, r_sq) : stable_sqrt(r_sq);
  // notself * r and notself * soft2 of the reference as selects (the same
  // values for finite r)
  const bool other = self != i;
  double K = changeover_K_seeded(div_seeded((other ? r : 0.0) - S.rc01, S.rc09));
  double w = K;
  // (r <= rc) (1 - K) + (r > rc) K: the same value, NaN where either is
  if (BS) w = r <= S.rc ? 1.0 - K : K;
  if (other) r_sq += soft2;
  const double den = r_sq * r;
  return w * ((__double_as_longlong(den) << 1) != 0 ? div_seeded(S.m, den) : stable_div(S.m, den));
}
template <bool BS>
__device__ __forceinline__ void pair_exact(const d3& pos, int self, int i, const FastSrc& S, double soft2, d3& acc) {
  d3 d;
  const double wa = pair_exact_w<BS>(pos, self, i, S, soft2, d);
  acc.x = fma(wa, d.x, acc.x);
  acc.y = fma(wa, d.y, acc.y);
  acc.z = fma(wa, d.z, acc.z);
}

// The encounter body's own frozen position as a source of its sub-step
// (sim.cuh:344-374 with notself = 0): K(y < 0) = 0, so the weight is 1 inside
// r_crit and 0 outside, with no softening: m (x_self - pos) / r^3 for r <=
// r_crit.  The same decision r <= r_crit as the reference; the fast formula
// for 1 / r^3 where r_crit is a positive finite number and r^2 is in the seed
// range, the reference formula otherwise.
__device__ __forceinline__ void bs_self_term(const FU& U, const d3& pos, int self, const FastSrc& S, double soft2,
                                             d3& acc) {
  const d3 d = {S.x - pos.x, S.y - pos.y, S.z - pos.z};
  const double r_sq = mag2(d);
  if (!(S.rc > 0.0) || !(S.rc < 1e150) || !seed_in_range(r_sq)) {
    pair_exact<true>(pos, self, self, S, soft2, acc);
    return;
  }
  if (!(stable_sqrt(r_sq) <= S.rc)) return;
  const double wa = fmul(U, S.m, inv_softened_r3(U, r_sq, r_sq));
  acc.x = fma(wa, d.x, acc.x);
  acc.y = fma(wa, d.y, acc.y);
  acc.z = fma(wa, d.z, acc.z);
}

// One pair on the fast path when possible.
template <bool BS>
__device__ __forceinline__ void pair_fast(const FU& U, const d3& pos, int self, int i, const FastSrc& S, double soft2,
                                          d3& acc) {
  double dx = fsub(U, S.x, pos.x), dy = fsub(U, S.y, pos.y), dz = fsub(U, S.z, pos.z);
  double r2 = fma(dx, dx, fma(dy, dy, fmul(U, dz, dz)));
  if (hi_word(r2) > S.rc2_hi && i != self && seed_in_range(r2)) {
    double w = fmul(U, S.m, inv_softened_r3(U, r2, fadd(U, r2, soft2)));
    acc.x = fma(w, dx, acc.x);
    acc.y = fma(w, dy, acc.y);
    acc.z = fma(w, dz, acc.z);
  } else if (BS && i == self) {
    bs_self_term(U, pos, self, S, soft2, acc);
  } else if (BS || i != self || r2 != 0.0) {
    // (in the plain kick a body's own entry, at distance zero, contributes
    // exactly zero: K = 0 and the guarded division returns 0)
    pair_exact<BS>(pos, self, i, S, soft2, acc);
  }
}

// pair_fast<false> as a term: whether the pair adds w d to the kick's sum
// (with the same three fmas), and w and d (the same values, so a sum of terms
// computed on other lanes and added in source order has pair_fast's bits)
__device__ __forceinline__ bool kick_term(const FU& U, const d3& pos, int self, int i, const FastSrc& S,
                                          double soft2, double& w, d3& d) {
  const double dx = fsub(U, S.x, pos.x), dy = fsub(U, S.y, pos.y), dz = fsub(U, S.z, pos.z);
  const double r2 = fma(dx, dx, fma(dy, dy, fmul(U, dz, dz)));
  if (hi_word(r2) > S.rc2_hi && i != self && seed_in_range(r2)) {
    w = fmul(U, S.m, inv_softened_r3(U, r2, fadd(U, r2, soft2)));
    d = {dx, dy, dz};
    return true;
  }
  if (i != self || r2 != 0.0) {
    w = pair_exact_w<false>(pos, self, i, S, soft2, d);
    return true;
  }
  return false;
}

// Sun pull of the encounter sub-stepper: -pos / ((r^2 + eps^2) r)
// (sim.cuh:431-441), fast where the seed range allows.
__device__ __forceinline__ d3 sun_accel(const FU& U, const d3& pos, double soft2) {
  double r2 = fma(pos.x, pos.x, fma(pos.y, pos.y, fmul(U, pos.z, pos.z)));
  double s = fadd(U, r2, soft2);
  if (seed_in_range(r2)) {
    double u = inv_softened_r3(U, r2, s);
    return {fmul(U, -pos.x, u), fmul(U, -pos.y, u), fmul(U, -pos.z, u)};
  }
  double r = stable_sqrt(r2);
  double denom = s * r;
  return {-(pos.x / denom), -(pos.y / denom), -(pos.z / denom)};
}

// Component c of sun_accel (posc = pos.x, pos.y or pos.z): the same operations.
__device__ __forceinline__ double sun_accel_c(const FU& U, const d3& pos, double posc, double soft2) {
  double r2 = fma(pos.x, pos.x, fma(pos.y, pos.y, fmul(U, pos.z, pos.z)));
  double s = fadd(U, r2, soft2);
  if (seed_in_range(r2)) return fmul(U, -posc, inv_softened_r3(U, r2, s));
  double r = stable_sqrt(r2);
  double denom = s * r;
  return -(posc / denom);
}

// x as an FP32 number by integer operations on the high word (sign, exponent
// rebias, the top 20 mantissa bits; no conversion on the FP64 pipe): within
// 2^-20 of x relative, 0 below the FP32 normal range (|x| < 2^-126), NaN above
// it and for infinities and NaN (so that the prefilter answers "maybe").
__device__ __forceinline__ float f32_trunc(double x) {
  const int h = __double2hiint(x), m = h & 0x7fffffff;
  if (m < 0x38100000) return 0.0f;
  if (m >= 0x47F00000) return __int_as_float(0x7fc00000);
  return __int_as_float((h & (int)0x80000000) | ((m - 0x38000000) << 3));
}

// FP32 positions of a body for the encounter prefilter: float copies and the
// largest component magnitude (the scale of their truncation error).
struct F4 {
  float x, y, z, sc;
};
__device__ __forceinline__ F4 f4_of(float x, float y, float z) {
  return {x, y, z, fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z)))};
}

// FP32 prefilter of the encounter test: false only when the pair is certainly
// farther apart than r_crit.  The float copies (f32_trunc) are off by at most
// 2^-20 of the body's largest coordinate (2^-126 below the normal range), the
// difference and its square add a few 2^-24 relative roundings, so |d| >=
// |d_f| (1 - 3e-7) - 1.7e-6 (sc_s + sc_t) - 4e-38, and r_crit in FP32 is at
// most 2^-20 below r_crit; the limit r_crit (1 + 1e-5) + 1e-5 (sc_s + sc_t) +
// 1e-37 covers that with room.  NaN anywhere -> maybe.
__device__ __forceinline__ bool ce_maybe(const F4& t, const F4& s, float rc) {
  float dx = s.x - t.x, dy = s.y - t.y, dz = s.z - t.z;
  float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  float lim = fmaf(rc, 1.00001f, fmaf(1e-5f, s.sc + t.sc, 1e-37f));
  return !(r2 > lim * lim && lim > 0.0f);
}

// ce_maybe of a pair in both directions (t vs source s with r_crit rc_s, s vs
// source t with rc_t), the distance computed once: the same answers as two
// ce_maybe calls (the difference changes sign exactly, the scale sum is
// commutative).
__device__ __forceinline__ void ce_maybe2(const F4& t, const F4& s, float rc_s, float rc_t, bool& m_t, bool& m_s) {
  float dx = s.x - t.x, dy = s.y - t.y, dz = s.z - t.z;
  float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float pad = fmaf(1e-5f, s.sc + t.sc, 1e-37f);
  const float lt = fmaf(rc_s, 1.00001f, pad), ls = fmaf(rc_t, 1.00001f, pad);
  m_t = !(r2 > lt * lt && lt > 0.0f);
  m_s = !(r2 > ls * ls && ls > 0.0f);
}

// Encounter test of one pair, exact: sqrt(r^2) < r_crit and not self
// (sim.cuh:602-609); the sqrt is skipped when r^2 is clearly above r_crit^2.
__device__ __forceinline__ bool pair_ce(const d3& pos, int self, int i, const FastSrc& S) {
  double dx = S.x - pos.x, dy = S.y - pos.y, dz = S.z - pos.z;
  double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
  if (hi_word(r2) > S.rc2_hi) return false;
  return (sqrt(r2) < S.rc) && (self != i);
}

// The same test behind the FP32 prefilter (no FP64 work for far pairs).
__device__ __forceinline__ bool pair_ce_f(const d3& pos, const F4& tf, int self, int i, const FastSrc& S,
                                          const F4& sf) {
  if (!ce_maybe(tf, sf, f32_trunc(S.rc))) return false;
  return pair_ce(pos, self, i, S);
}

}  // namespace merc
