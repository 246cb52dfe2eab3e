// merc_kernels.cuh - kernels of the Mercurius step (included by merc_engine.cu).
//
// Systems are classified at load time:
//  - small systems (n_massive <= kSmallNm) are served one thread per body,
//    each thread looping over its system's few sources (read-only cache
//    broadcasts); the encounter sub-step is one thread per encounter body;
//  - big systems (more sources) are served by work items of kTile targets x a
//    chunk of sources, so a single system of ~2000 bodies fills all SMs; the
//    per-chunk partial sums go to a scratch buffer and are added in chunk
//    order (deterministic); the encounter sub-step gives each encounter body
//    one block whose threads split the sources.
// The element-drift path always uses the exact per-body kernels (reference
// operation order); the universal path uses the classified fast kernels.
#pragma once
#include <cooperative_groups.h>

namespace {

constexpr int kThreads = 128;
constexpr int kNumCounters = 5;  // entries of Dev::counters
constexpr int kTile = 128;       // targets per work item (one per thread)
constexpr int kSrcTile = 256;    // sources staged in shared memory per pass
constexpr int kSmallNm = 32;     // systems with more sources use the tiled kernels
constexpr int kEncThreads = 128; // threads per block of an encounter body of a big system
constexpr int kEncCluster = 4;   // blocks (a thread-block cluster) per encounter body of a big system

// Programmatic dependent launch: wait until the preceding kernel of the
// stream has completed and its writes are visible (a no-op when the kernel
// was launched without the attribute), then allow the next kernel to be
// scheduled.  Called first in every kernel of the step graphs.
__device__ __forceinline__ void griddep_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Let the next kernel of the stream launch before this one completes (it
// still waits in griddep_enter unless it is written to wait elsewhere).
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// The dependency wait of griddep_enter, for a kernel that waits at its end.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

struct Work {
  int sys, t0, c0, c1, chunk;
};

struct Dev {
  FU u = {1.0, -0.0};  // run-time unit constants (fadd / fmul)
  int n = 0;     // bodies, all systems
  int nsys = 0;  // systems
  const int* off = nullptr;
  const int* nm = nullptr;
  int nm0 = 0;  // massive bodies of system 0 when it is the only system (read without a load)
  const int* sys = nullptr;  // system of each body
  const unsigned char* big = nullptr;  // per system: served by the tiled kernels
  const int* nchunk = nullptr;         // per system: source chunks of the tiled kick
  double* x = nullptr;       // 3 n
  double* v = nullptr;       // 3 n
  float* xf = nullptr;       // 3 n, FP32 copies of x after each solar jump (encounter prefilter)
  double* xo = nullptr;      // 3 n, drift output
  double* vo = nullptr;      // 3 n
  const double* m = nullptr;
  double* hc = nullptr;      // n, cbrt(m / 3) * hill_factor (massive bodies; written by k_rc)
  double* alag = nullptr;
  uint32_t* flags = nullptr;
  unsigned char* ce = nullptr;  // encounter flag of the current step
  // 4 doubles per body: rc, 0.1 rc, 0.9 rc, fast threshold (massive bodies),
  // then one int per body: the far-field threshold (rc_far_thr)
  double* rc[2] = {nullptr, nullptr};
  double* P = nullptr;               // 3 per system
  double* part = nullptr;            // kick partial sums of test-particle targets [chunk][3][n]
  double* part_sym = nullptr;        // far-field partial sums of massive targets, 2 sets of per system [block][3][nm]
  uint32_t* near_mask = nullptr;     // near-pair bits, 2 sets of per system [block][nm] (one bit per source)
  const long long* sym_base = nullptr;  // per system: offset of its block partials in a set (-1: none)
  long long sym_set = 0;             // doubles per partial set (the mask set has sym_set / 3 words)
  int* gate = nullptr;               // set when a merged kick must recompute the far field
  // a single big system: bit b set when a body of its 32-body block b moved its
  // far-field threshold (gate_words words; cleared with the gate)
  unsigned long long* gate_blocks = nullptr;
  int gate_words = 0;
  double* far_acc = nullptr;         // 3 n: far-field sum of each massive body of a big system, kept by
                                     //     the first reduce of a merged kick for the second
  unsigned long long* far_recomputes = nullptr;  // gated far-field passes that ran
  int* ce_list = nullptr;            // encounter bodies of small systems
  int* ce_list_big = nullptr;        // encounter bodies of big systems
  int* ce_count = nullptr;           // [0] small list, [1] big list
  unsigned long long* counters = nullptr;  // kNumCounters: CE body-steps, Kepler iterations, solves,
                                           // non-converged, iterations executed per warp (SIMT)
  // encounter task kernel, per entry of the big-system encounter list:
  double* enc_q = nullptr;    // kEncQ: part sums of the 7 evaluations (enc_parts(row, e) x 3 each)
  double* enc_st = nullptr;   // 27: per row z0, z1, vel after its last published evaluation
  double* enc_res = nullptr;  // 18: per row the sub-step result (position, velocity)
  int* enc_cnt = nullptr;     // 11: parts done per evaluation (7), evaluations published per row (3),
                              //     rows done (1); zero between steps
  int* enc_head = nullptr;    // [0] next task (cleared by the first jump), [1] a bounded wait gave up
};

__device__ __forceinline__ SrcView src_view(const Dev& D, const double* rc, int b0) {
  SrcView S;
  S.x = D.x + b0;
  S.y = D.x + D.n + b0;
  S.z = D.x + 2 * D.n + b0;
  S.m = D.m + b0;
  S.rc = rc + 4 * (size_t)b0;
  S.u = D.u;
  return S;
}

__device__ __forceinline__ d3 load3(const double* a, int n, int j) { return {a[j], a[n + j], a[2 * n + j]}; }
__device__ __forceinline__ void store3(double* a, int n, int j, const d3& v) {
  a[j] = v.x;
  a[n + j] = v.y;
  a[2 * n + j] = v.z;
}
__device__ __forceinline__ int self_index(int local, int compat_block) {
  return compat_block > 0 ? local % compat_block : local;
}

// Doubles of one r_crit table of n bodies (4 doubles and one int per body).
__host__ __device__ constexpr size_t rc_table_doubles(size_t n) { return 4 * n + (n + 1) / 2; }
__device__ __forceinline__ int* rc_far_thr(const double* rc, int n) { return (int*)(rc + 4 * (size_t)n); }
__device__ __forceinline__ const int* rc_far_thr_c(const double* rc, int n) {
  return (const int*)(rc + 4 * (size_t)n);
}

// Far-field radius of a source: kFarRadius Hill-scaled heliocentric
// distances, T = max(R, r_crit) with R = kFarRadius * |x| * cbrt(m/3) * hill.
// r_crit = a cbrt(m/3) hill, so T = R whenever a <= kFarRadius |x|, which
// holds for bound orbits with e < 1/3; then T depends on the position alone
// and the two kicks around a step boundary (same positions, r_crit before
// and after the first of them) split their pairs identically.  Returned as
// the high-word threshold of T^2 (a pair is far when hi(r^2) exceeds it);
// no far pairs for a source without a finite positive r_crit.
constexpr double kFarRadius = 1.5;
__device__ __forceinline__ int far_threshold(double rc, const d3& x, double hc) {
  if (!pos_below_1e150(rc)) return 0x7fffffff;
  const double R = kFarRadius * hc * sqrt(mag2(x));
  return rc2_threshold(R > rc ? R : rc);
}

// r_crit table entries of massive body j; hc = cbrt(m_j / 3) * hill_factor;
// returns the far-field threshold it wrote
__device__ __forceinline__ int write_rc(double* rc, int n, int j, const d3& x, const d3& v, double hc) {
  double r = rcrit_hc(x, v, hc);
  rc[4 * (size_t)j] = r;
  rc[4 * (size_t)j + 1] = 0.1 * r;
  rc[4 * (size_t)j + 2] = 0.9 * r;
  rc[4 * (size_t)j + 3] = thr_pack(rc2_threshold(r));
  const int far = far_threshold(r, x, hc);
  rc_far_thr(rc, n)[j] = far;
  return far;
}

// write_rc for the universal-drift path, where the kernels are checked
// against the CPU check to 1e-12 rather than bit for bit: the reference's
// r_crit formula (rcrit_hc) with 1 / |x| from the FP32-seeded reciprocal
// square root, |x| = |x|^2 (1 / |x|), and the division by 1 - e^2 as a
// multiplication by the seeded reciprocal (each within about an ulp of the
// IEEE operation; outside the seed range, or for 1 - e^2 <= 0, the IEEE
// forms).  The square root and the two divisions of write_rc were the
// longest part of the solar jump (3.9 of its 8 us, %globaltimer stamps per
// phase).
__device__ __forceinline__ int write_rc_fast(const FU& U, double* rc, int n, int j, const d3& x, const d3& v,
                                             double hc) {
  const d3 h = {fma(x.y, v.z, -x.z * v.y), fma(x.z, v.x, -x.x * v.z), fma(x.x, v.y, -x.y * v.x)};
  const double h2 = mag2(h);
  const double xx = mag2(x);
  const double ir = rsqrt_fast(U, xx);
  const double v2 = mag2(v);
  const double rdv = fma(x.x, v.x, fma(x.y, v.y, x.z * v.z));
  const double factor = v2 - ir;
  const d3 ev = {fma(factor, x.x, -rdv * v.x), fma(factor, x.y, -rdv * v.y), fma(factor, x.z, -rdv * v.z)};
  const double q = 1.0 - mag2(ev);
  // (q > 0 on the bit pattern: positive, not NaN)
  const long long qb = __double_as_longlong(q);
  const double a = (qb > 0 && qb <= 0x7ff0000000000000LL) ? h2 * rcp_fast(q) : h2 / q;
  const double r = a * hc;
  rc[4 * (size_t)j] = r;
  rc[4 * (size_t)j + 1] = 0.1 * r;
  rc[4 * (size_t)j + 2] = 0.9 * r;
  rc[4 * (size_t)j + 3] = thr_pack(rc2_threshold(r));
  int far = 0x7fffffff;
  if (pos_below_1e150(r)) {
    const double R = kFarRadius * hc * (xx * ir);
    far = rc2_threshold(R > r ? R : r);
  }
  rc_far_thr(rc, n)[j] = far;
  return far;
}

__device__ __forceinline__ F4 load_f4(const Dev& D, int g) {
  return f4_of(__ldg(D.xf + g), __ldg(D.xf + D.n + g), __ldg(D.xf + 2 * D.n + g));
}

__device__ __forceinline__ FastSrc load_src(const Dev& D, const double* __restrict__ rc, int g) {
  FastSrc S;
  S.x = __ldg(D.x + g);
  S.y = __ldg(D.x + D.n + g);
  S.z = __ldg(D.x + 2 * D.n + g);
  S.m = __ldg(D.m + g);
  S.rc = __ldg(rc + 4 * (size_t)g);
  S.rc01 = __ldg(rc + 4 * (size_t)g + 1);
  S.rc09 = __ldg(rc + 4 * (size_t)g + 2);
  S.rc2_hi = thr_unpack(__ldg(rc + 4 * (size_t)g + 3));
  return S;
}

// after a kick: store v, r_crit of the new state for massive bodies, flags
__device__ __forceinline__ void kick_epilogue(const Dev& D, int j, int local, int nm, const d3& pos, const d3& vel,
                                              double* rc_out, double hill, double eject_r2, int last) {
  store3(D.v, D.n, j, vel);
  if (rc_out && local < nm) write_rc(rc_out, D.n, j, pos, vel, D.hc[j]);
  if (last) {
    uint32_t f = D.flags[j] & ~MERC_FLAG_CE_LAST;
    if (D.ce[j]) f |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
    if (eject_r2 > 0.0 && mag2(pos) > eject_r2) f |= MERC_FLAG_EJECTED;
    bool fin = mm::isfinite_(pos.x) && mm::isfinite_(pos.y) && mm::isfinite_(pos.z) && mm::isfinite_(vel.x) &&
               mm::isfinite_(vel.y) && mm::isfinite_(vel.z);
    if (!fin) f |= MERC_FLAG_NONFINITE;
    D.flags[j] = f;
  }
}

// ---------------------------------------------------------------------------
// prologue / epilogue kernels (sim.cuh:654-677 and :744-765)
// ---------------------------------------------------------------------------
__global__ void k_from_elements(Dev D, const double* __restrict__ el, int iters) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n;
  PV pv = cart_from_elem(el[j], el[n + j], el[2 * n + j], el[3 * n + j], el[4 * n + j], el[5 * n + j], iters);
  store3(D.x, n, j, pv.pos);
  store3(D.v, n, j, pv.vel);
  D.alag[j] = el[5 * n + j];
}

__global__ void k_to_elements(Dev D, double* __restrict__ el) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n;
  Elem e = elem_from_cart(load3(D.x, n, j), load3(D.v, n, j));
  el[j] = e.inc;
  el[n + j] = e.node;
  el[2 * n + j] = e.peri;
  el[3 * n + j] = e.M;
  el[4 * n + j] = e.e;
  el[5 * n + j] = e.a;
}

// democratic_heliocentric_conversion (sim.cuh:555-587): per-system sums in the
// reference order, then every body of the system is shifted.
__global__ void k_dh_sums(Dev D, bool reverse) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.nsys) return;
  const int b0 = D.off[s], nm = D.nm[s], n = D.n;
  double total = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
  for (int i = 0; i < nm; i++) {
    double mi = D.m[b0 + i];
    total += mi;
    mx = fma(mi, D.v[b0 + i], mx);
    my = fma(mi, D.v[n + b0 + i], my);
    mz = fma(mi, D.v[2 * n + b0 + i], mz);
  }
  double not_rev = reverse ? 0.0 : 1.0;
  double scale = 1.0 / fma(not_rev, total, 1.0);
  D.P[3 * s] = mx * scale;
  D.P[3 * s + 1] = my * scale;
  D.P[3 * s + 2] = mz * scale;
}

__global__ void k_dh_apply(Dev D, double sgn) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int s = D.sys[j], n = D.n;
  D.v[j] = fma(sgn, D.P[3 * s], D.v[j]);
  D.v[n + j] = fma(sgn, D.P[3 * s + 1], D.v[n + j]);
  D.v[2 * n + j] = fma(sgn, D.P[3 * s + 2], D.v[2 * n + j]);
}

__global__ void k_rc(Dev D, double* rc_out, double hill) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int s = D.sys[j];
  if (j - D.off[s] >= D.nm[s]) return;
  const double hc = mm::cbrt(D.m[j] / 3.0) * hill;
  D.hc[j] = hc;
  write_rc(rc_out, D.n, j, load3(D.x, D.n, j), load3(D.v, D.n, j), hc);
}

// ---------------------------------------------------------------------------
// exact path (element drift): reference operation order
// ---------------------------------------------------------------------------
// Half kick of every body (sim.cuh:683-685, 739-741); skip_big leaves the
// bodies of big systems to k_kick_big_exact_pipe.
__global__ void k_kick(Dev D, const double* __restrict__ rc_in, double* __restrict__ rc_out, double hdt,
                       double soft2, int compat_block, double hill, double eject_r2, int last, int skip_big) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
  if (skip_big && D.big[s]) return;
  const int local = j - b0;
  SrcView S = src_view(D, rc_in, b0);
  d3 pos = load3(D.x, n, j);
  d3 vel = kick_exact<false>(pos, load3(D.v, n, j), self_index(local, compat_block), S, nm, hdt, soft2);
  kick_epilogue(D, j, local, nm, pos, vel, rc_out, hill, eject_r2, last);
}

// The exact path of the big systems (warp_kick_exact and
// warp_close_encounter give the bits of the per-thread forms): the same
// arithmetic and order, with the source terms computed 32 at a time.
constexpr int kExactWarps = 4;  // warps per block

// The kick of the big systems' bodies as a pipeline: one block per group of
// G <= kPipeGroupMax bodies of one system, warp 0 runs the 3G fma chains
// (lane 3b + c: body b, component c) while kPipeTermWarps warps compute the
// next 32 sources' terms for the G bodies (exact_term), double-buffered in
// shared memory.  The reference's order ends every source term in a
// sequential fma chain per body and component; a chain step is a warp
// instruction on the FP64 pipe however few lanes run it (one body per warp,
// lanes 0-2: ~32 of ~72 FP64 instructions per directed pair), so one step
// here serves G bodies, and the term warps do not wait for the chain's
// ~90-cycle dependent steps.  Same bits as warp_kick_exact.
constexpr int kPipeTermWarps = 3;
constexpr int kPipeGroupMax = 9;
__global__ void __launch_bounds__(32 * (1 + kPipeTermWarps))
    k_kick_big_exact_pipe(Dev D, const int2* __restrict__ groups, int ngroups, const double* __restrict__ rc_in,
                          double* __restrict__ rc_out, double hdt, double soft2, int compat_block, double hill,
                          double eject_r2, int last) {
  __shared__ double stage[2][kPipeGroupMax][4][32];
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int j0 = groups[g].x, cnt = groups[g].y;
    const int n = D.n, s = D.sys[j0], b0 = D.off[s], nm = D.nm[s];
    SrcView S = src_view(D, rc_in, b0);
    const int nchunks = (nm + 31) / 32;
    double acc = 0.0;
    for (int c = 0; c <= nchunks; c++) {
      if (warp > 0 && c < nchunks) {
        const int i = 32 * c + lane;
        for (int b = warp - 1; b < cnt; b += kPipeTermWarps) {
          const d3 pos = load3(D.x, n, j0 + b);
          d3 d = {0.0, 0.0, 0.0};
          const double wa = i < nm ? exact_term<false>(pos, self_index(j0 + b - b0, compat_block), S, i, soft2, d)
                                   : 0.0;
          double* st = stage[c & 1][b][0];
          st[lane] = wa;
          st[32 + lane] = d.x;
          st[64 + lane] = d.y;
          st[96 + lane] = d.z;
        }
      }
      if (warp == 0 && c >= 1 && lane < 3 * cnt) {
        const int cb = lane / 3, cc = lane - 3 * cb;
        acc = chain_fma<32>(stage[(c - 1) & 1][cb][0], stage[(c - 1) & 1][cb][1 + cc], min(32, nm - 32 * (c - 1)),
                            acc);
      }
      __syncthreads();
    }
    if (warp == 0) {
      for (int b = 0; b < cnt; b++) {
        const double ax = __shfl_sync(0xffffffffu, acc, 3 * b), ay = __shfl_sync(0xffffffffu, acc, 3 * b + 1),
                     az = __shfl_sync(0xffffffffu, acc, 3 * b + 2);
        if (lane == b) {
          const int j = j0 + b;
          const d3 pos = load3(D.x, n, j);
          d3 vel = load3(D.v, n, j);
          vel.x = fma(ax, hdt, vel.x);
          vel.y = fma(ay, hdt, vel.y);
          vel.z = fma(az, hdt, vel.z);
          kick_epilogue(D, j, j - b0, nm, pos, vel, rc_out, hill, eject_r2, last);
        }
      }
    }
  }
}

// Encounter flags of the bodies of big systems (close_encounter_p,
// sim.cuh:589-613), one warp per body, for k_drift_elements.
__global__ void __launch_bounds__(32 * kExactWarps) k_ce_big_exact(Dev D, const double* __restrict__ rc_in,
                                                                   int compat_block) {
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  for (int j = blockIdx.x * kExactWarps + warp; j < D.n; j += gridDim.x * kExactWarps) {
    const int n = D.n, s = D.sys[j];
    if (!D.big[s]) continue;
    const int b0 = D.off[s], nm = D.nm[s];
    SrcView S = src_view(D, rc_in, b0);
    // close_encounter_p by the warp, behind the FP32 prefilter: a pair that
    // ce_maybe clears is certainly outside r_crit (its proven bound) and
    // needs no FP64 work; every other pair takes the reference's test, so the
    // flag is warp_close_encounter's
    const d3 pos = load3(D.x, n, j);
    const F4 pf = load_f4(D, j);
    const int self = self_index(j - b0, compat_block);
    bool ce = false;
    for (int i = lane; i < nm; i += 32)
      if (ce_maybe(pf, load_f4(D, b0 + i), f32_trunc(S.rc[4 * (size_t)i]))) ce = ce || ce_pair(pos, self, S, i);
    ce = __any_sync(0xffffffffu, ce);
    if (lane == 0) {
      D.ce[j] = ce;
      if (ce) {  // the encounter list of the element path (k_drift_elements lists the small systems')
        D.ce_list[atomicAdd(&D.ce_count[0], 1)] = j;
        atomicAdd(&D.counters[0], 1ull);
      }
    }
  }
}

// sum_i m_i v_i of each big system in the reference order (main_body_kinetic,
// sim.cuh:394-399), one warp per system: the masses and velocities of 32
// bodies loaded at a time (the next chunk's loads issued before the current
// chunk is added), added in body order by lanes 0-2 with the reference's fma
// chain, one component each.
__global__ void __launch_bounds__(32 * kExactWarps) k_momentum_big_exact(Dev D, const double* __restrict__ vsrc) {
  __shared__ double stage[kExactWarps][128];
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  double* st = stage[warp];
  for (int s = blockIdx.x * kExactWarps + warp; s < D.nsys; s += gridDim.x * kExactWarps) {
    if (!D.big[s]) continue;
    const int b0 = D.off[s], nm = D.nm[s], n = D.n;
    double acc = 0.0;  // lane c < 3: component c
    double m = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
    if (lane < nm) {
      m = D.m[b0 + lane];
      vx = vsrc[b0 + lane];
      vy = vsrc[n + b0 + lane];
      vz = vsrc[2 * n + b0 + lane];
    }
    for (int base = 0; base < nm; base += 32) {
      st[lane] = m;
      st[32 + lane] = vx;
      st[64 + lane] = vy;
      st[96 + lane] = vz;
      __syncwarp();
      const int i = base + 32 + lane;
      m = vx = vy = vz = 0.0;
      if (i < nm) {
        m = D.m[b0 + i];
        vx = vsrc[b0 + i];
        vy = vsrc[n + b0 + i];
        vz = vsrc[2 * n + b0 + i];
      }
      if (lane < 3) {
        const int cnt = min(32, nm - base);
        const double* vc = st + 32 * (lane + 1);
        acc = chain_fma<32>(st, vc, cnt, acc);
      }
      __syncwarp();
    }
    if (lane < 3) D.P[3 * s + lane] = acc;
  }
}

// sum_i m_i v_i of each system in the reference order (main_body_kinetic,
// sim.cuh:394-399); `vsrc` is the velocity array to sum.  skip_big leaves the
// big systems to k_momentum_big.
__global__ void k_momentum(Dev D, const double* __restrict__ vsrc, int skip_big) {
  griddep_enter();
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.nsys) return;
  if (skip_big && D.big[s]) return;
  const int b0 = D.off[s], nm = D.nm[s], n = D.n;
  double px = 0.0, py = 0.0, pz = 0.0;
  for (int i = 0; i < nm; i++) {
    double mi = D.m[b0 + i];
    px = fma(mi, vsrc[b0 + i], px);
    py = fma(mi, vsrc[n + b0 + i], py);
    pz = fma(mi, vsrc[2 * n + b0 + i], pz);
  }
  D.P[3 * s] = px;
  D.P[3 * s + 1] = py;
  D.P[3 * s + 2] = pz;
}

// Solar jump x = xsrc + dt/2 P (sim.cuh:402-404); copies vsrc -> v when the
// drift wrote to the output buffers; massive bodies write their new r_crit.
// BIG_P: the momentum P = sum m v of every big system is summed here by each
// block that holds bodies of the system (thread t adds massive bodies t,
// t + 128, ..., then a fixed tree, so every block gets the same bits); small
// systems read D.P (k_momentum).  CLEAR: also clears the encounter flags and
// list counts for the step's encounter test.
#ifndef MERC_JUMP_THREADS
#define MERC_JUMP_THREADS 128
#endif
constexpr int kJumpThreads = MERC_JUMP_THREADS;  // block of the universal-path jumps
#ifndef MERC_JUMP_BATCH
#define MERC_JUMP_BATCH 8
#endif
constexpr int kJumpBatch = MERC_JUMP_BATCH;  // momentum terms loaded per thread before they are added
template <bool BIG_P, bool CLEAR>
__global__ void __launch_bounds__(kJumpThreads) k_jump(Dev D, const double* __restrict__ xsrc,
                                                      const double* __restrict__ vsrc, double* rc_out, double hdt) {
  griddep_enter();
  __shared__ double wsum[kJumpThreads / 32][3];
  __shared__ double Pb[kJumpThreads][3];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    if (D.gate) *D.gate = 0;  // the last merged kick has read it
    if (CLEAR) D.ce_count[0] = D.ce_count[1] = 0;
    if (CLEAR && D.enc_head) D.enc_head[0] = 0;
  }
  if (D.gate_blocks && j < D.gate_words) D.gate_blocks[j] = 0ull;
  const int n = D.n;
  const int j0 = blockIdx.x * blockDim.x, j1 = min(n, j0 + (int)blockDim.x);
  if (j0 >= n) return;  // whole block
  const int s0 = D.sys[j0];
  if (BIG_P) {
    // thread t adds massive bodies t, t + B, ...; a fixed butterfly per warp;
    // thread 0 adds the warp sums in warp order
    const int s1 = D.sys[j1 - 1];
    const double* vv = vsrc ? vsrc : D.v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = s0; q <= s1; q++) {
      if (!D.big[q]) continue;  // the same for every thread of the block
      const int b0 = D.off[q], nm = D.nm[q];
      double px = 0.0, py = 0.0, pz = 0.0;
      // kJumpBatch bodies' loads in flight before their products are added
      // (same order of additions as one body at a time)
      for (int i0 = threadIdx.x; i0 < nm; i0 += kJumpBatch * (int)blockDim.x) {
        double mb[kJumpBatch], xb[kJumpBatch], yb[kJumpBatch], zb[kJumpBatch];
#pragma unroll
        for (int u = 0; u < kJumpBatch; u++) {
          const int i = i0 + u * (int)blockDim.x;
          const bool ok = i < nm;
          mb[u] = ok ? D.m[b0 + i] : 0.0;
          xb[u] = ok ? vv[b0 + i] : 0.0;
          yb[u] = ok ? vv[n + b0 + i] : 0.0;
          zb[u] = ok ? vv[2 * n + b0 + i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kJumpBatch; u++) {
          if (i0 + u * (int)blockDim.x < nm) {
            px = fma(mb[u], xb[u], px);
            py = fma(mb[u], yb[u], py);
            pz = fma(mb[u], zb[u], pz);
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        px += __shfl_xor_sync(0xffffffffu, px, o);
        py += __shfl_xor_sync(0xffffffffu, py, o);
        pz += __shfl_xor_sync(0xffffffffu, pz, o);
      }
      if (lane == 0) {
        wsum[warp][0] = px;
        wsum[warp][1] = py;
        wsum[warp][2] = pz;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int w = 0; w < nw; w++) {
          sx += wsum[w][0];
          sy += wsum[w][1];
          sz += wsum[w][2];
        }
        Pb[q - s0][0] = sx;
        Pb[q - s0][1] = sy;
        Pb[q - s0][2] = sz;
      }
      __syncthreads();
    }
  }
  if (j >= n) return;
  const int s = D.sys[j];
  if (CLEAR) D.ce[j] = 0;
  double px, py, pz;
  if (BIG_P && D.big[s]) {
    px = Pb[s - s0][0];
    py = Pb[s - s0][1];
    pz = Pb[s - s0][2];
  } else {
    px = D.P[3 * s];
    py = D.P[3 * s + 1];
    pz = D.P[3 * s + 2];
  }
  d3 x = load3(xsrc, n, j);
  x.x = fma(px, hdt, x.x);
  x.y = fma(py, hdt, x.y);
  x.z = fma(pz, hdt, x.z);
  store3(D.x, n, j, x);
  D.xf[j] = f32_trunc(x.x);
  D.xf[n + j] = f32_trunc(x.y);
  D.xf[2 * n + j] = f32_trunc(x.z);
  d3 v;
  if (vsrc) {
    v = load3(vsrc, n, j);
    store3(D.v, n, j, v);
  } else {
    v = load3(D.v, n, j);
  }
  if (j - D.off[s] < D.nm[s]) {
    if (BIG_P)  // big systems, universal drift only
      write_rc_fast(D.u, rc_out, n, j, x, v, D.hc[j]);
    else
      write_rc(rc_out, n, j, x, v, D.hc[j]);
  }
}

// Totals of (x, y, z) over the 32 lanes of a warp by a reduce-scatter: at the
// first level lanes 0-15 keep x and y and lanes 16-31 keep z (and an empty
// fourth sum), at the second each group of eight lanes keeps one component,
// and three more levels finish it; six FP64 additions in all, against fifteen
// for three butterflies (the FP64 pipe is the bound of the sub-step).  A fixed
// tree: every lane ends with the same totals, whatever the schedule.
__device__ __forceinline__ d3 warp_sum3(const FU& U, const d3& a) {
  const unsigned full = 0xffffffffu;
  const int lane = (int)(threadIdx.x & 31);
  const bool up = (lane & 16) != 0, b3 = (lane & 8) != 0;
  double k0 = up ? a.z : a.x, k1 = up ? 0.0 : a.y;
  const double s0 = up ? a.x : a.z, s1 = up ? a.y : 0.0;
  k0 = fadd(U, k0, __shfl_xor_sync(full, s0, 16));
  k1 = fadd(U, k1, __shfl_xor_sync(full, s1, 16));
  double k = b3 ? k1 : k0;
  k = fadd(U, k, __shfl_xor_sync(full, b3 ? k0 : k1, 8));
  k = fadd(U, k, __shfl_xor_sync(full, k, 4));
  k = fadd(U, k, __shfl_xor_sync(full, k, 2));
  k = fadd(U, k, __shfl_xor_sync(full, k, 1));
  return {__shfl_sync(full, k, 0), __shfl_sync(full, k, 8), __shfl_sync(full, k, 16)};
}

// Solar jump of a single big system (system 0 holds every body) by clusters
// of kJumpCluster blocks: block r of a cluster sums the momentum of massive
// bodies [r nm / 8, (r + 1) nm / 8) (thread t adds bodies t, t + B, ...;
// warp_sum3 per warp; warp sums in warp order), the cluster exchanges
// the eight partials through distributed shared memory and every block adds
// them in rank order, so every cluster gets the same bits with one eighth of
// the momentum work per block.  Then as k_jump: x = xsrc + dt/2 P, v copied
// from vsrc when given, new r_crit of massive bodies; CLEAR also clears the
// encounter flags and list counts.  The grid is a whole number of clusters.
constexpr int kJumpCluster = 8;
template <bool CLEAR>
__global__ void __cluster_dims__(kJumpCluster, 1, 1) __launch_bounds__(kJumpThreads)
    k_jump_cluster(Dev D, const double* __restrict__ xsrc, const double* __restrict__ vsrc, double* rc_out,
                   double hdt) {
  griddep_enter();
  namespace cg = cooperative_groups;
  __shared__ double wsum[kJumpThreads / 32][3];
  __shared__ double part[3];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    if (D.gate) *D.gate = 0;  // the last merged kick has read it
    if (CLEAR) D.ce_count[0] = D.ce_count[1] = 0;
    if (CLEAR && D.enc_head) D.enc_head[0] = 0;
  }
  if (D.gate_blocks && j < D.gate_words) D.gate_blocks[j] = 0ull;
  const int n = D.n, nm = D.nm0;
  const double* vv = vsrc ? vsrc : D.v;
  // this thread's body, loaded before the momentum (it does not depend on it)
  const bool mine = j < n;
  const d3 x0 = mine ? load3(xsrc, n, j) : d3{0.0, 0.0, 0.0};
  const d3 v = mine ? load3(vv, n, j) : d3{0.0, 0.0, 0.0};
  const double hc_j = (mine && j < nm) ? D.hc[j] : 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int i0 = (int)((int64_t)rank * nm / kJumpCluster), i1 = (int)((int64_t)(rank + 1) * nm / kJumpCluster);
  double px = 0.0, py = 0.0, pz = 0.0;
  for (int c = i0 + (int)threadIdx.x; c < i1; c += kJumpBatch * (int)blockDim.x) {
    double mb[kJumpBatch], xb[kJumpBatch], yb[kJumpBatch], zb[kJumpBatch];
#pragma unroll
    for (int u = 0; u < kJumpBatch; u++) {
      const int i = c + u * (int)blockDim.x;
      const bool ok = i < i1;
      mb[u] = ok ? D.m[i] : 0.0;
      xb[u] = ok ? vv[i] : 0.0;
      yb[u] = ok ? vv[n + i] : 0.0;
      zb[u] = ok ? vv[2 * n + i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kJumpBatch; u++) {
      if (c + u * (int)blockDim.x < i1) {
        px = fma(mb[u], xb[u], px);
        py = fma(mb[u], yb[u], py);
        pz = fma(mb[u], zb[u], pz);
      }
    }
  }
  // (every FP64 instruction of these sums costs its warp's sub-partition a
  // full warp slot however few lanes need the result, and each warp of this
  // kernel is alone on its sub-partition: the sums run one component per
  // lane where they can)
  const d3 wt = warp_sum3(D.u, d3{px, py, pz});
  if (lane == 0) {
    wsum[warp][0] = wt.x;
    wsum[warp][1] = wt.y;
    wsum[warp][2] = wt.z;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double sc = 0.0;
    for (int w = 0; w < nw; w++) sc += wsum[w][threadIdx.x];
    part[threadIdx.x] = sc;
  }
  cl.sync();
  // the partials of the cluster's blocks, added in rank order by lanes 0-2
  // of every warp (one component each; the remote loads in flight before the
  // additions), then handed to the other lanes
  double q[kJumpCluster];
  const int c = lane < 3 ? lane : 0;
#pragma unroll
  for (int r = 0; r < kJumpCluster; r++) q[r] = cl.map_shared_rank(part, r)[c];
  double Pc = 0.0;
#pragma unroll
  for (int r = 0; r < kJumpCluster; r++) Pc += q[r];
  const double Px = __shfl_sync(0xffffffffu, Pc, 0), Py = __shfl_sync(0xffffffffu, Pc, 1),
               Pz = __shfl_sync(0xffffffffu, Pc, 2);
  // no block leaves while another may still read its partial: arrive now,
  // wait at the end, after this thread's own work
  auto reads_done = cl.barrier_arrive();
  if (mine) {
    if (CLEAR) D.ce[j] = 0;
    const d3 x = {fma(Px, hdt, x0.x), fma(Py, hdt, x0.y), fma(Pz, hdt, x0.z)};
    store3(D.x, n, j, x);
    D.xf[j] = f32_trunc(x.x);
    D.xf[n + j] = f32_trunc(x.y);
    D.xf[2 * n + j] = f32_trunc(x.z);
    if (vsrc) store3(D.v, n, j, v);
    if (j < nm) write_rc_fast(D.u, rc_out, n, j, x, v, hc_j);
  }
  cl.barrier_wait(std::move(reads_done));
}

// Sets body j's encounter flag (one byte of D.ce, by an atomic OR on its
// aligned 32-bit word; the flag array is allocated in whole words); true for
// the first caller of the step, which appends the body to the list.
__device__ __forceinline__ bool mark_ce(unsigned char* ce, int j) {
  unsigned* w = (unsigned*)(ce + (j & ~3));
  const unsigned bit = 1u << (8 * (j & 3));
  return !(atomicOr(w, bit) & bit);
}

// warp-aggregated append to an encounter list (ballot + prefix count)
__device__ __forceinline__ void append_ce(bool flag, int j, int* list, int* count, unsigned long long* tally) {
  const int lane = threadIdx.x & 31;
  unsigned mask = __ballot_sync(0xffffffffu, flag);
  if (mask) {
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (flag) list[base + __popc(mask & ((1u << lane) - 1u))] = j;
    if (lane == leader) atomicAdd(tally, (unsigned long long)__popc(mask));
  }
}

// Encounter test and element drift of every body, reference order
// (sim.cuh:692-713).  Bodies in encounter are appended to the encounter list;
// every body writes its Kepler result to xo/vo (for encounter bodies it enters
// the blend fma(0, kep, bs) of sim.cuh:718-730, completed by k_encounter).
// ce_big: the flags of big systems' bodies were set, and those bodies listed,
// by k_ce_big_exact (the encounter sub-step of the big systems may then run
// beside this kernel).
__global__ void k_drift_elements(Dev D, const double* __restrict__ rc_in, double dt, int compat_block,
                                 int kep_iters, int ce_big, int trigger) {
  // trigger: the big systems' encounter sub-step that follows runs beside
  // this kernel (it waits for it before its stores)
  if (trigger) griddep_launch();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  bool is_ce = false, listed = false;
  if (j < D.n) {
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    const int self = self_index(j - b0, compat_block);
    SrcView S = src_view(D, rc_in, b0);
    d3 pos = load3(D.x, n, j), vel = load3(D.v, n, j);
    if (ce_big && D.big[s]) {
      is_ce = D.ce[j] != 0;  // flagged and listed by k_ce_big_exact
    } else {
      is_ce = close_encounter(pos, self, S, nm);
      D.ce[j] = is_ce;
      listed = is_ce;
    }
    const double tp = 6.283185307179586476925286766559005768394338798750211641949;
    double a = D.alag[j];
    double nmot = rsqrt_ieee(a * a * a);  // mean motion of the previous elements (sim.cuh:692)
    Elem el = elem_from_cart(pos, vel);
    D.alag[j] = el.a;
    double Mn = (double)(!is_ce) * fmod(fma(nmot, dt, el.M), tp) + (double)(is_ce)*el.M;
    PV kep = cart_from_elem(el.inc, el.node, el.peri, Mn, el.e, el.a, kep_iters);
    store3(D.xo, n, j, kep.pos);
    store3(D.vo, n, j, kep.vel);
  }
  append_ce(listed, j, D.ce_list, &D.ce_count[0], &D.counters[0]);
}

// Encounter sub-step (Richardson extrapolation of modified-midpoint steps
// against sources frozen at the start of the drift, sim.cuh:701-702) in the
// reference order; one thread per listed body, grid-stride.  skip_big leaves
// the bodies of big systems to k_encounter_big_pipe.
__device__ __forceinline__ void encounter_elements_store(const Dev& D, int j, PV bs) {
  const int n = D.n;
  d3 kp = load3(D.xo, n, j), kv = load3(D.vo, n, j);
  bs.pos = {fma(0.0, kp.x, bs.pos.x), fma(0.0, kp.y, bs.pos.y), fma(0.0, kp.z, bs.pos.z)};
  bs.vel = {fma(0.0, kv.x, bs.vel.x), fma(0.0, kv.y, bs.vel.y), fma(0.0, kv.z, bs.vel.z)};
  store3(D.xo, n, j, bs.pos);
  store3(D.vo, n, j, bs.vel);
}
__global__ void k_encounter_elements(Dev D, const double* __restrict__ rc_in, double dt, int compat_block,
                                     int rows, double soft2, int skip_big) {
  const int count = D.ce_count[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int j = D.ce_list[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    if (skip_big && D.big[s]) continue;
    SrcView S = src_view(D, rc_in, b0);
    ExactVelTotal<1> vt{&S, nm, self_index(j - b0, compat_block), soft2};
    PV c = {load3(D.x, n, j), load3(D.v, n, j)};
    encounter_elements_store(D, j, richardson(c, vt, dt, rows));
  }
}
// The big systems' listed bodies: one group of kExactRowThreads threads per
// Richardson row computes the terms of its row's evaluations, and the grid
// has kExactEncBlocksPerSM blocks per SM.  Measured on the 2002-body disk
// (element path, ms per step at ~150 / ~188 encounter bodies): 128 threads,
// one block per SM 1.640 / 1.833 (more encounter bodies than SMs take a
// second round); 64 threads, two blocks per SM 1.509 / 1.513 (three: the
// same); 96 threads, two 1.558 / 1.561; 32 threads, two or four 1.523 /
// 1.525.  The sums are the same chains in the same order: same bits.
constexpr int kExactRowThreads = 64;
constexpr int kExactEncBlocksPerSM = 2;

// The encounter sub-step of the big systems' listed bodies, the rows side by
// side in lock step with one warp for all their fma chains: one block per
// encounter body, warp 0 runs the 3 x rows chains (lane
// 3r + c: row r, component c) while the rows' kExactRowThreads-thread groups
// compute the next kExactRowThreads sources' terms (exact_term with the
// encounter weighting),
// double-buffered in shared memory.  Round k evaluates the velocity update
// of every row whose modified midpoint has more than k sub-steps (row r has
// 2^r), at the row's position of that sub-step; between rounds each group
// advances its row's state exactly as mod_midpoint does.  Each evaluation is
// bound by its chain (one dependent fma per source); a chain step costs the
// FP64 pipe one warp instruction for all rows, and the term groups do not
// wait for it.  Same bits as richardson() with ExactVelTotal (thread 0
// combines the rows as richardson() does).  Launched with
// 32 + kExactRowThreads x rows threads.
__global__ void __launch_bounds__(32 + 4 * kExactRowThreads)
    k_encounter_big_pipe(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, int rows,
                         double soft2, int late_wait) {
  // late_wait: launched beside the element drift (the kernel before it,
  // started after the encounter test completed); the drift writes every
  // body's Kepler result, which encounter_elements_store reads and blends,
  // so each block waits for the drift before its first store and before it
  // leaves (this kernel's completion then implies the drift's)
  constexpr int NT = kExactRowThreads;
  __shared__ double stage[2][4][4][NT];
  __shared__ double accs[4][3];
  __shared__ PV res[4];
  const bool chainw = threadIdx.x < 32;
  const int lane = (int)(threadIdx.x & 31);
  const int g = chainw ? 0 : ((int)threadIdx.x - 32) / NT, tid = chainw ? 0 : ((int)threadIdx.x - 32) % NT;
  const int count = D.ce_count[0];
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const int j = D.ce_list[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    if (!D.big[s]) continue;
    SrcView S = src_view(D, rc_in, b0);
    const int self = self_index(j - b0, compat_block);
    const PV c0 = {load3(D.x, n, j), load3(D.v, n, j)};
    // row g's modified midpoint (mod_midpoint) state, kept by its group
    const int N = 1 << g;
    const double h = dt * inv_pow2(N), h2 = 2.0 * h;
    d3 z0 = c0.pos, z1 = c0.pos;
    z1.x = fma(c0.vel.x, h, z1.x);
    z1.y = fma(c0.vel.y, h, z1.y);
    z1.z = fma(c0.vel.z, h, z1.z);
    PV c = {z1, c0.vel};
    const int nchunks = (nm + NT - 1) / NT;
    const int rounds = 1 << (rows - 1);
    for (int round = 0; round < rounds; round++) {
      const bool active = !chainw && round < N;
      if (active && round > 0) {
        const d3 t = {fma(h2, c.vel.x, z0.x), fma(h2, c.vel.y, z0.y), fma(h2, c.vel.z, z0.z)};
        z0 = z1;
        z1 = t;
        c.pos = z1;
      }
      // rows still running this round: r < rows with 2^r > round
      int nact = 0;
      while (nact < rows && (1 << nact) <= round) nact++;
      const int r_lo = nact, nrun = rows - r_lo;
      double acc = 0.0;  // chain warp, lane 3 q + cc: row r_lo + q
      for (int ch = 0; ch <= nchunks; ch++) {
        if (active && ch < nchunks) {
          const int i = ch * NT + tid;
          d3 d = {0.0, 0.0, 0.0};
          const double wa = i < nm ? exact_term<true>(c.pos, self, S, i, soft2, d) : 0.0;
          double* st = stage[ch & 1][g][0];
          st[tid] = wa;
          st[NT + tid] = d.x;
          st[2 * NT + tid] = d.y;
          st[3 * NT + tid] = d.z;
        }
        if (chainw && ch >= 1 && lane < 3 * nrun) {
          const int q = lane / 3, cc = lane - 3 * q;
          const double* st = stage[(ch - 1) & 1][r_lo + q][0];
          acc = chain_fma<NT>(st, st + NT * (cc + 1), min(NT, nm - (ch - 1) * NT), acc);
        }
        __syncthreads();
      }
      if (chainw && lane < 3 * nrun) accs[r_lo + lane / 3][lane % 3] = acc;
      __syncthreads();
      if (active) {
        // ExactVelTotal: the kick's sum, then the Sun
        d3 nv = {fma(accs[g][0], h, c.vel.x), fma(accs[g][1], h, c.vel.y), fma(accs[g][2], h, c.vel.z)};
        double r_sq = mag2(c.pos);
        const double r = stable_sqrt(r_sq);
        r_sq += soft2;
        const double denom = r_sq * r;
        const d3 rv = {c.pos.x / denom, c.pos.y / denom, c.pos.z / denom};
        nv.x = fma(-rv.x, h, nv.x);
        nv.y = fma(-rv.y, h, nv.y);
        nv.z = fma(-rv.z, h, nv.z);
        c.vel = nv;
        if (round == N - 1 && tid == 0)
          res[g] = PV{{0.5 * (z1.x + fma(c.vel.x, h, z0.x)), 0.5 * (z1.y + fma(c.vel.y, h, z0.y)),
                       0.5 * (z1.z + fma(c.vel.z, h, z0.z))},
                      c.vel};
      }
      __syncthreads();  // accs is rewritten next round
    }
    if (threadIdx.x == 0) {
      if (late_wait) griddep_wait();
      encounter_elements_store(D, j, richardson_of_rows(res, rows));
    }
    __syncthreads();  // res is rewritten for the next body
  }
  if (late_wait && threadIdx.x == 0) griddep_wait();
}

// ---------------------------------------------------------------------------
// fast path (universal drift)
// ---------------------------------------------------------------------------
// Half kick of the bodies of small systems.
__global__ void k_kick_small(Dev D, const double* __restrict__ rc_in, double* __restrict__ rc_out, double hdt,
                             double soft2, int compat_block, double hill, double eject_r2, int last) {
  griddep_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n, s = D.sys[j];
  if (D.big[s]) return;
  const int b0 = D.off[s], nm = D.nm[s], local = j - b0, self = self_index(local, compat_block);
  d3 pos = load3(D.x, n, j);
  d3 acc = {0.0, 0.0, 0.0};
  for (int i = 0; i < nm; i++) pair_fast<false>(D.u, pos, self, i, load_src(D, rc_in, b0 + i), soft2, acc);
  d3 vel = load3(D.v, n, j);
  vel.x = fma(acc.x, hdt, vel.x);
  vel.y = fma(acc.y, hdt, vel.y);
  vel.z = fma(acc.z, hdt, vel.z);
  kick_epilogue(D, j, local, nm, pos, vel, rc_out, hill, eject_r2, last);
}

// stage sources [c, c + cnt) of system starting at b0 into shared memory
__device__ __forceinline__ void stage_sources(const Dev& D, const double* __restrict__ rc, int b0, int c, int cnt,
                                              FastSrc* tile) {
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) tile[k] = load_src(D, rc, b0 + c + k);
}

// Tiled half kick of the big systems: block = work item (kTile targets x a
// chunk of sources).  One chunk: finish the kick; several: write the partial.
__global__ void __launch_bounds__(kTile) k_kick_tiled(Dev D, const Work* __restrict__ work,
                                                      const double* __restrict__ rc_in, double* __restrict__ rc_out,
                                                      double hdt, double soft2, int compat_block, double hill,
                                                      double eject_r2, int last) {
  griddep_enter();
  __shared__ FastSrc tile[kSrcTile];
  const Work W = work[blockIdx.x];
  const int n = D.n, s = W.sys, b0 = D.off[s], b1 = D.off[s + 1], nm = D.nm[s];
  const int j = W.t0 + threadIdx.x;
  const bool active = j < b1;
  const int local = j - b0, self = self_index(local, compat_block);
  d3 pos = active ? load3(D.x, n, j) : d3{0.0, 0.0, 0.0};
  d3 acc = {0.0, 0.0, 0.0};
  for (int c = W.c0; c < W.c1; c += kSrcTile) {
    const int cnt = min(kSrcTile, W.c1 - c);
    __syncthreads();
    stage_sources(D, rc_in, b0, c, cnt, tile);
    __syncthreads();
    if (active)
      for (int k = 0; k < cnt; k++) pair_fast<false>(D.u, pos, self, c + k, tile[k], soft2, acc);
  }
  if (!active) return;
  if (D.nchunk[s] == 1) {
    d3 vel = load3(D.v, n, j);
    vel.x = fma(acc.x, hdt, vel.x);
    vel.y = fma(acc.y, hdt, vel.y);
    vel.z = fma(acc.z, hdt, vel.z);
    kick_epilogue(D, j, local, nm, pos, vel, rc_out, hill, eject_r2, last);
  } else {
    double* p = D.part + (size_t)W.chunk * 3 * n;
    store3(p, n, j, acc);
  }
}

// Test particles of the big systems (one source chunk): the second half kick
// of this step (table B) and the first of the next step (table A) in one pass
// over the sources.  Positions do not move between the two; a pair outside
// both changeover radii computes its term once and adds it to both
// accumulators, in source order, so the result equals two separate kicks bit
// for bit.  Flags are taken after the first of the two kicks.
__global__ void __launch_bounds__(kTile) k_kick_tiled_merged(Dev D, const Work* __restrict__ work,
                                                             const double* __restrict__ rcB,
                                                             const double* __restrict__ rcA, double hdt,
                                                             double soft2, int compat_block, double eject_r2) {
  griddep_enter();
  __shared__ FastSrc tile[kSrcTile];
  __shared__ double tileA[kSrcTile][4];
  const Work W = work[blockIdx.x];
  const int n = D.n, s = W.sys, b0 = D.off[s], b1 = D.off[s + 1], nm = D.nm[s];
  const int j = W.t0 + threadIdx.x;
  const bool active = j < b1;
  const int local = j - b0, self = self_index(local, compat_block);
  d3 pos = active ? load3(D.x, n, j) : d3{0.0, 0.0, 0.0};
  // accA repeats accB's operations until the first pair that is not far in
  // both kicks, so one accumulator serves both until then (same bits)
  d3 accB = {0.0, 0.0, 0.0}, accA = {0.0, 0.0, 0.0};
  bool split = false;
  for (int c = W.c0; c < W.c1; c += kSrcTile) {
    const int cnt = min(kSrcTile, W.c1 - c);
    __syncthreads();
    stage_sources(D, rcB, b0, c, cnt, tile);
    for (int k = threadIdx.x; k < cnt; k += blockDim.x)
      for (int q = 0; q < 4; q++) tileA[k][q] = rcA[4 * (size_t)(b0 + c + k) + q];
    __syncthreads();
    if (active) {
      for (int k = 0; k < cnt; k++) {
        const FastSrc& SB = tile[k];
        const int i = c + k;
        double dx = fsub(D.u, SB.x, pos.x), dy = fsub(D.u, SB.y, pos.y), dz = fsub(D.u, SB.z, pos.z);
        double r2 = fma(dx, dx, fma(dy, dy, fmul(D.u, dz, dz)));
        if (hi_word(r2) > max(SB.rc2_hi, thr_unpack(tileA[k][3])) && i != self && seed_in_range(r2)) {
          double w = fmul(D.u, SB.m, inv_softened_r3(D.u, r2, fadd(D.u, r2, soft2)));
          accB.x = fma(w, dx, accB.x);
          accB.y = fma(w, dy, accB.y);
          accB.z = fma(w, dz, accB.z);
          if (split) {
            accA.x = fma(w, dx, accA.x);
            accA.y = fma(w, dy, accA.y);
            accA.z = fma(w, dz, accA.z);
          }
        } else {
          if (!split) {
            accA = accB;
            split = true;
          }
          pair_fast<false>(D.u, pos, self, i, SB, soft2, accB);
          FastSrc SA = SB;
          SA.rc = tileA[k][0];
          SA.rc01 = tileA[k][1];
          SA.rc09 = tileA[k][2];
          SA.rc2_hi = thr_unpack(tileA[k][3]);
          pair_fast<false>(D.u, pos, self, i, SA, soft2, accA);
        }
      }
    }
  }
  if (!active) return;
  if (!split) accA = accB;
  d3 vel = load3(D.v, n, j);
  vel.x = fma(accB.x, hdt, vel.x);
  vel.y = fma(accB.y, hdt, vel.y);
  vel.z = fma(accB.z, hdt, vel.z);
  kick_epilogue(D, j, local, nm, pos, vel, nullptr, 0.0, eject_r2, 1);
  vel.x = fma(accA.x, hdt, vel.x);
  vel.y = fma(accA.y, hdt, vel.y);
  vel.z = fma(accA.z, hdt, vel.z);
  store3(D.v, n, j, vel);
}

// Sum of the chunk partials in chunk order, then the kick of big-system bodies
// with more than one chunk.
__global__ void k_kick_reduce(Dev D, double* __restrict__ rc_out, double hdt, double hill, double eject_r2,
                              int last) {
  griddep_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n, s = D.sys[j], C = D.nchunk[s];
  if (!D.big[s] || C <= 1) return;
  d3 acc = {0.0, 0.0, 0.0};
  for (int c = 0; c < C; c++) {
    const double* p = D.part + (size_t)c * 3 * n;
    acc.x += p[j];
    acc.y += p[n + j];
    acc.z += p[2 * n + j];
  }
  d3 pos = load3(D.x, n, j), vel = load3(D.v, n, j);
  vel.x = fma(acc.x, hdt, vel.x);
  vel.y = fma(acc.y, hdt, vel.y);
  vel.z = fma(acc.z, hdt, vel.z);
  kick_epilogue(D, j, j - D.off[s], D.nm[s], pos, vel, rc_out, hill, eject_r2, last);
}

// ---- symmetric massive-massive interactions of the big systems ----
// The massive bodies of a big system are cut into blocks of 32.  A warp takes
// one unordered block pair (I, J), I <= J: lane t keeps target i = 32 I + t and
// a rotating source j = 32 J + ((t + k) mod 32) that moves one lane per
// iteration together with its reverse accumulator, so after 32 iterations
// every lane has met every source and the reverse sums are back home.  Both
// directions of a pair share d, r^2 and u = 1 / ((r^2 + eps^2) r): 22 FP64
// operations per unordered pair instead of 2 x 18.  The diagonal block runs
// k = 1..16 (k = 16 on lanes 0..15 only).
//
// The kick pass sums the far field only: a pair is far when r exceeds both
// sources' far-field radii (far_threshold; K = 1 in both directions) and the
// FP32 seed range allows the fast formula.  Every other pair sets one bit per
// direction in the near-pair masks, and k_kick_reduce_sym adds those pairs
// with the reference formula.  The far field depends on the positions and the
// far-field thresholds only, so a kick whose thresholds equal those of the
// kick before it (the two kicks around a step boundary) reuses its sums.
struct SymTask {
  int sys, I, J;
};

// Task t of a single system of NB 32-body blocks, in the host list's order:
// the off-diagonal pairs I < J row by row, then the diagonal ones (I, I).
// Row I starts at I (2 NB - I - 1) / 2; the FP32 root estimates the row and
// integer steps correct it.  Decoded instead of loaded, so the block's first
// loads are its bodies' (one memory round trip before the pair work rather
// than three: task, system offsets, bodies).
__device__ __forceinline__ SymTask sym_decode(int t, int NB) {
  const long long nb = NB, np = nb * (nb - 1) / 2;
  if (t >= np) return SymTask{0, (int)(t - np), (int)(t - np)};
  const float b = 2.0f * (float)NB - 1.0f;
  long long r = (long long)((b - sqrtf(fmaxf(b * b - 8.0f * (float)t, 0.0f))) * 0.5f);
  r = r < 0 ? 0 : (r > nb - 2 ? nb - 2 : r);
  while (r > 0 && r * (2 * nb - r - 1) / 2 > t) r--;
  while ((r + 1) * (2 * nb - r - 2) / 2 <= t) r++;
  return SymTask{0, (int)r, (int)(t - r * (2 * nb - r - 1) / 2 + r + 1)};
}

struct RotSrc {
  double x, y, z, m;
  int thr, idx;
  F4 f;       // FP32 position copy (encounter prefilter)
  float rcf;  // r_crit in FP32 (encounter prefilter)
};

// KICK rotates the FP64 source and the reverse accumulators; the encounter
// test rotates the FP32 copies only (the rare pairs that pass its prefilter
// read the FP64 position and r_crit of the source from memory)
template <bool KICK>
__device__ __forceinline__ void rotate(RotSrc& r, d3& acc, uint32_t& bits) {
  const int src = (threadIdx.x + 1) & 31;
  r.idx = __shfl_sync(0xffffffffu, r.idx, src);
  if (!KICK) {
    r.f.x = __shfl_sync(0xffffffffu, r.f.x, src);
    r.f.y = __shfl_sync(0xffffffffu, r.f.y, src);
    r.f.z = __shfl_sync(0xffffffffu, r.f.z, src);
    r.f.sc = __shfl_sync(0xffffffffu, r.f.sc, src);
    r.rcf = __shfl_sync(0xffffffffu, r.rcf, src);
  } else {
    r.x = __shfl_sync(0xffffffffu, r.x, src);
    r.y = __shfl_sync(0xffffffffu, r.y, src);
    r.z = __shfl_sync(0xffffffffu, r.z, src);
    r.m = __shfl_sync(0xffffffffu, r.m, src);
    r.thr = __shfl_sync(0xffffffffu, r.thr, src);
    acc.x = __shfl_sync(0xffffffffu, acc.x, src);
    acc.y = __shfl_sync(0xffffffffu, acc.y, src);
    acc.z = __shfl_sync(0xffffffffu, acc.z, src);
  }
  bits = __shfl_sync(0xffffffffu, bits, src);
}

// KICK: far-field sums and near-pair masks into partial set `set` (thresholds
// from rc's far-field table); with `gate`, only when *gate is set (and for a
// single system only the block pairs that D.gate_blocks marks).
// !KICK: encounter test flags (rc's fast thresholds; the flags must be clear
// before the launch), the flagged bodies appended to the big-system list
// (set 0) or to the element path's list (set 1).
// Each block-pair task runs on kSymSplit warps of one block, each taking a
// contiguous share of the rotations; the far-field pass (KICK) adds their
// sums in warp order through shared memory (a fixed order), the encounter
// test ORs their flags.  The FP64
// unit is per SM sub-partition, and with one warp per task the 2016 tasks of
// a 2002-body system put three or four warps on a sub-partition (warp end
// times 66-84 us within one pass); split in two, a sub-partition holds six or
// seven half tasks.  Measured: about 1 us less per pass (0.2540 -> 0.2530 ms
// per step), far less than the load difference suggests: the end times were
// spread evenly rather than in two groups.
constexpr int kSymSplit = 2;
// Tasks per block of the gated second far-field pass.  It is usually empty
// (its blocks read the clear gate and leave): 2016 one-task blocks took
// 3.2 us to do that.  On the 2002-body disk, where it never runs, half and a
// quarter of the blocks (two or four tasks each) saved 0.6 and 1.1 us per
// step; with 300 embryos at e = 0.6, where it runs at almost every step,
// they cost 2.6 and 12.4 us per step (0.3023 -> 0.3049 and 0.3147 ms).  Two
// tasks per block: the smaller loss where the pass runs.  (The encounter test
// keeps one task per block and two warps per task: two tasks per block
// measured +3 us per step, four and eight warps per task +0.9 and +2.9 us.)
constexpr int kSymGatedDiv = 2;
// One block-pair task on the kSymSplit warps of a block (k_sym); ONE: a
// single system (tasks decoded from the index, no table or system lookups).
template <bool KICK, bool ONE>
__device__ __forceinline__ void sym_task(const Dev& D, const SymTask* __restrict__ tasks, int warp,
                                         const double* __restrict__ rc, double soft2, int set) {
  constexpr int SPLIT = kSymSplit;
  // warp `part` of SPLIT takes its share of the task's rotations
  const int part = (int)(threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const SymTask T = ONE ? sym_decode(warp, (D.nm0 + 31) / 32) : tasks[warp];
  const int s = T.sys, b0 = ONE ? 0 : D.off[s], nm = ONE ? D.nm0 : D.nm[s];
  const int* far_thr = rc_far_thr_c(rc, D.n);
  const int i = 32 * T.I + lane;
  const bool iv = i < nm;
  RotSrc A, B;
  A.x = iv ? D.x[b0 + i] : 0.0;
  A.y = iv ? D.x[D.n + b0 + i] : 0.0;
  A.z = iv ? D.x[2 * D.n + b0 + i] : 0.0;
  A.m = (KICK && iv) ? D.m[b0 + i] : 0.0;
  A.thr = iv ? (KICK ? far_thr[b0 + i] : thr_unpack(rc[4 * (size_t)(b0 + i) + 3])) : 0x7fffffff;
  A.idx = i;
  A.f = (!KICK && iv) ? load_f4(D, b0 + i) : F4{0.f, 0.f, 0.f, 0.f};
  A.rcf = (!KICK && iv) ? f32_trunc(rc[4 * (size_t)(b0 + i)]) : 0.f;
  // rotation steps of the task (step k pairs lane t with source lane t + k of
  // block J; the diagonal task takes k = 1..16, lanes 0-15 only at k = 16),
  // and this warp's share of them
  const bool diag = T.I == T.J;
  const int kbeg = diag ? 1 : 0, kend = diag ? 16 : 31;
  const int span_k = kend - kbeg + 1;
  const int k0 = kbeg + (part * span_k) / SPLIT, k1 = kbeg + ((part + 1) * span_k) / SPLIT - 1;
  // the source rotated to step k0 from the start: lane t holds source t + k0
  const int jb = 32 * T.J + ((lane + k0) & 31);
  const int j0 = 32 * T.J + lane;
  const bool jv0 = j0 < nm, jvb = jb < nm;
  B.x = (KICK && jvb) ? D.x[b0 + jb] : 0.0;
  B.y = (KICK && jvb) ? D.x[D.n + b0 + jb] : 0.0;
  B.z = (KICK && jvb) ? D.x[2 * D.n + b0 + jb] : 0.0;
  B.m = (KICK && jvb) ? D.m[b0 + jb] : 0.0;
  B.thr = (KICK && jvb) ? far_thr[b0 + jb] : 0x7fffffff;
  B.idx = jvb ? jb : -1;
  B.f = (!KICK && jvb) ? load_f4(D, b0 + jb) : F4{0.f, 0.f, 0.f, 0.f};
  B.rcf = (!KICK && jvb) ? f32_trunc(rc[4 * (size_t)(b0 + jb)]) : 0.f;
  d3 accA = {0.0, 0.0, 0.0}, accB = {0.0, 0.0, 0.0};
  // KICK: near-pair bits (bit q: source 32 J + q for A, 32 I + q for B);
  // !KICK: encounter flags
  uint32_t bitsA = 0u, bitsB = 0u;
  int rotations = k0;
  for (int k = k0; k <= k1; k++) {
    const bool act = iv && B.idx >= 0 && !(diag && k == 16 && lane >= 16);
    if (act) {
      if (!KICK) {
        // encounter of i with source j uses r_crit(j), of j with i uses r_crit(i);
        // the FP32 prefilter clears far pairs without FP64 work
        bool mA, mB;
        ce_maybe2(A.f, B.f, B.rcf, A.rcf, mA, mB);
        if (mA || mB) {
          const int g = b0 + B.idx;
          const double dx = D.x[g] - A.x, dy = D.x[D.n + g] - A.y, dz = D.x[2 * D.n + g] - A.z;
          const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
          const int h = __double2hiint(r2);
          if (mA && h <= thr_unpack(rc[4 * (size_t)g + 3]) && sqrt(r2) < rc[4 * (size_t)g]) bitsA = 1u;
          if (mB && h <= A.thr && sqrt(r2) < rc[4 * (size_t)(b0 + A.idx)]) bitsB = 1u;
        }
      } else {
        const FU& U = D.u;
        const double dx = fsub(U, B.x, A.x), dy = fsub(U, B.y, A.y), dz = fsub(U, B.z, A.z);
        const double r2 = fma(dx, dx, fma(dy, dy, fmul(U, dz, dz)));
        const int h = __double2hiint(r2);
        if (h > max(A.thr, B.thr) && seed_in_range(r2)) {
          const double u = inv_softened_r3(U, r2, fadd(U, r2, soft2));
          const double wa = fmul(U, B.m, u), wb = fmul(U, A.m, u);
          accA.x = fma(wa, dx, accA.x);
          accA.y = fma(wa, dy, accA.y);
          accA.z = fma(wa, dz, accA.z);
          accB.x = fma(-wb, dx, accB.x);
          accB.y = fma(-wb, dy, accB.y);
          accB.z = fma(-wb, dz, accB.z);
        } else {
          bitsA |= 1u << (B.idx & 31);
          bitsB |= 1u << lane;
        }
      }
    }
    rotate<KICK>(B, accB, bitsB);
    rotations++;
  }
  // bring the reverse accumulators home: lane t takes from lane t + 32 - R
  {
    const int src = (lane + 32 - (rotations & 31)) & 31;
    if (KICK) {
      accB.x = __shfl_sync(0xffffffffu, accB.x, src);
      accB.y = __shfl_sync(0xffffffffu, accB.y, src);
      accB.z = __shfl_sync(0xffffffffu, accB.z, src);
    }
    bitsB = __shfl_sync(0xffffffffu, bitsB, src);
  }
  if (SPLIT > 1) {
    // the warps' shares added in warp order (KICK) and their flags or
    // near-pair bits OR-ed, by warp 0
    __shared__ double xs[KICK ? kSymSplit - 1 : 1][KICK ? 6 : 1][32];
    __shared__ uint32_t xb[kSymSplit - 1][2][32];
    if (part > 0) {
      if (KICK) {
        double* p = &xs[part - 1][0][0];
        p[lane] = accA.x;
        p[32 + lane] = accA.y;
        p[64 + lane] = accA.z;
        p[96 + lane] = accB.x;
        p[128 + lane] = accB.y;
        p[160 + lane] = accB.z;
      }
      xb[part - 1][0][lane] = bitsA;
      xb[part - 1][1][lane] = bitsB;
    }
    __syncthreads();
    if (part > 0) return;
    for (int w = 0; w < SPLIT - 1; w++) {
      if (KICK) {
        const double* p = &xs[w][0][0];
        accA.x += p[lane];
        accA.y += p[32 + lane];
        accA.z += p[64 + lane];
        accB.x += p[96 + lane];
        accB.y += p[128 + lane];
        accB.z += p[160 + lane];
      }
      bitsA |= xb[w][0][lane];
      bitsB |= xb[w][1][lane];
    }
  }
  if (KICK) {
    const size_t stride = 3 * (size_t)nm;
    const long long sbase = ONE ? 0 : D.sym_base[s];
    double* base = D.part_sym + (size_t)set * D.sym_set + sbase;
    uint32_t* mask = D.near_mask + (size_t)set * (D.sym_set / 3) + sbase / 3;
    if (diag) {
      if (iv) {
        double* p = base + (size_t)T.I * stride;
        p[i] = accA.x + accB.x;
        p[nm + i] = accA.y + accB.y;
        p[2 * nm + i] = accA.z + accB.z;
        mask[(size_t)T.I * nm + i] = bitsA | bitsB;
      }
    } else {
      if (iv) {
        double* p = base + (size_t)T.J * stride;  // block I's slot for source block J
        p[i] = accA.x;
        p[nm + i] = accA.y;
        p[2 * nm + i] = accA.z;
        mask[(size_t)T.J * nm + i] = bitsA;
      }
      if (jv0) {
        double* p = base + (size_t)T.I * stride;  // block J's slot for source block I
        p[j0] = accB.x;
        p[nm + j0] = accB.y;
        p[2 * nm + j0] = accB.z;
        mask[(size_t)T.I * nm + j0] = bitsB;
      }
    }
  } else {
    // flags and the big-system encounter list (each body once)
    const bool fa = iv && bitsA && mark_ce(D.ce, b0 + i);
    const bool fb = jv0 && bitsB && mark_ce(D.ce, b0 + j0);
    // set 1: the element path's list (k_drift_elements lists the small
    // systems' encounter bodies beside these)
    int* list = set ? D.ce_list : D.ce_list_big;
    int* cnt = set ? &D.ce_count[0] : &D.ce_count[1];
    append_ce(fa, b0 + i, list, cnt, &D.counters[0]);
    append_ce(fb, b0 + j0, list, cnt, &D.counters[0]);
  }
}
// Tasks blockIdx.x, blockIdx.x + gridDim.x, ... (whole blocks leave
// together; a barrier between tasks keeps the next task's shared-memory
// exchange after this one's reads).
template <bool KICK, bool ONE>
__global__ void __launch_bounds__(32 * kSymSplit)
    k_sym(Dev D, const SymTask* __restrict__ tasks, int ntasks, const double* __restrict__ rc, double soft2,
          int set, const int* __restrict__ gate) {
  griddep_enter();
  if (KICK && gate && *gate == 0) return;
  if (KICK && gate && blockIdx.x == 0 && (threadIdx.x & 31) == 0) atomicAdd(D.far_recomputes, 1ull);
  for (int t = (int)blockIdx.x; t < ntasks; t += (int)gridDim.x) {
    // the gated pass of a single system: only the block pairs with a block
    // whose far-field threshold moved (the others are the same in both sets)
    if (KICK && ONE && gate) {
      const SymTask T = sym_decode(t, (D.nm0 + 31) / 32);
      const unsigned long long* gb = D.gate_blocks;
      if (!(((gb[T.I >> 6] >> (T.I & 63)) | (gb[T.J >> 6] >> (T.J & 63))) & 1ull)) continue;
    }
    sym_task<KICK, ONE>(D, tasks, t, rc, soft2, set);
    __syncthreads();
  }
}

constexpr int kRedThreads = 16;  // threads per body of k_kick_reduce_sym
constexpr int kRedBodies = kThreads / kRedThreads;  // bodies per block
constexpr int kRedBatch = 4;     // partials loaded per thread before they are added
constexpr int kNearList = 32;    // near pairs per body dealt out over its threads
static_assert(kRedBodies <= 32 && kThreads % 32 == 0, "one lane per body in the epilogue warp");

// Totals of six values over the 16 threads of a body (lanes 16h .. 16h + 15
// of a warp) by a reduce-scatter: at each level half of the values go to the
// partner lane, so 4 + 2 + 1 + 1 FP64 additions instead of 6 x 4 for
// butterflies (the FP64 unit of a sub-partition takes a warp instruction at
// the same cost however few of its lanes need the result).  Thread sub ends
// with the total of value 4 bit3 + 2 bit2 + bit1 of sub (6 and 7 are empty);
// a fixed tree, so the result does not depend on scheduling.
__device__ __forceinline__ double red_scatter6(const double (&v)[6], int sub) {
  const unsigned full = 0xffffffffu;
  const bool h8 = (sub & 8) != 0, h4 = (sub & 4) != 0, h2 = (sub & 2) != 0;
  double k[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const double lo = v[i], hi = i < 2 ? v[4 + i] : 0.0;
    k[i] = (h8 ? hi : lo) + __shfl_xor_sync(full, h8 ? lo : hi, 8);
  }
  double m[2];
#pragma unroll
  for (int i = 0; i < 2; i++) m[i] = (h4 ? k[2 + i] : k[i]) + __shfl_xor_sync(full, h4 ? k[i] : k[2 + i], 4);
  double r = (h2 ? m[1] : m[0]) + __shfl_xor_sync(full, h2 ? m[0] : m[1], 2);
  return r + __shfl_xor_sync(full, r, 1);
}

// Kick of every body of a big system whose sums are in partials: massive
// bodies add their far-field block partials (symmetric kernel, set 1 when
// *gate is set, else set 0) and then their near pairs (reference formula,
// rc = the kick's r_crit table); test particles add their chunk partials (when
// there is more than one chunk; a single chunk was applied by the tiled
// kernel).  kRedThreads threads per body each take every kRedThreads-th
// block; their sums are combined by red_scatter6, so the result does not
// depend on scheduling.  The epilogue (velocity, r_crit, flags) of the block's
// kRedBodies bodies runs on one warp, one body per lane, with the totals
// handed over in shared memory: on the body's own lead thread it took each
// warp the FP64 instructions of two bodies' epilogues on two lanes.  check:
// after writing rc_out, set *D.gate if a massive body's far-field threshold in
// rc_out differs from the one in rc (the far field of the next kick must then
// be recomputed).
template <bool ONE>
__global__ void k_kick_reduce_sym(Dev D, const double* __restrict__ rc, const int* __restrict__ gate,
                                  double* __restrict__ rc_out, double hdt, double soft2, double hill,
                                  double eject_r2, int last, int massive_only, int check, int far_mode) {
  griddep_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = t / kRedThreads, sub = t % kRedThreads;
  const int n = D.n;
  // which bodies have a kick here: massive bodies of big systems, and test
  // particles of big systems with more than one chunk partial
  struct Body {
    int s, b0, nm, local;
    bool work, massive;
  };
  auto classify = [&](int jj) {
    Body B;
    const bool valid = jj < n;
    // ONE: a single system, big (no per-body system lookups)
    B.s = ONE ? 0 : (valid ? D.sys[jj] : 0);
    B.work = valid && (ONE || D.big[B.s]);
    B.b0 = (ONE || !B.work) ? 0 : D.off[B.s];
    B.nm = B.work ? (ONE ? D.nm0 : D.nm[B.s]) : 0;
    B.local = jj - B.b0;
    B.massive = B.work && B.local < B.nm;
    if (B.work && !B.massive && !(D.nchunk[B.s] > 1 && !massive_only)) B.work = false;
    return B;
  };
  // far_mode 1: keep the far-field sum of each massive body in D.far_acc;
  // 2: take it from there when the gate is clear (the far field of the
  // second kick of a merged pair is then the first's, the same partials in
  // the same order)
  const int set = (gate && *gate) ? 1 : 0;
  const bool reuse_set = far_mode == 2 && set == 0;
  // the epilogue warp (spread over the sub-partitions by the block index) and
  // its lanes' bodies; their inputs are loaded before the sums, which they do
  // not depend on
  const int lane = (int)(threadIdx.x & 31);
  const bool epi = (int)(threadIdx.x >> 5) == (int)(blockIdx.x & (kThreads / 32 - 1)) && lane < kRedBodies;
  const int je = (int)blockIdx.x * kRedBodies + lane;
  Body E = {0, 0, 0, 0, false, false};
  d3 pos_e = {0.0, 0.0, 0.0}, vel_e = {0.0, 0.0, 0.0}, far_e = {0.0, 0.0, 0.0};
  double hc_e = 0.0;
  uint32_t flags_e = 0u;
  bool ce_e = false;
  int thr_e = 0;
  if (epi) {
    E = classify(je);
    if (E.work) {
      pos_e = load3(D.x, n, je);
      vel_e = load3(D.v, n, je);
      if (E.massive && far_mode == 2) far_e = load3(D.far_acc, n, je);  // used when the gate is clear
      if (rc_out && E.massive) hc_e = D.hc[je];
      if (last) {
        flags_e = D.flags[je];
        ce_e = D.ce[je] != 0;
      }
      if (check && E.massive) thr_e = rc_far_thr_c(rc, n)[je];
    }
  }
  const Body B = classify(j);
  const bool work = B.work, massive = B.massive;
  const int s = B.s, b0 = B.b0, nm = B.nm, local = B.local;
  int count = 0;
  const double* base = nullptr;
  const uint32_t* mask = nullptr;
  size_t stride = 0;
  int index = 0;
  const bool reuse = massive && reuse_set;
  // (a single system's partials start at 0)
  const long long sbase = ONE ? 0 : (massive ? D.sym_base[s] : 0);
  // A single system whose gate is set: the gated pass recomputed only the
  // block pairs with a block whose far-field threshold moved (into set 1);
  // the others are the same in both sets (same positions, same thresholds),
  // so each pair's partial and near-pair word come from the set it was last
  // computed in: the bits of a full recompute.
  const bool pick = ONE && massive && set == 1;
  const int blk = local >> 5;
  const bool blk_moved = pick && ((D.gate_blocks[blk >> 6] >> (blk & 63)) & 1ull);
  // set 1 -> set 0 for pair (blk, b) when neither block moved
  auto back = [&](int b) { return pick && !blk_moved && !((D.gate_blocks[b >> 6] >> (b & 63)) & 1ull); };
  const uint32_t* mask0 = nullptr;
  if (massive) {
    count = (nm + 31) / 32;
    mask0 = D.near_mask + sbase / 3;
    base = D.part_sym + sbase + (size_t)set * D.sym_set;
    mask = mask0 + (size_t)set * (D.sym_set / 3);
    stride = 3 * (size_t)nm;
    index = local;
  } else if (work) {
    count = D.nchunk[s];
    base = D.part;
    stride = 3 * (size_t)n;
    index = j;
  }
  const size_t span = stride / 3;
  d3 acc = {0.0, 0.0, 0.0};
  d3 pos = {0.0, 0.0, 0.0};
  if (work) pos = load3(D.x, n, j);
  // kRedBatch partials' loads in flight before they are added (same order of
  // additions as one at a time); the near-pair mask words with them
  uint32_t words[kRedBatch];
#pragma unroll
  for (int u = 0; u < kRedBatch; u++) words[u] = 0u;
  // the second kick of a merged pair: the near-pair words of partial set 0,
  // loaded beside the gate rather than after it (a set gate, which is rare,
  // reloads them from set 1 with the partials below)
  if (massive && far_mode == 2) {
#pragma unroll
    for (int u = 0; u < kRedBatch; u++) {
      const int b = sub + u * kRedThreads;
      words[u] = b < count ? mask0[(size_t)b * nm + local] : 0u;
    }
  }
  for (int b0r = sub, r = 0; !reuse && b0r < count; b0r += kRedBatch * kRedThreads, r++) {
    double px[kRedBatch], py[kRedBatch], pz[kRedBatch];
#pragma unroll
    for (int u = 0; u < kRedBatch; u++) {
      const int b = b0r + u * kRedThreads;
      const bool ok = b < count;
      const bool bk = ok && back(b);
      const double* p = base + (size_t)b * stride - (bk ? D.sym_set : 0);
      px[u] = ok ? p[index] : 0.0;
      py[u] = ok ? p[span + index] : 0.0;
      pz[u] = ok ? p[2 * span + index] : 0.0;
      if (r == 0) words[u] = (ok && massive) ? (mask - (bk ? D.sym_set / 3 : 0))[(size_t)b * nm + local] : 0u;
    }
#pragma unroll
    for (int u = 0; u < kRedBatch; u++) {
      if (b0r + u * kRedThreads < count) {
        acc.x += px[u];
        acc.y += py[u];
        acc.z += pz[u];
      }
    }
  }
  // Near pairs (reference formula, a chain of ~45 dependent FP64 operations
  // each): a body's set mask bits usually sit in one or two words, i.e. with
  // one or two of its threads.  They are listed in shared memory in (thread,
  // word, bit) order and the list is dealt out over the body's threads, so
  // the chain is about one pair long; thread sub adds entries sub,
  // sub + kRedThreads, ... in order (a fixed order, whatever the schedule).  A
  // body with more than kNearList near pairs keeps them with their threads.
  __shared__ int near_list[kThreads / kRedThreads][kNearList];
  int own = 0;
#pragma unroll
  for (int u = 0; u < kRedBatch; u++) own += __popc(words[u]);
  // near-pair word of source block b from the set its pair was last computed in
  auto mword = [&](int b) { return (mask - (back(b) ? D.sym_set / 3 : 0))[(size_t)b * nm + local]; };
  for (int b = sub + kRedBatch * kRedThreads; massive && b < count; b += kRedThreads)
    own += __popc(mword(b));
  int incl = own;
  for (int o = 1; o < kRedThreads; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o, kRedThreads);
    if (sub >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, kRedThreads - 1, kRedThreads);
  const bool dealt = total <= kNearList;
  int* list = near_list[threadIdx.x / kRedThreads];
  if (dealt && massive) {
    int at = incl - own;
#pragma unroll
    for (int u = 0; u < kRedBatch; u++)
      for (uint32_t w = words[u]; w; w &= w - 1u) list[at++] = 32 * (sub + u * kRedThreads) + __ffs(w) - 1;
    for (int b = sub + kRedBatch * kRedThreads; b < count; b += kRedThreads)
      for (uint32_t w = mword(b); w; w &= w - 1u) list[at++] = 32 * b + __ffs(w) - 1;
  }
  __syncwarp();
  d3 near = {0.0, 0.0, 0.0};
  if (massive && dealt) {
    for (int q = sub; q < total; q += kRedThreads) {
      const int src = list[q];
      pair_exact<false>(pos, local, src, load_src(D, rc, b0 + src), soft2, near);
    }
  } else if (massive) {
#pragma unroll
    for (int u = 0; u < kRedBatch; u++) {
      const int b = sub + u * kRedThreads;
      for (uint32_t w = words[u]; w; w &= w - 1u) {
        const int src = 32 * b + __ffs(w) - 1;
        pair_exact<false>(pos, local, src, load_src(D, rc, b0 + src), soft2, near);
      }
    }
    for (int b = sub + kRedBatch * kRedThreads; b < count; b += kRedThreads) {
      for (uint32_t w = mword(b); w; w &= w - 1u) {
        const int src = 32 * b + __ffs(w) - 1;
        pair_exact<false>(pos, local, src, load_src(D, rc, b0 + src), soft2, near);
      }
    }
  }
  // the body's totals (far field x, y, z, near pairs x, y, z) to shared
  // memory, one value per even thread of the body
  __shared__ double tot[kRedBodies][6];
  {
    const double v6[6] = {acc.x, acc.y, acc.z, near.x, near.y, near.z};
    const double tv = red_scatter6(v6, sub);
    const int vi = 4 * ((sub >> 3) & 1) + 2 * ((sub >> 2) & 1) + ((sub >> 1) & 1);
    if ((sub & 1) == 0 && vi < 6) tot[threadIdx.x / kRedThreads][vi] = tv;
  }
  __syncthreads();
  if (!epi || !E.work) return;
  // kick_epilogue with the prefetched inputs, one body per lane
  d3 a = {tot[lane][0], tot[lane][1], tot[lane][2]};
  if (E.massive) {
    if (reuse_set)
      a = far_e;
    else if (far_mode == 1)
      store3(D.far_acc, n, je, a);
    a.x += tot[lane][3];
    a.y += tot[lane][4];
    a.z += tot[lane][5];
  }
  d3 vel = vel_e;
  vel.x = fma(a.x, hdt, vel.x);
  vel.y = fma(a.y, hdt, vel.y);
  vel.z = fma(a.z, hdt, vel.z);
  store3(D.v, n, je, vel);
  if (rc_out && E.massive) {
    const int far = write_rc_fast(D.u, rc_out, n, je, pos_e, vel, hc_e);
    if (check && far != thr_e) {
      atomicOr(D.gate, 1);
      if (ONE) atomicOr(D.gate_blocks + (E.local >> 11), 1ull << ((E.local >> 5) & 63));
    }
  }
  if (last) {
    uint32_t f = flags_e & ~MERC_FLAG_CE_LAST;
    if (ce_e) f |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
    if (eject_r2 > 0.0 && mag2(pos_e) > eject_r2) f |= MERC_FLAG_EJECTED;
    bool fin = mm::isfinite_(pos_e.x) && mm::isfinite_(pos_e.y) && mm::isfinite_(pos_e.z) &&
               mm::isfinite_(vel.x) && mm::isfinite_(vel.y) && mm::isfinite_(vel.z);
    if (!fin) f |= MERC_FLAG_NONFINITE;
    D.flags[je] = f;
  }
}

// Tiled encounter test of the big systems: any source of the chunk within
// r_crit sets ce[j] (the flags were cleared before the launch) and appends j
// to the big-system encounter list once.
__global__ void __launch_bounds__(kTile) k_ce_tiled(Dev D, const Work* __restrict__ work,
                                                    const double* __restrict__ rc_in, int compat_block) {
  griddep_enter();
  __shared__ FastSrc tile[kSrcTile];
  __shared__ F4 tilef[kSrcTile];
  __shared__ float tilerc[kSrcTile];  // the sources' r_crit as FP32 (f32_trunc), once per source
  const Work W = work[blockIdx.x];
  const int n = D.n, s = W.sys, b0 = D.off[s], b1 = D.off[s + 1];
  const int j = W.t0 + threadIdx.x;
  const bool active = j < b1;
  const int self = self_index(j - b0, compat_block);
  d3 pos = active ? load3(D.x, n, j) : d3{0.0, 0.0, 0.0};
  F4 pf = active ? load_f4(D, j) : F4{0.f, 0.f, 0.f, 0.f};
  bool ce = false;
  for (int c = W.c0; c < W.c1; c += kSrcTile) {
    const int cnt = min(kSrcTile, W.c1 - c);
    __syncthreads();
    stage_sources(D, rc_in, b0, c, cnt, tile);
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
      tilef[k] = load_f4(D, b0 + c + k);
      tilerc[k] = f32_trunc(rc_in[4 * (size_t)(b0 + c + k)]);
    }
    __syncthreads();
    if (active) {
      // the FP32 prefilter of four sources at a time without branches; the
      // exact test (pair_ce, FP64) only where one of them says "maybe" (the
      // flag is the OR of pair_ce_f over the sources, in any order)
      int k = 0;
      for (; k + 4 <= cnt; k += 4) {
        const bool m0 = ce_maybe(pf, tilef[k], tilerc[k]), m1 = ce_maybe(pf, tilef[k + 1], tilerc[k + 1]),
                   m2 = ce_maybe(pf, tilef[k + 2], tilerc[k + 2]), m3 = ce_maybe(pf, tilef[k + 3], tilerc[k + 3]);
        if ((m0 | m1 | m2 | m3) && !ce) {
          if (m0) ce = pair_ce(pos, self, c + k, tile[k]);
          if (m1 && !ce) ce = pair_ce(pos, self, c + k + 1, tile[k + 1]);
          if (m2 && !ce) ce = pair_ce(pos, self, c + k + 2, tile[k + 2]);
          if (m3 && !ce) ce = pair_ce(pos, self, c + k + 3, tile[k + 3]);
        }
      }
      for (; k < cnt; k++)
        if (!ce && ce_maybe(pf, tilef[k], tilerc[k])) ce = pair_ce(pos, self, c + k, tile[k]);
    }
  }
  const bool first = active && ce && mark_ce(D.ce, j);
  append_ce(first, j, D.ce_list_big, &D.ce_count[1], &D.counters[0]);
}

// Momentum of each big system: block per system, strided partial sums and a
// fixed-order tree (deterministic).
constexpr int kMomThreads = 512;
__global__ void __launch_bounds__(kMomThreads) k_momentum_big(Dev D, const int* __restrict__ big_ids,
                                                              const double* __restrict__ vsrc) {
  const int s = big_ids[blockIdx.x];
  const int b0 = D.off[s], nm = D.nm[s], n = D.n;
  __shared__ double red[3][kMomThreads];
  double px = 0.0, py = 0.0, pz = 0.0;
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    double mi = D.m[b0 + i];
    px = fma(mi, vsrc[b0 + i], px);
    py = fma(mi, vsrc[n + b0 + i], py);
    pz = fma(mi, vsrc[2 * n + b0 + i], pz);
  }
  red[0][threadIdx.x] = px;
  red[1][threadIdx.x] = py;
  red[2][threadIdx.x] = pz;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
      red[2][threadIdx.x] += red[2][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    D.P[3 * s] = red[0][0];
    D.P[3 * s + 1] = red[1][0];
    D.P[3 * s + 2] = red[2][0];
  }
}

// Encounter test (small systems inline, big systems from ce[]) and universal
// drift of every body not in encounter; encounter bodies of small systems go
// to the small list (the big systems' list was built by their encounter test,
// so this kernel may run beside the big systems' encounter sub-step).
// guess: kGuessPlain or kGuessSeries (universal_drift); mlp != nullptr:
// learned warm start of the solve (merc_mlp.cuh).  log_data
// != nullptr: every solve with x1 >= kWarmMinX1 appends its features and
// training target (5 floats) while the log has room; the network is
// consulted for drifts with x1 >= kWarmNetX1 (warm_long, merc_mlp.cuh).
constexpr float kWarmMinX1 = 1e-5f;
#ifndef MERC_DRIFT_THREADS
#define MERC_DRIFT_THREADS 128
#endif
constexpr int kDriftThreads = MERC_DRIFT_THREADS;  // block of the universal drift (a multiple of 32)

__global__ void k_drift_universal(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, double tol,
                                  int max_iter, double guess, const float* __restrict__ mlp,
                                  float* __restrict__ log_data, unsigned long long* __restrict__ log_count,
                                  long long log_cap, int trigger) {
  griddep_enter();
  // trigger: the encounter task kernel that follows runs beside this one
  if (trigger) griddep_launch();
  __shared__ float blob[kBlob];
  if (mlp) {
    for (int k = threadIdx.x; k < kBlob; k += blockDim.x) blob[k] = mlp[k];
    __syncthreads();
  }
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool ce_small = false, logit = false;
  int its = 0, nonconv = 0, solved = 0;
  float rec[5];
  if (j < D.n) {
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    d3 pos = load3(D.x, n, j);
    bool is_ce;
    if (D.big[s]) {
      is_ce = D.ce[j] != 0;
    } else {
      const int self = self_index(j - b0, compat_block);
      const F4 pf = load_f4(D, j);
      is_ce = false;
      for (int i = 0; i < nm; i++)
        is_ce = is_ce || pair_ce_f(pos, pf, self, i, load_src(D, rc_in, b0 + i), load_f4(D, b0 + i));
      D.ce[j] = is_ce;
      ce_small = is_ce;
    }
    if (!is_ce) {
      d3 vel = load3(D.v, n, j);
      WarmIn w;
      double s0 = guess;  // kGuessPlain or kGuessSeries unless the network guesses
      float rel = 0.0f;
      if (log_data) w = warm_features(pos, vel, dt);  // the logged features in FP64
      if (mlp) {
        float f[4];
        if (warm_long(pos, f32_trunc(dt))) {
          warm_features_f32(pos, vel, f32_trunc(dt), f);
          const float d = warm_delta(blob, f);
          if (d == d) {
            s0 = kGuessRel;
            rel = d;
          }
        }
      }
      UD u = universal_drift(D.u, pos, vel, dt, s0, tol, max_iter, rel);
      store3(D.xo, n, j, u.out.pos);
      store3(D.vo, n, j, u.out.vel);
      its = u.iters;
      nonconv = !u.converged;
      solved = 1;
      if (log_data && u.converged && w.f[0] >= kWarmMinX1) {
        logit = true;
        rec[0] = warm_input0(w);
        rec[1] = w.f[1];
        rec[2] = w.f[2];
        rec[3] = w.f[3];
        rec[4] = warm_target(w, u.s);
      }
    }
  }
  append_ce(ce_small, j, D.ce_list, &D.ce_count[0], &D.counters[0]);
  if (log_data) {
    unsigned mask = __ballot_sync(0xffffffffu, logit);
    if (mask) {
      int leader = __ffs(mask) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(log_count, (unsigned long long)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      unsigned long long slot = base + __popc(mask & ((1u << lane) - 1u));
      if (logit && slot < (unsigned long long)log_cap)
        for (int k = 0; k < 5; k++) log_data[5 * slot + k] = rec[k];
    }
  }
  int wits = __reduce_add_sync(0xffffffffu, its);
  int wsol = __reduce_add_sync(0xffffffffu, solved);
  int wnc = __reduce_add_sync(0xffffffffu, nonconv);
  // iterations the warp executed: the most any of its solves took, for every solving lane
  int wmax = __reduce_max_sync(0xffffffffu, solved ? its : 0);
  if (lane == 0 && wsol) {
    atomicAdd(&D.counters[1], (unsigned long long)wits);
    atomicAdd(&D.counters[2], (unsigned long long)wsol);
    if (wnc) atomicAdd(&D.counters[3], (unsigned long long)wnc);
    atomicAdd(&D.counters[4], (unsigned long long)wmax * (unsigned long long)wsol);
  }
}

// velocity update of an encounter sub-step, one thread, fast pairs
struct FastVelTotal {
  const Dev* D;
  const double* rc;
  int b0, nm, self;
  double soft2;
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    d3 acc = {0.0, 0.0, 0.0};
    for (int i = 0; i < nm; i++) pair_fast<true>(D->u, pos, self, i, load_src(*D, rc, b0 + i), soft2, acc);
    d3 sa = sun_accel(D->u, pos, soft2);
    d3 nv;
    nv.x = fma(sa.x, dt, fma(acc.x, dt, vel.x));
    nv.y = fma(sa.y, dt, fma(acc.y, dt, vel.y));
    nv.z = fma(sa.z, dt, fma(acc.z, dt, vel.z));
    return nv;
  }
};

__global__ void k_encounter_small(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, int rows,
                                  double soft2) {
  griddep_enter();
  const int count = D.ce_count[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int j = D.ce_list[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s];
    FastVelTotal vt{&D, rc_in, b0, D.nm[s], self_index(j - b0, compat_block), soft2};
    PV c = {load3(D.x, n, j), load3(D.v, n, j)};
    PV bs = richardson(c, vt, dt, rows);
    store3(D.xo, n, j, bs.pos);
    store3(D.vo, n, j, bs.vel);
  }
}

// velocity update of an encounter sub-step, the threads of a block split the
// sources; the block sum is a fixed-order tree (all threads get the result)
struct BlockVelTotal {
  const Dev* D;
  const double* rc;
  int b0, nm, self;
  double soft2;
  double* red;  // shared, 3 * blockDim.x
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    d3 acc = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < nm; i += blockDim.x)
      pair_fast<true>(D->u, pos, self, i, load_src(*D, rc, b0 + i), soft2, acc);
    const int t = threadIdx.x, B = blockDim.x;
    __syncthreads();
    red[t] = acc.x;
    red[B + t] = acc.y;
    red[2 * B + t] = acc.z;
    __syncthreads();
    for (int w = B / 2; w > 0; w >>= 1) {
      if (t < w) {
        red[t] += red[t + w];
        red[B + t] += red[B + t + w];
        red[2 * B + t] += red[2 * B + t + w];
      }
      __syncthreads();
    }
    acc = {red[0], red[B], red[2 * B]};
    d3 sa = sun_accel(D->u, pos, soft2);
    d3 nv;
    nv.x = fma(sa.x, dt, fma(acc.x, dt, vel.x));
    nv.y = fma(sa.y, dt, fma(acc.y, dt, vel.y));
    nv.z = fma(sa.z, dt, fma(acc.z, dt, vel.z));
    return nv;
  }
};

__global__ void __launch_bounds__(kEncThreads) k_encounter_big(Dev D, const double* __restrict__ rc_in, double dt,
                                                               int compat_block, int rows, double soft2) {
  __shared__ double red[3 * kEncThreads];
  const int count = D.ce_count[1];
  for (int k = blockIdx.x; k < count; k += gridDim.x) {
    const int j = D.ce_list_big[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s];
    BlockVelTotal vt{&D, rc_in, b0, D.nm[s], self_index(j - b0, compat_block), soft2, red};
    PV c = {load3(D.x, n, j), load3(D.v, n, j)};
    PV bs = richardson(c, vt, dt, rows);
    if (threadIdx.x == 0) {
      store3(D.xo, n, j, bs.pos);
      store3(D.vo, n, j, bs.vel);
    }
    __syncthreads();
  }
}

// Fast term of one source of the encounter sub-step (sim.cuh:357-361 with
// r > r_crit, i.e. weight 1), computed without branches so that consecutive
// sources overlap; returns true when the pair needs the reference formula
// instead (inside r_crit, the body itself, or outside the seed range), in which
// case nothing was added.
__device__ __forceinline__ bool bs_fast_term(const Dev& D, const double* __restrict__ rc, int b0, int self, int i,
                                             const d3& pos, double soft2, d3& acc) {
  const int g = b0 + i;
  const double dx = fsub(D.u, __ldg(D.x + g), pos.x), dy = fsub(D.u, __ldg(D.x + D.n + g), pos.y),
               dz = fsub(D.u, __ldg(D.x + 2 * D.n + g), pos.z);
  const double r2 = fma(dx, dx, fma(dy, dy, fmul(D.u, dz, dz)));
  const bool far = hi_word(r2) > thr_unpack(__ldg(rc + 4 * (size_t)g + 3)) && i != self && seed_in_range(r2);
  const double u = inv_softened_r3(D.u, r2, fadd(D.u, r2, soft2));
  const double w = far ? fmul(D.u, __ldg(D.m + g), u) : 0.0;
  acc.x = fma(w, dx, acc.x);
  acc.y = fma(w, dy, acc.y);
  acc.z = fma(w, dz, acc.z);
  return !far;
}


// Sum over sources c0..c1 - 1 of the encounter body's pull, by one warp:
// sources c0 + lane + 32 k, even k into a0, odd k into a1 (two independent
// FP64 chains in flight), pairs that need the reference formula marked and
// added to ae after each chunk of 64 k (skipped when no lane of the warp has
// one: adding zero changes nothing); then warp_sum3, so every lane ends with
// the same total.
__device__ __forceinline__ d3 warp_source_sum(const Dev& D, const double* __restrict__ rc, int b0, int c0, int c1,
                                              int self, const d3& pos, double soft2) {
  const int lane = (int)(threadIdx.x & 31);
  d3 a0 = {0.0, 0.0, 0.0}, a1 = {0.0, 0.0, 0.0}, ae = {0.0, 0.0, 0.0};
  bool any_slow = false;
  for (int base = c0; base < c1; base += 64 * 32) {
    const int end = min(c1, base + 64 * 32);
    unsigned long long slow = 0ull;
    int k = 0, i = base + lane;
    for (; i + 32 < end; i += 64, k += 2) {
      if (bs_fast_term(D, rc, b0, self, i, pos, soft2, a0)) slow |= 1ull << k;
      if (bs_fast_term(D, rc, b0, self, i + 32, pos, soft2, a1)) slow |= 1ull << (k + 1);
    }
    if (i < end && bs_fast_term(D, rc, b0, self, i, pos, soft2, a0)) slow |= 1ull << k;
    any_slow |= slow != 0ull;
    while (slow) {
      const int q = __ffsll((long long)slow) - 1;
      slow &= slow - 1ull;
      const int src = base + lane + 32 * q;
      if (src == self)
        bs_self_term(D.u, pos, self, load_src(D, rc, b0 + src), soft2, ae);
      else
        pair_exact<true>(pos, self, src, load_src(D, rc, b0 + src), soft2, ae);
    }
  }
  d3 acc = {fadd(D.u, a0.x, a1.x), fadd(D.u, a0.y, a1.y), fadd(D.u, a0.z, a1.z)};
  if (__any_sync(0xffffffffu, any_slow))
    acc = {fadd(D.u, acc.x, ae.x), fadd(D.u, acc.y, ae.y), fadd(D.u, acc.z, ae.z)};
  return warp_sum3(D.u, acc);
}

// Velocity update of an encounter sub-step split over the blocks of a
// thread-block cluster: block `rank` sums its quarter of the sources (fixed
// tree), publishes the partial in its shared memory, and after one cluster
// barrier every block adds the partials of ranks 0..3 in order through
// distributed shared memory.  The partial slots are double-buffered by the
// evaluation parity, so one barrier per evaluation separates the writes of
// evaluation e+1 from the reads of evaluation e-1.
struct ClusterVelTotal {
  const Dev* D;
  const double* rc;
  int b0, c0, c1, self;
  double soft2;
  double* slot;  // shared, 2 x 4 doubles (3 used)
  int* parity;   // per-thread evaluation counter
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    d3 acc = warp_source_sum(*D, rc, b0, c0, c1, self, pos, soft2);
    const int buf = *parity & 1;
    if (threadIdx.x == 0) {
      slot[4 * buf] = acc.x;
      slot[4 * buf + 1] = acc.y;
      slot[4 * buf + 2] = acc.z;
    }
    cl.sync();
    acc = {0.0, 0.0, 0.0};
    for (int r = 0; r < kEncCluster; r++) {
      const double* rs = cl.map_shared_rank(slot, r) + 4 * buf;
      acc.x += rs[0];
      acc.y += rs[1];
      acc.z += rs[2];
    }
    (*parity)++;
    d3 sa = sun_accel(D->u, pos, soft2);
    d3 nv;
    nv.x = fma(sa.x, dt, fma(acc.x, dt, vel.x));
    nv.y = fma(sa.y, dt, fma(acc.y, dt, vel.y));
    nv.z = fma(sa.z, dt, fma(acc.z, dt, vel.z));
    return nv;
  }
};

// Encounter sub-step of the big systems' encounter bodies: one cluster of
// kEncCluster one-warp blocks per body (grid-stride over the list by
// cluster).  The scalar sub-step arithmetic runs in every warp of the
// cluster, so one warp per block keeps that redundancy at kEncCluster warps.
// Every thread of the cluster runs the same Richardson scheme, so the cluster
// barriers inside the velocity updates are reached uniformly.
__global__ void __cluster_dims__(kEncCluster, 1, 1) __launch_bounds__(32)
    k_encounter_cluster(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, int rows,
                        double soft2) {
  griddep_enter();
  namespace cg = cooperative_groups;
  __shared__ double slot[8];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int cid = blockIdx.x / kEncCluster, ncl = gridDim.x / kEncCluster;
  const int count = D.ce_count[1];
  int parity = 0;
  for (int k = cid; k < count; k += ncl) {
    const int j = D.ce_list_big[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    const int c0 = (int)((int64_t)rank * nm / kEncCluster), c1 = (int)((int64_t)(rank + 1) * nm / kEncCluster);
    ClusterVelTotal vt{&D, rc_in, b0, c0, c1, self_index(j - b0, compat_block), soft2, slot, &parity};
    PV c = {load3(D.x, n, j), load3(D.v, n, j)};
    PV bs = richardson(c, vt, dt, rows);
    if (rank == 0 && threadIdx.x == 0) {
      store3(D.xo, n, j, bs.pos);
      store3(D.vo, n, j, bs.vel);
    }
  }
  cl.sync();  // no block leaves while another may still read its slots
}

// Modified-midpoint state of one Richardson row, one evaluation at a time
// (the arithmetic of mod_midpoint with ClusterVelTotal's velocity update):
// the next evaluation is at z1; finish_eval applies the velocity update with
// the summed pull of the sources and advances to the next evaluation point.
struct MidRow {
  d3 z0, z1, vel;
  double h, h2;
  int N, done;
  __device__ __forceinline__ void start(const PV& c, double dt, int nsub) {
    N = nsub;
    h = dt * inv_pow2(N);  // = dt / N exactly
    h2 = 2.0 * h;
    done = 0;
    z1 = {fma(c.vel.x, h, c.pos.x), fma(c.vel.y, h, c.pos.y), fma(c.vel.z, h, c.pos.z)};
    z0 = c.pos;
    vel = c.vel;
  }
  __device__ __forceinline__ void finish_eval(const FU& U, const d3& acc, double soft2) {
    const d3 sa = sun_accel(U, z1, soft2);
    vel = {fma(sa.x, h, fma(acc.x, h, vel.x)), fma(sa.y, h, fma(acc.y, h, vel.y)),
           fma(sa.z, h, fma(acc.z, h, vel.z))};
    if (++done < N) {
      const d3 t = {fma(h2, vel.x, z0.x), fma(h2, vel.y, z0.y), fma(h2, vel.z, z0.z)};
      z0 = z1;
      z1 = t;
    }
  }
  __device__ __forceinline__ PV result() const {
    PV r;
    r.pos = {0.5 * (z1.x + fma(vel.x, h, z0.x)), 0.5 * (z1.y + fma(vel.y, h, z0.y)),
             0.5 * (z1.z + fma(vel.z, h, z0.z))};
    r.vel = vel;
    return r;
  }
};


// Encounter sub-step of the big systems (three Richardson rows, N = 1, 2, 4)
// as a persistent task kernel.  The work of an encounter body is
// enc_tasks_per_body() part sums: evaluations 0-3 of row 2 (N = 4
// sub-steps), 0-1 of row 1 (N = 2) and 0 of row 0 (N = 1), each over
// enc_parts(row, e) contiguous parts of the sources (warp_source_sum).  The rows are independent until the final
// extrapolation, so the critical path is row 2's four evaluations.  Warps take
// tasks from one atomic counter in units of one (row, evaluation) for every
// body, in the order kEncOrder, where every unit follows the one it depends
// on: a task's predecessors were all handed out before it, to warps that are
// running, and a warp whose evaluation e > 0 is not yet published waits for
// it (bounded; then it sets enc_head[1] and every warp stops).  The warp that
// completes the last part of an evaluation (atomic count) adds the part sums
// in part order, advances the row's modified midpoint (MidRow) and publishes
// its state; the warp that completes the last row combines the three rows
// (Richardson) and clears the body's counters for the next step.  The sums
// and their order are fixed (the parts of a row and their order do not depend
// on the schedule), so the results do not depend on which warp runs what.
// Measured on the 2002-body disk (~190 encounter bodies per step): 138 us per
// step against 155 us for a cluster of 7 blocks per two bodies running the
// rows side by side with one cluster barrier per evaluation round; two blocks
// of four warps per SM (one or three or four: slower, more warps lengthen
// every task on the shared FP64 unit); the waits poll with the whole warp
// (a wait by lane 0 alone, the other lanes parked in a shuffle, slowed the
// working warps of the SM 2-3 times).
constexpr int kEncTaskWarps = 4;       // warps per block
constexpr unsigned kEncSleepMax = 256;  // longest sleep between polls, ns (2 us: waiters woke later)
constexpr int kEncSpin = 1 << 22;      // polls of a dependency wait in a step (about two seconds)
constexpr int kEncBlocksPerSM = 2;     // more warps lengthen every task on the shared FP64 unit
// Evaluation slots of an encounter body: 0-3 row 2's evaluations, 4-5 row 1's,
// 6 row 0's.
__host__ __device__ constexpr int enc_slot(int row, int e) { return row == 2 ? e : (row == 1 ? 4 + e : 6); }
// parts of the sources per evaluation slot, one task each, 4 bits per slot.
// Measured on the 2002-body disk (ms per step at ~150 / ~190 encounter
// bodies), by row (0, 1, 2) with every evaluation of a row alike: 3, 3, 5
// parts 0.2695 / 0.2836; 4, 4, 4 0.2757 / 0.2880; 4, 4, 8 0.2821 / 0.2998;
// 2, 2, 2 0.331 / 0.347.  Shorter tasks on the critical row, longer ones
// (fewer per-task costs) on the filler rows.  Six parts on row 2's last
// evaluation (the last tasks handed out) shorten the kernel's tail: 0.2618
// -> 0.2603 ms per step at ~188 encounter bodies (eight: 0.2618; 6 or 8
// parts on earlier evaluations, or 4 on row 1's second, did not pay).
constexpr unsigned kEncPartsBySlot = 5u | 5u << 4 | 5u << 8 | 6u << 12 | 3u << 16 | 3u << 20 | 3u << 24;
__host__ __device__ constexpr int enc_parts_slot(int slot) { return (int)((kEncPartsBySlot >> (4 * slot)) & 15u); }
__host__ __device__ constexpr int enc_parts(int row, int e) { return enc_parts_slot(enc_slot(row, e)); }
// tasks per encounter body, and the first part sum of an evaluation slot
// within a body's kEncQ (3 per part, slots in order)
__host__ __device__ constexpr int enc_tasks_per_body() {
  int t = 0;
  for (int s = 0; s < 7; s++) t += enc_parts_slot(s);
  return t;
}
__host__ __device__ constexpr int enc_qoff(int slot) {
  int o = 0;
  for (int s = 0; s < slot; s++) o += 3 * enc_parts_slot(s);
  return o;
}
// part sums per encounter body: 3 per part of the seven evaluations
constexpr int kEncQ = 3 * enc_tasks_per_body();
// Hand-out order of the seven (row, evaluation) units of enc_parts(row, e) x
// count tasks, 4 bits each (row | e << 2), every unit after the unit it depends
// on: the critical row 2 first, the other rows' units as filler between its
// evaluations.
constexpr unsigned enc_unit(int row, int e) { return (unsigned)(row | e << 2); }
constexpr unsigned kEncOrder = enc_unit(2, 0) | enc_unit(1, 0) << 4 | enc_unit(2, 1) << 8 | enc_unit(0, 0) << 12 |
                               enc_unit(2, 2) << 16 | enc_unit(1, 1) << 20 | enc_unit(2, 3) << 24;
__host__ __device__ constexpr int enc_unit_parts(int unit) {
  return enc_parts((int)((kEncOrder >> (4 * unit)) & 3u), (int)((kEncOrder >> (4 * unit + 2)) & 3u));
}

// Release / acquire forms of the encounter task kernel's publications: the
// part sums and row states a warp stores are ordered before the counter it
// updates (release), and a warp that reads the counter orders its later loads
// after it (acquire), without a full fence on either side.
__device__ __forceinline__ int atom_add_acq_rel(int* p, int v) {
  int r;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int r;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(r) : "l"(p) : "memory");
  return r;
}

// The whole warp polls *flag >= want (one load of the same address; the
// lanes stay converged, so no lane waits in a warp-synchronous instruction
// while another polls); bounded, and it stops early when another warp gave
// up (the shared give-up flag is read every 64th poll).  The sleep between
// polls doubles from 128 ns to kEncSleepMax.  False when the wait gave up.
__device__ __forceinline__ bool enc_wait(const int* flag, int want, int* err, int spin) {
  unsigned ns = 128;
  for (int it = 0; it < spin; it++) {
    if (__all_sync(0xffffffffu, ld_acquire(flag) >= want)) return true;
    if ((it & 63) == 63 && __any_sync(0xffffffffu, *(volatile const int*)err != 0)) return false;
    __nanosleep(ns);
    ns = ns < kEncSleepMax ? 2 * ns : ns;
  }
  if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
  return false;
}

// ONE: a single system (no per-task system lookups)
template <bool ONE>
__global__ void __launch_bounds__(32 * kEncTaskWarps)
    k_encounter_tasks(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, double soft2,
                      int spin, int late_wait) {
  // late_wait: the preceding kernel is the drift, launched after the
  // encounter test completed and independent of this kernel; wait for it at
  // the end instead, so that this kernel's completion implies the drift's
  if (!late_wait) griddep_enter();
  const int lane = (int)(threadIdx.x & 31);
  const int count = D.ce_count[1];
  const int total = enc_tasks_per_body() * count;
  const int nm1 = ONE ? D.nm0 : 0;
  int* err = D.enc_head + 1;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(D.enc_head, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= total || *(volatile const int*)err) break;
    // seven units of enc_parts(row, e) x count tasks, (row, evaluation) in hand-out order
    int unit = 0, u = t;
    while (u >= enc_unit_parts(unit) * count) {
      u -= enc_unit_parts(unit) * count;
      unit++;
    }
    const int row = (kEncOrder >> (4 * unit)) & 3, e = (kEncOrder >> (4 * unit + 2)) & 3;
    const int P = enc_parts(row, e);
    const int k = u / P, q = u % P;
    const int j = D.ce_list_big[k];
    const int n = D.n, s = ONE ? 0 : D.sys[j], b0 = ONE ? 0 : D.off[s], nm = ONE ? nm1 : D.nm[s];
    const int self = self_index(j - b0, compat_block);
    int* cnt = D.enc_cnt + 11 * (size_t)k;
    double* st = D.enc_st + 27 * (size_t)k + 9 * row;
    const int N = 1 << row, slot = enc_slot(row, e);
    MidRow m;
    if (e == 0) {
      m.start(PV{load3(D.x, n, j), load3(D.v, n, j)}, dt, N);
    } else {
      if (!enc_wait(cnt + 7 + row, e, err, spin)) break;
      m.N = N;
      m.h = dt * inv_pow2(N);
      m.h2 = 2.0 * m.h;
      m.done = e;
      m.z0 = {__ldcg(st), __ldcg(st + 1), __ldcg(st + 2)};
      m.z1 = {__ldcg(st + 3), __ldcg(st + 4), __ldcg(st + 5)};
      m.vel = {__ldcg(st + 6), __ldcg(st + 7), __ldcg(st + 8)};
    }
    // part q: whole groups of 32 sources (only the system's last group is
    // partial), so no lane idles in a part's last iteration but the last part's
    const int G = (nm + 31) / 32;
    const int c0 = 32 * (int)((int64_t)q * G / P), c1 = min(32 * (int)((int64_t)(q + 1) * G / P), nm);
    const d3 S = warp_source_sum(D, rc_in, b0, c0, c1, self, m.z1, soft2);
    double* qs = D.enc_q + kEncQ * (size_t)k + enc_qoff(slot);
    int last = 0;
    if (lane == 0) {
      qs[3 * q] = S.x;
      qs[3 * q + 1] = S.y;
      qs[3 * q + 2] = S.z;
      last = atom_add_acq_rel(cnt + slot, 1) == P - 1;
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) continue;
    __syncwarp();  // the other lanes' loads below after lane 0's acquire
    // last part: finish evaluation e of the row (MidRow::finish_eval and
    // result), one component per lane on lanes 0-2 (the other lanes repeat
    // lane 0's and store nothing): the part sums in part order, the sun's
    // pull at z1, the velocity and the next point, each component with the
    // operations of the d3 form
    const int c = lane < 3 ? lane : 0;
    double a = 0.0;
    for (int r = 0; r < P; r++) a += __ldcg(qs + 3 * r + c);
    // The final evaluation of a row: when the other two rows have published
    // their results already (read beside the part sums), this warp is the
    // last of the body and combines the rows at once, their results loaded
    // beside its own finish and its own row's taken from lanes 0-2, without
    // the counter's round trip and the reload (the same values either way).
    // Lanes 0-11 hold the pair of rows their Richardson quotient needs: lanes
    // 0-5 rows 1 and 0 (b11), lanes 6-11 rows 2 and 1 (b21), component cr.
    const bool final_eval = e + 1 == N;
    int others = 0;
    if (final_eval && lane == 0) others = ld_acquire(cnt + 10);
    const bool last_row = __shfl_sync(0xffffffffu, others, 0) == 2;
    __syncwarp();  // the other lanes' loads below after lane 0's acquire
    double* res = D.enc_res + 18 * (size_t)k;
    const int cr = lane < 6 ? lane : lane - 6;  // component: pos x, y, z, vel x, y, z
    const int rhi = lane < 6 ? 1 : 2;           // the finer row; the coarser is rhi - 1
    double o_hi = 0.0, o_lo = 0.0;
    if (last_row && lane < 12) {
      if (rhi != row) o_hi = __ldcg(res + 6 * rhi + cr);
      if (rhi - 1 != row) o_lo = __ldcg(res + 6 * (rhi - 1) + cr);
    }
    const double z0c = c == 0 ? m.z0.x : (c == 1 ? m.z0.y : m.z0.z);
    const double z1c = c == 0 ? m.z1.x : (c == 1 ? m.z1.y : m.z1.z);
    double vc = c == 0 ? m.vel.x : (c == 1 ? m.vel.y : m.vel.z);
    vc = fma(sun_accel_c(D.u, m.z1, z1c, soft2), m.h, fma(a, m.h, vc));
    if (!final_eval) {
      if (lane < 3) {
        st[c] = z1c;                      // z0 of the next evaluation
        st[3 + c] = fma(m.h2, vc, z0c);   // z1, the next evaluation point
        st[6 + c] = vc;
      }
      __syncwarp();  // lanes 1-2's stores before lane 0's release
      if (lane == 0) st_release(cnt + 7 + row, e + 1);
      continue;
    }
    const double pc = 0.5 * (z1c + fma(vc, m.h, z0c));
    if (last_row) {
      const int src = cr < 3 ? cr : cr - 3;
      const double sp = __shfl_sync(0xffffffffu, pc, src & 31), sv = __shfl_sync(0xffffffffu, vc, src & 31);
      const double own = cr < 3 ? sp : sv;
      if (rhi == row) o_hi = own;
      if (rhi - 1 == row) o_lo = own;
    } else {
      if (lane < 3) {
        double* rs = res + 6 * row;
        rs[c] = pc;
        rs[3 + c] = vc;
      }
      __syncwarp();  // lanes 1-2's stores before lane 0's release
      int fin = 0;
      if (lane == 0) fin = atom_add_acq_rel(cnt + 10, 1) == 2;
      if (!__shfl_sync(0xffffffffu, fin, 0)) continue;
      __syncwarp();  // the other lanes' loads below after lane 0's acquire
      if (lane < 12) {
        o_hi = __ldcg(res + 6 * rhi + cr);
        o_lo = __ldcg(res + 6 * (rhi - 1) + cr);
      }
    }
    // The Richardson combination (rich_combine's arithmetic per component),
    // one component per lane: lanes 0-5 combine rows 1 and 0 (b11), lanes
    // 6-11 rows 2 and 1 (b21), then lanes 0-5 b21 and b11 (b22).  A warp
    // instruction costs the FP64 unit the same however few lanes run it, so
    // the eighteen quotients take a few instructions instead of dozens.
    {
      double b = 0.0;
      if (lane < 12) b = rich_q(o_hi, o_lo, 4.0);
      const double b21 = __shfl_sync(0xffffffffu, b, (lane + 6) & 31);
      if (lane < 6) {
        const double b22 = rich_q(b21, b, 16.0);
        if (cr < 3)
          D.xo[(size_t)cr * n + j] = b22;
        else
          D.vo[(size_t)(cr - 3) * n + j] = b22;
      }
    }
    if (lane < 11) cnt[lane] = 0;  // every task of this body is done
  }
  if (late_wait) griddep_wait();
}

// ---------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------
// Energy of each system's massive bodies with the Sun (unsoftened, DH
// variables): one block per system.
__global__ void k_energy(Dev D, double* out) {
  const int s = blockIdx.x;
  const int b0 = D.off[s], nm = D.nm[s], n = D.n;
  __shared__ double red[kThreads];
  double e = 0.0;
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    int g = b0 + i;
    d3 x = load3(D.x, n, g), v = load3(D.v, n, g);
    double mi = D.m[g];
    e += 0.5 * mi * mag2(v) - mi / sqrt(mag2(x));
    for (int k = i + 1; k < nm; k++) {
      d3 y = load3(D.x, n, b0 + k);
      d3 d = {x.x - y.x, x.y - y.y, x.z - y.z};
      e -= mi * D.m[b0 + k] / sqrt(mag2(d));
    }
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double px = 0, py = 0, pz = 0;
    for (int i = 0; i < nm; i++) {
      double mi = D.m[b0 + i];
      px += mi * D.v[b0 + i];
      py += mi * D.v[n + b0 + i];
      pz += mi * D.v[2 * n + b0 + i];
    }
    out[s] = red[0] + 0.5 * (px * px + py * py + pz * pz);
  }
}

// Angular momentum of each system's massive bodies, sum of m x cross v over
// heliocentric positions and democratic-heliocentric (barycentric) velocities,
// which is the system's total (the Sun's share is in the barycentric momenta):
// one block per system, strided partial sums and a fixed tree.
__global__ void k_angmom(Dev D, double* out) {
  const int s = blockIdx.x;
  const int b0 = D.off[s], nm = D.nm[s], n = D.n;
  __shared__ double red[3][kThreads];
  d3 L = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    const int g = b0 + i;
    const d3 x = load3(D.x, n, g), v = load3(D.v, n, g);
    const double mi = D.m[g];
    L.x = fma(mi, fma(x.y, v.z, -x.z * v.y), L.x);
    L.y = fma(mi, fma(x.z, v.x, -x.x * v.z), L.y);
    L.z = fma(mi, fma(x.x, v.y, -x.y * v.x), L.z);
  }
  red[0][threadIdx.x] = L.x;
  red[1][threadIdx.x] = L.y;
  red[2][threadIdx.x] = L.z;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 3; c++) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; c++) out[3 * s + c] = red[c][0];
}

__global__ void k_mm_eval(int fn, int n, const double* x, const double* y, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = x[i];
  double r;
  switch (fn) {
    case 0: r = mm::sin(a); break;
    case 1: r = mm::cos(a); break;
    case 2: r = mm::atan2(a, y[i]); break;
    case 3: r = mm::acos(a); break;
    case 4: r = mm::log(a); break;
    case 5: r = mm::sinh(a); break;
    case 6: r = mm::cosh(a); break;
    case 7: r = mm::cbrt(a); break;
    case 9: r = div_known(a, 3.0, 1.0 / 3.0); break;
    case 10: r = a / y[i]; break;
    case 11: r = div_known(a, 15.0, 1.0 / 15.0); break;
    case 12: r = div_known(a, 63.0, 1.0 / 63.0); break;
    default: r = mm::exp(a); break;
  }
  out[i] = r;
}

// FP64 FMA throughput probe: 8 independent fma chains per thread.
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

inline unsigned blocks_for(int n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace
