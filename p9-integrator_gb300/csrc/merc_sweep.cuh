// merc_sweep.cuh - persistent kernel for batches of small systems.
//
// One launch integrates every system of the batch for all the steps of a
// merc_step call.  Persistent blocks take systems from a device work queue
// (an atomic counter over the systems sorted by size, largest first, so the
// last systems handed out are the shortest).
//
// Test particles are massless: nothing in the step depends on them except
// their own state.  So for a chunk of steps the block's first warp integrates
// the massive bodies (<= 32, one lane each, state in shared memory) and
// records what the test particles need from every step (the history: the two
// momenta of the solar jumps, the massive positions and r_crit tables after
// each jump, the table of the next step's first kick); then every thread
// integrates test particles through the whole chunk, each in registers, with
// no barrier between the phases of a step.  The state of the test particles
// stays in global memory between chunks.  Per body the operations are those
// of the per-phase kernels, in the same order, so the results are the same
// bit for bit.
//
// Adjacent half kicks are merged: the second half kick of step k and the first
// of step k+1 see the same positions, and differ only through the changeover
// radii, which the first one takes from the velocities after the second.  So a
// test particle visits its sources once: a pair outside both radii computes
// its term once and adds it to both kicks' accumulators; the few pairs inside
// either radius get each kick's own weight.  Both accumulators are summed in
// source order exactly as two separate kicks would be, so the result does not
// depend on how the steps are split into calls (and equals the per-phase
// kernels bit for bit).  The massive bodies take the two kicks separately, the
// first of step k+1 after the radii are recomputed.
#pragma once

namespace {

constexpr int kSweepMaxNm = kSmallNm;  // 32

// A work item of the persistent kernel: the test particles [j0, j1) (indices
// within system s) of one system.  A system with many test particles is split
// into several items; every item integrates the system's massive bodies
// itself (bit for bit the same in every item), and the primary item (one
// per system) writes them back through the staging buffers.
struct SweepItem {
  int s, j0, j1, primary;
};

struct SweepArgs {
  Dev D;
  const SweepItem* items;  // largest systems first
  int* queue;              // work counter (zeroed before the launch)
  int nitems, nmax;        // work items, largest system size
  const int* moff;         // per system: first staging slot of its massive bodies
  double* stage;           // 6 per massive body: final position and velocity
  uint32_t* stage_f;       // final flags of each massive body
  int nh;            // largest massive count of the batch (history stride)
  int chunk;         // steps per history chunk
  int steps;
  double dt, soft2, hill, tol, eject_r2;
  double guess;      // kGuessPlain or kGuessSeries
  int compat_block, rows, max_iter;
  const float* mlp;  // warm-start blob or nullptr
  double* rc_final;  // r_crit table for the next call (massive bodies), like D.rc
};

// r_crit table entry of a massive body in shared memory: rc, 0.1 rc, 0.9 rc,
// threshold (as in write_rc)
__device__ __forceinline__ void rc_entry(double* t, int i, const d3& x, const d3& v, double hc) {
  double r = rcrit_hc(x, v, hc);
  t[4 * i] = r;
  t[4 * i + 1] = 0.1 * r;
  t[4 * i + 2] = 0.9 * r;
  t[4 * i + 3] = thr_pack(rc2_threshold(r));
}

__device__ __forceinline__ FastSrc smem_src(const double* X, const double* M, const double* T, int nmax, int i) {
  FastSrc S;
  S.x = X[i];
  S.y = X[nmax + i];
  S.z = X[2 * nmax + i];
  S.m = M[i];
  S.rc = T[4 * i];
  S.rc01 = T[4 * i + 1];
  S.rc09 = T[4 * i + 2];
  S.rc2_hi = thr_unpack(T[4 * i + 3]);
  return S;
}

// History of one step of the massive bodies (stride nh): momenta of the two
// jumps; positions, r_crit table and FP32 prefilter copies after the first
// jump (encounter test and frozen sources of the sub-step); positions and
// r_crit table after the second jump (second half kick) and the table of the
// next step's first half kick.
struct Hist {
  double *P1, *P2, *X1, *T1, *X2, *T2, *TN;
  F4* F1;
  float* R1;
};
__host__ __device__ constexpr size_t hist_step_doubles(int nh) {
  return 6 + 18 * (size_t)nh + 2 * (size_t)nh + ((size_t)nh + 1) / 2;
}
__device__ __forceinline__ Hist hist_at(double* base, int nh, int k) {
  double* p = base + hist_step_doubles(nh) * k;
  Hist h;
  h.P1 = p;
  h.P2 = p + 3;
  h.X1 = p + 6;
  h.T1 = h.X1 + 3 * nh;
  h.X2 = h.T1 + 4 * nh;
  h.T2 = h.X2 + 3 * nh;
  h.TN = h.T2 + 4 * nh;
  h.F1 = (F4*)(h.TN + 4 * nh);
  h.R1 = (float*)(h.F1 + nh);
  return h;
}

struct SmemVelTotal {  // encounter sub-step velocity update, sources in shared memory
  const double *X, *M, *T;
  int nmax, nm, self;
  double soft2;
  FU U;
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    d3 acc = {0.0, 0.0, 0.0};
    for (int i = 0; i < nm; i++) pair_fast<true>(U, pos, self, i, smem_src(X, M, T, nmax, i), soft2, acc);
    d3 sa = sun_accel(U, pos, soft2);
    d3 nv;
    nv.x = fma(sa.x, dt, fma(acc.x, dt, vel.x));
    nv.y = fma(sa.y, dt, fma(acc.y, dt, vel.y));
    nv.z = fma(sa.z, dt, fma(acc.z, dt, vel.z));
    return nv;
  }
};

// (at most 128 registers: the tuner's 128-thread blocks keep 4 blocks per SM;
// 133 registers without the bound cost more than the few spills)
__global__ void __launch_bounds__(256, 2) k_sweep_persistent(SweepArgs A) {
  extern __shared__ double sm[];
  const int nh = A.nh, C = A.chunk;
  double* hist = sm;  // 2 x C steps of history (double-buffered)
  // the network's weights stay in global memory (read through L1): the gate
  // keeps them off the sweep's short drifts, and 5 KB more shared memory per
  // block would cost the small blocks occupancy
  const float* __restrict__ blob = A.mlp;
  auto hist_buf = [&](int b) { return hist + (size_t)b * hist_step_doubles(nh) * C; };
  __shared__ double M[kSweepMaxNm], HC[kSweepMaxNm];           // masses, cbrt(m / 3) * hill
  __shared__ double XM[3 * kSweepMaxNm], VM[3 * kSweepMaxNm];  // massive state
  __shared__ double X0[3 * kSweepMaxNm], T0[4 * kSweepMaxNm];  // positions and table of the call's first kick
  __shared__ int sys_slot, tp_next;
  __shared__ unsigned long long tally[kNumCounters];  // as Dev::counters

  const Dev& D = A.D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double hdt = 0.5 * A.dt;
  unsigned long long my_ce = 0, my_it = 0, my_sol = 0, my_nc = 0, my_simt = 0;
  // Kepler drift or encounter sub-step of one body whose sources are (Xs, Ts)
  auto drift = [&](d3& pos, d3& vel, int self, const Hist& h, int nm, bool& ce) {
    const F4 pf = f4_of(f32_trunc(pos.x), f32_trunc(pos.y), f32_trunc(pos.z));
    ce = false;
    for (int i = 0; i < nm; i++)
      ce = ce || (ce_maybe(pf, h.F1[i], h.R1[i]) && pair_ce(pos, self, i, smem_src(h.X1, M, h.T1, nh, i)));
    PV out;
    if (ce) {
      SmemVelTotal vt{h.X1, M, h.T1, nh, nm, self, A.soft2, D.u};
      out = richardson(PV{pos, vel}, vt, A.dt, A.rows);
      my_ce++;
    } else {
      double s0 = A.guess;  // kGuessPlain or kGuessSeries unless the network guesses
      float rel = 0.0f;
      if (A.mlp) {
        float f[4];
        if (warm_long(pos, f32_trunc(A.dt))) {
          warm_features_f32(pos, vel, f32_trunc(A.dt), f);
          const float d = warm_delta(blob, f);
          if (d == d) {
            s0 = kGuessRel;
            rel = d;
          }
        }
      }
      UD u = universal_drift(D.u, pos, vel, A.dt, s0, A.tol, A.max_iter, rel);
      out = u.out;
      my_it += u.iters;
      my_sol++;
      my_nc += !u.converged;
      {  // iterations the warp executed: the most among the lanes solving here
        const unsigned act = __activemask();
        my_simt += (unsigned long long)__reduce_max_sync(act, u.iters);
      }
    }
    pos = out.pos;
    vel = out.vel;
  };
  auto kick_sum = [&](const d3& pos, int self, const double* Xs, const double* Ts, int nm) {
    d3 acc = {0.0, 0.0, 0.0};
    for (int i = 0; i < nm; i++) pair_fast<false>(D.u, pos, self, i, smem_src(Xs, M, Ts, nh, i), A.soft2, acc);
    return acc;
  };
  auto step_flags = [&](uint32_t f, const d3& pos, const d3& vel) {
    if (A.eject_r2 > 0.0 && mag2(pos) > A.eject_r2) f |= MERC_FLAG_EJECTED;
    bool fin = mm::isfinite_(pos.x) && mm::isfinite_(pos.y) && mm::isfinite_(pos.z) && mm::isfinite_(vel.x) &&
               mm::isfinite_(vel.y) && mm::isfinite_(vel.z);
    if (!fin) f |= MERC_FLAG_NONFINITE;
    return f;
  };

  for (;;) {
    if (tid == 0) sys_slot = atomicAdd(A.queue, 1);
    if (tid < kNumCounters) tally[tid] = 0ull;
    __syncthreads();
    const int slot = sys_slot;
    if (slot >= A.nitems) break;
    const SweepItem item = A.items[slot];
    const int s = item.s;
    const int b0 = D.off[s], nm = D.nm[s];
    // massive bodies: lane i of warp 0 owns body i
    uint32_t fm = 0;
    if (warp == 0 && lane < nm) {
      const int g = b0 + lane;
      M[lane] = D.m[g];
      HC[lane] = mm::cbrt(M[lane] / 3.0) * A.hill;
      for (int c = 0; c < 3; c++) {
        XM[c * kSweepMaxNm + lane] = D.x[c * D.n + g];
        VM[c * kSweepMaxNm + lane] = D.v[c * D.n + g];
      }
      fm = D.flags[g];
    }
    __syncwarp();
    // ---- warp 0: the massive bodies through the chunk of steps c0.., recording
    // the history into hb (counted by the primary item only) ----
    auto massive_chunk = [&](int c0, double* hb) {
      const int cn = min(C, A.steps - c0);
      const unsigned long long sv_ce = my_ce, sv_it = my_it, sv_sol = my_sol, sv_nc = my_nc, sv_simt = my_simt;
      if (warp == 0) {
        const bool act = lane < nm;
        const int self = self_index(lane, A.compat_block);
        auto xm = [&]() { return d3{XM[lane], XM[kSweepMaxNm + lane], XM[2 * kSweepMaxNm + lane]}; };
        auto vm = [&]() { return d3{VM[lane], VM[kSweepMaxNm + lane], VM[2 * kSweepMaxNm + lane]}; };
        auto set_x = [&](const d3& x) {
          XM[lane] = x.x;
          XM[kSweepMaxNm + lane] = x.y;
          XM[2 * kSweepMaxNm + lane] = x.z;
        };
        auto set_v = [&](const d3& v) {
          VM[lane] = v.x;
          VM[kSweepMaxNm + lane] = v.y;
          VM[2 * kSweepMaxNm + lane] = v.z;
        };
        // sum_i m_i v_i in source order (as k_momentum), one component per
        // lane (an FP64 instruction costs the warp's sub-partition the same
        // however few lanes run it)
        auto momentum = [&](double* P) {
          if (lane < 3) {
            double p = 0.0;
            for (int i = 0; i < nm; i++) p = fma(M[i], VM[lane * kSweepMaxNm + i], p);
            P[lane] = p;
          }
          __syncwarp();
        };
        auto jump = [&](const double* P) {
          if (act) {
            d3 x = xm();
            x.x = fma(P[0], hdt, x.x);
            x.y = fma(P[1], hdt, x.y);
            x.z = fma(P[2], hdt, x.z);
            set_x(x);
          }
          __syncwarp();
        };
        // positions and table of a kick (stride nh copies of XM)
        auto record = [&](double* Xs, double* Ts) {
          if (act) {
            const d3 x = xm();
            Xs[lane] = x.x;
            Xs[nh + lane] = x.y;
            Xs[2 * nh + lane] = x.z;
            rc_entry(Ts, lane, x, vm(), HC[lane]);
          }
          __syncwarp();
        };
        // with nm^2 <= 32 the pair terms of all targets in one round, lane
        // t nm + j for target t and source j, then each target's lane adds
        // its terms in source order (kick_term: kick_sum's bits)
        auto kick = [&](const double* Xs, const double* Ts) {
          d3 a = {0.0, 0.0, 0.0};
          if (nm * nm <= 32) {
            const int t = lane / max(nm, 1), j = lane - t * nm;
            double w = 0.0;
            d3 d = {0.0, 0.0, 0.0};
            bool add = false;
            if (lane < nm * nm) {
              const d3 xt = {XM[t], XM[kSweepMaxNm + t], XM[2 * kSweepMaxNm + t]};
              add = kick_term(D.u, xt, self_index(t, A.compat_block), j, smem_src(Xs, M, Ts, nh, j), A.soft2, w, d);
            }
            for (int k = 0; k < nm; k++) {
              const int src = (act ? lane : 0) * nm + k;
              const double ws = __shfl_sync(0xffffffffu, w, src), dx = __shfl_sync(0xffffffffu, d.x, src),
                           dy = __shfl_sync(0xffffffffu, d.y, src), dz = __shfl_sync(0xffffffffu, d.z, src);
              if (__shfl_sync(0xffffffffu, (int)add, src) && act) {
                a.x = fma(ws, dx, a.x);
                a.y = fma(ws, dy, a.y);
                a.z = fma(ws, dz, a.z);
              }
            }
          } else if (act) {
            a = kick_sum(xm(), self, Xs, Ts, nm);
          }
          if (act) {
            d3 v = vm();
            v.x = fma(a.x, hdt, v.x);
            v.y = fma(a.y, hdt, v.y);
            v.z = fma(a.z, hdt, v.z);
            set_v(v);
          }
          __syncwarp();
        };
        if (c0 == 0) {  // the call's first half kick
          record(X0, T0);
          kick(X0, T0);
        }
        for (int k = 0; k < cn; k++) {
          const bool last = c0 + k == A.steps - 1;
          Hist h = hist_at(hb, nh, k);
          momentum(h.P1);
          jump(h.P1);
          record(h.X1, h.T1);
          if (act) {
            h.F1[lane] = f4_of(f32_trunc(h.X1[lane]), f32_trunc(h.X1[nh + lane]), f32_trunc(h.X1[2 * nh + lane]));
            h.R1[lane] = f32_trunc(h.T1[4 * lane]);
          }
          __syncwarp();
          if (act) {
            d3 pos = xm(), vel = vm();
            bool ce;
            drift(pos, vel, self, h, nm, ce);
            fm &= ~MERC_FLAG_CE_LAST;
            if (ce) fm |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
            set_x(pos);
            set_v(vel);
          }
          __syncwarp();
          momentum(h.P2);
          jump(h.P2);
          record(h.X2, h.T2);
          kick(h.X2, h.T2);
          if (act) rc_entry(h.TN, lane, xm(), vm(), HC[lane]);
          __syncwarp();
          if (!last) kick(h.X2, h.TN);
          if (act) fm = step_flags(fm, xm(), vm());
        }
      }
      if (!item.primary) {
        my_ce = sv_ce;
        my_it = sv_it;
        my_sol = sv_sol;
        my_nc = sv_nc;
        my_simt = sv_simt;
      }
    };
    if (A.steps > 0) massive_chunk(0, hist_buf(0));
    for (int c0 = 0, ci = 0; c0 < A.steps; c0 += C, ci++) {
      const int cn = min(C, A.steps - c0);
      double* cur = hist_buf(ci & 1);
      if (tid == 0) tp_next = 0;
      __syncthreads();  // the chunk's history is complete, the other buffer free
      // warp 0 runs one chunk ahead: the next chunk's history into the other
      // buffer, then it joins the test particles of this chunk
      if (c0 + C < A.steps) massive_chunk(c0 + C, hist_buf((ci + 1) & 1));
      // ---- test particles through the chunk, each in registers; warps take
      // 32 at a time from the block's counter ----
      for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&tp_next, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (item.j0 + base >= item.j1) break;
        const int j = item.j0 + base + lane;
        // lanes past the end skip the body (no lane waits in a shuffle while
        // the others integrate)
        if (j < item.j1) {
          const int g = b0 + j, self = self_index(j, A.compat_block);
          d3 pos = {D.x[g], D.x[D.n + g], D.x[2 * D.n + g]};
          d3 vel = {D.v[g], D.v[D.n + g], D.v[2 * D.n + g]};
          uint32_t f = D.flags[g];
          if (c0 == 0) {  // the call's first half kick
            const d3 a = kick_sum(pos, self, X0, T0, nm);
            vel.x = fma(a.x, hdt, vel.x);
            vel.y = fma(a.y, hdt, vel.y);
            vel.z = fma(a.z, hdt, vel.z);
          }
          for (int k = 0; k < cn; k++) {
            const bool last = c0 + k == A.steps - 1;
            const Hist h = hist_at(cur, nh, k);
            pos.x = fma(h.P1[0], hdt, pos.x);
            pos.y = fma(h.P1[1], hdt, pos.y);
            pos.z = fma(h.P1[2], hdt, pos.z);
            bool ce;
            drift(pos, vel, self, h, nm, ce);
            f &= ~MERC_FLAG_CE_LAST;
            if (ce) f |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
            pos.x = fma(h.P2[0], hdt, pos.x);
            pos.y = fma(h.P2[1], hdt, pos.y);
            pos.z = fma(h.P2[2], hdt, pos.z);
            // the second half kick of this step and (unless this is the last
            // step of the call) the first of the next, in one pass
            // accA repeats accB's operations until the first pair that is not
            // far in both kicks, so one accumulator serves both until then
            d3 accB = {0.0, 0.0, 0.0}, accA = {0.0, 0.0, 0.0};
            bool split = false;
            for (int i = 0; i < nm; i++) {
              const FastSrc SB = smem_src(h.X2, M, h.T2, nh, i);
              const int thrA = thr_unpack(h.TN[4 * i + 3]);
              const double dx = fsub(D.u, SB.x, pos.x), dy = fsub(D.u, SB.y, pos.y), dz = fsub(D.u, SB.z, pos.z);
              const double r2 = fma(dx, dx, fma(dy, dy, fmul(D.u, dz, dz)));
              if (!last && hi_word(r2) > max(SB.rc2_hi, thrA) && i != self && seed_in_range(r2)) {
                const double w = fmul(D.u, SB.m, inv_softened_r3(D.u, r2, fadd(D.u, r2, A.soft2)));
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
                pair_fast<false>(D.u, pos, self, i, SB, A.soft2, accB);
                if (!last) pair_fast<false>(D.u, pos, self, i, smem_src(h.X2, M, h.TN, nh, i), A.soft2, accA);
              }
            }
            if (!split) accA = accB;
            vel.x = fma(accB.x, hdt, vel.x);
            vel.y = fma(accB.y, hdt, vel.y);
            vel.z = fma(accB.z, hdt, vel.z);
            if (!last) {
              vel.x = fma(accA.x, hdt, vel.x);
              vel.y = fma(accA.y, hdt, vel.y);
              vel.z = fma(accA.z, hdt, vel.z);
            }
            f = step_flags(f, pos, vel);
          }
          D.x[g] = pos.x;
          D.x[D.n + g] = pos.y;
          D.x[2 * D.n + g] = pos.z;
          D.v[g] = vel.x;
          D.v[D.n + g] = vel.y;
          D.v[2 * D.n + g] = vel.z;
          D.flags[g] = f;
          if (c0 + cn == A.steps) D.ce[g] = (f & MERC_FLAG_CE_LAST) ? 1 : 0;
        }
      }
      __syncthreads();  // before the next chunk overwrites this history
    }
    // the primary item stages the massive bodies (k_sweep_commit writes them
    // back after the launch: other items of the system may still read the
    // state they started from) and writes the radii the next call's first
    // kick uses
    if (item.primary && warp == 0 && lane < nm) {
      const int g = b0 + lane, c = A.moff[s] + lane;
      for (int k = 0; k < 3; k++) {
        A.stage[6 * (size_t)c + k] = XM[k * kSweepMaxNm + lane];
        A.stage[6 * (size_t)c + 3 + k] = VM[k * kSweepMaxNm + lane];
      }
      A.stage_f[c] = fm;
      if (A.steps > 0) {
        const Hist h = hist_at(hist_buf(((A.steps - 1) / C) & 1), nh, (A.steps - 1) % C);
        for (int k = 0; k < 4; k++) A.rc_final[4 * (size_t)g + k] = h.TN[4 * lane + k];
      }
    }
    atomicAdd(&tally[0], my_ce);
    atomicAdd(&tally[1], my_it);
    atomicAdd(&tally[2], my_sol);
    atomicAdd(&tally[3], my_nc);
    atomicAdd(&tally[4], my_simt);
    my_ce = my_it = my_sol = my_nc = my_simt = 0;
    __syncthreads();
    if (tid < kNumCounters && tally[tid]) atomicAdd(&D.counters[tid], tally[tid]);
    __syncthreads();
  }
}

// The staged massive bodies of a persistent launch back into the state
// (massive body c is global body mbody[c]).
__global__ void k_sweep_commit(Dev D, const int* __restrict__ mbody, const double* __restrict__ stage,
                               const uint32_t* __restrict__ stage_f, int nmass) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nmass) return;
  const int g = mbody[c];
  for (int k = 0; k < 3; k++) {
    D.x[k * (size_t)D.n + g] = stage[6 * (size_t)c + k];
    D.v[k * (size_t)D.n + g] = stage[6 * (size_t)c + 3 + k];
  }
  const uint32_t f = stage_f[c];
  D.flags[g] = f;
  D.ce[g] = (f & MERC_FLAG_CE_LAST) ? 1 : 0;
}

}  // namespace
