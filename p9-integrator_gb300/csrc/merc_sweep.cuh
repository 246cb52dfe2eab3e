// merc_sweep.cuh - persistent kernel for batches of small systems.
//
// One launch integrates every system of the batch for all the steps of a
// merc_step call.  Persistent blocks take systems from a device work queue
// (an atomic counter over the systems sorted by size, largest first, so the
// last systems handed out are the shortest).  A block keeps its system's
// whole state in shared memory for all the steps:
//   X[3][nmax], V[3][nmax]          every body (test particles in place)
//   massive-body tables (<= 32):    masses, r_crit tables A and B, drift output
// and runs the Mercurius step with block barriers between the phases.
//
// Adjacent half kicks are merged: the second half kick of step k and the first
// of step k+1 see the same positions, and differ only through the changeover
// radii, which the first one takes from the velocities after the second.  So a
// test particle visits its sources once: a pair outside both radii computes
// its term once and adds it to both kicks' accumulators; the few pairs inside
// either radius get each kick's own weight.  Both accumulators are summed in
// source order exactly as two separate kicks would be, so the result does not
// depend on how the steps are split into calls (and equals the per-phase
// kernels bit for bit).  The massive bodies (<= 32 of them) take the two
// kicks separately, the first of step k+1 after the radii are recomputed.
#pragma once

namespace {

constexpr int kSweepMaxNm = kSmallNm;  // 32

struct SweepArgs {
  Dev D;
  const int* order;  // systems, largest first
  int* queue;        // work counter (zeroed before the launch)
  int nsys, nmax;    // systems, largest system size (shared-memory capacity)
  int steps;
  double dt, soft2, hill, tol, eject_r2;
  int compat_block, rows, max_iter;
  const float* mlp;  // warm-start blob or nullptr
  double* rc_final;  // r_crit table for the next call (massive bodies), like D.rc
};

// r_crit table entry of a massive body in shared memory: rc, 0.1 rc, 0.9 rc,
// threshold (as in write_rc)
__device__ __forceinline__ void rc_entry(double* t, int i, const d3& x, const d3& v, double m, double hill) {
  double r = rcrit(x, v, m, hill);
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

struct SmemVelTotal {  // encounter sub-step velocity update, sources in shared memory
  const double *X, *M, *T;
  int nmax, nm, self;
  double soft2;
  __device__ __forceinline__ d3 operator()(const d3& pos, const d3& vel, double dt) const {
    d3 acc = {0.0, 0.0, 0.0};
    for (int i = 0; i < nm; i++) pair_fast<true>(pos, self, i, smem_src(X, M, T, nmax, i), soft2, acc);
    d3 sa = sun_accel(pos, soft2);
    d3 nv;
    nv.x = fma(sa.x, dt, fma(acc.x, dt, vel.x));
    nv.y = fma(sa.y, dt, fma(acc.y, dt, vel.y));
    nv.z = fma(sa.z, dt, fma(acc.z, dt, vel.z));
    return nv;
  }
};

__global__ void k_sweep_persistent(SweepArgs A) {
  extern __shared__ double sm[];
  const int nmax = A.nmax;
  double* X = sm;                            // 3 nmax
  double* V = X + 3 * (size_t)nmax;          // 3 nmax
  double* M = V + 3 * (size_t)nmax;          // 32
  double* TA = M + kSweepMaxNm;              // 4 x 32
  double* TB = TA + 4 * kSweepMaxNm;         // 4 x 32
  double* XO = TB + 4 * kSweepMaxNm;         // 3 x 32 drift output of massive bodies
  double* VO = XO + 3 * kSweepMaxNm;         // 3 x 32
  double* P = VO + 3 * kSweepMaxNm;          // 4
  F4* SF = (F4*)(P + 4);                     // 32 FP32 copies of the massive positions + r_crit (prefilter)
  float* SRC = (float*)(SF + kSweepMaxNm);   // 32 r_crit (FP32)
  uint32_t* F = (uint32_t*)(SRC + kSweepMaxNm);  // nmax flags
  float* blob = (float*)(F + nmax + (nmax & 1));  // kBlob floats when warm start is on
  __shared__ int sys_slot;
  __shared__ unsigned long long tally[4];    // encounter body-steps, iterations, solves, non-converged

  const Dev& D = A.D;
  const int T = blockDim.x, tid = threadIdx.x;
  const double hdt = 0.5 * A.dt;
  if (A.mlp) {
    for (int k = tid; k < kBlob; k += T) blob[k] = A.mlp[k];
  }
  for (;;) {
    if (tid == 0) sys_slot = atomicAdd(A.queue, 1);
    if (tid < 4) tally[tid] = 0ull;
    __syncthreads();
    const int slot = sys_slot;
    if (slot >= A.nsys) break;
    const int s = A.order[slot];
    const int b0 = D.off[s], n = D.off[s + 1] - b0, nm = D.nm[s];
    // load the system
    for (int j = tid; j < n; j += T) {
      X[j] = D.x[b0 + j];
      X[nmax + j] = D.x[D.n + b0 + j];
      X[2 * nmax + j] = D.x[2 * D.n + b0 + j];
      V[j] = D.v[b0 + j];
      V[nmax + j] = D.v[D.n + b0 + j];
      V[2 * nmax + j] = D.v[2 * D.n + b0 + j];
      F[j] = D.flags[b0 + j];
    }
    if (tid < nm) M[tid] = D.m[b0 + tid];
    __syncthreads();
    if (tid < nm) {
      d3 x = {X[tid], X[nmax + tid], X[2 * nmax + tid]}, v = {V[tid], V[nmax + tid], V[2 * nmax + tid]};
      rc_entry(TA, tid, x, v, M[tid], A.hill);
    }
    __syncthreads();
    unsigned long long my_ce = 0, my_it = 0, my_sol = 0, my_nc = 0;
    // sum_i m_i v_i in source order (as k_momentum), one thread
    auto momentum = [&](const double* VV) {
      if (tid == 0) {
        double px = 0.0, py = 0.0, pz = 0.0;
        for (int i = 0; i < nm; i++) {
          px = fma(M[i], VV[i], px);
          py = fma(M[i], VV[nmax + i], py);
          pz = fma(M[i], VV[2 * nmax + i], pz);
        }
        P[0] = px;
        P[1] = py;
        P[2] = pz;
      }
    };
    // one half kick of body j with table TT (plain kick: self at distance 0 adds nothing)
    auto kick_one = [&](int j, const double* TT) {
      d3 pos = {X[j], X[nmax + j], X[2 * nmax + j]};
      const int self = self_index(j, A.compat_block);
      d3 acc = {0.0, 0.0, 0.0};
      for (int i = 0; i < nm; i++) pair_fast<false>(pos, self, i, smem_src(X, M, TT, nmax, i), A.soft2, acc);
      return acc;
    };
    // first half kick of the call
    for (int j = tid; j < n; j += T) {
      d3 a = kick_one(j, TA);
      V[j] = fma(a.x, hdt, V[j]);
      V[nmax + j] = fma(a.y, hdt, V[nmax + j]);
      V[2 * nmax + j] = fma(a.z, hdt, V[2 * nmax + j]);
    }
    __syncthreads();
    for (int step = 0; step < A.steps; step++) {
      const bool last = step == A.steps - 1;
      // solar jump, then the radii of the drift
      momentum(V);
      __syncthreads();
      for (int j = tid; j < n; j += T) {
        X[j] = fma(P[0], hdt, X[j]);
        X[nmax + j] = fma(P[1], hdt, X[nmax + j]);
        X[2 * nmax + j] = fma(P[2], hdt, X[2 * nmax + j]);
      }
      __syncthreads();
      if (tid < nm) {
        d3 x = {X[tid], X[nmax + tid], X[2 * nmax + tid]}, v = {V[tid], V[nmax + tid], V[2 * nmax + tid]};
        rc_entry(TB, tid, x, v, M[tid], A.hill);
        SF[tid] = f4_of((float)x.x, (float)x.y, (float)x.z);
        SRC[tid] = (float)TB[4 * tid];
      }
      __syncthreads();
      // encounter test and drift / encounter sub-step (sources frozen: the
      // massive bodies write to XO/VO until every body has finished)
      for (int j = tid; j < n; j += T) {
        d3 pos = {X[j], X[nmax + j], X[2 * nmax + j]}, vel = {V[j], V[nmax + j], V[2 * nmax + j]};
        const int self = self_index(j, A.compat_block);
        const F4 pf = f4_of((float)pos.x, (float)pos.y, (float)pos.z);
        bool ce = false;
        for (int i = 0; i < nm; i++)
          ce = ce || (ce_maybe(pf, SF[i], SRC[i]) && pair_ce(pos, self, i, smem_src(X, M, TB, nmax, i)));
        PV out;
        if (ce) {
          SmemVelTotal vt{X, M, TB, nmax, nm, self, A.soft2};
          out = richardson(PV{pos, vel}, vt, A.dt, A.rows);
          my_ce++;
        } else {
          double s0 = 0.0;  // plain guess
          if (A.mlp) {
            const WarmIn w = warm_features(pos, vel, A.dt);
            if (w.f[0] >= kWarmMinX1) s0 = warm_guess(blob, w);
          }
          UD u = universal_drift(pos, vel, A.dt, s0, A.tol, A.max_iter);
          out = u.out;
          my_it += u.iters;
          my_sol++;
          my_nc += !u.converged;
        }
        uint32_t f = F[j] & ~MERC_FLAG_CE_LAST;
        if (ce) f |= MERC_FLAG_CE_LAST | MERC_FLAG_CE_EVER;
        F[j] = f;
        if (j < nm) {
          XO[j] = out.pos.x;
          XO[kSweepMaxNm + j] = out.pos.y;
          XO[2 * kSweepMaxNm + j] = out.pos.z;
          VO[j] = out.vel.x;
          VO[kSweepMaxNm + j] = out.vel.y;
          VO[2 * kSweepMaxNm + j] = out.vel.z;
        } else {
          X[j] = out.pos.x;
          X[nmax + j] = out.pos.y;
          X[2 * nmax + j] = out.pos.z;
          V[j] = out.vel.x;
          V[nmax + j] = out.vel.y;
          V[2 * nmax + j] = out.vel.z;
        }
      }
      __syncthreads();
      if (tid < nm) {
        X[tid] = XO[tid];
        X[nmax + tid] = XO[kSweepMaxNm + tid];
        X[2 * nmax + tid] = XO[2 * kSweepMaxNm + tid];
        V[tid] = VO[tid];
        V[nmax + tid] = VO[kSweepMaxNm + tid];
        V[2 * nmax + tid] = VO[2 * kSweepMaxNm + tid];
      }
      __syncthreads();
      // second solar jump, radii of the second half kick
      momentum(V);
      __syncthreads();
      for (int j = tid; j < n; j += T) {
        X[j] = fma(P[0], hdt, X[j]);
        X[nmax + j] = fma(P[1], hdt, X[nmax + j]);
        X[2 * nmax + j] = fma(P[2], hdt, X[2 * nmax + j]);
      }
      __syncthreads();
      if (tid < nm) {
        d3 x = {X[tid], X[nmax + tid], X[2 * nmax + tid]}, v = {V[tid], V[nmax + tid], V[2 * nmax + tid]};
        rc_entry(TB, tid, x, v, M[tid], A.hill);
      }
      __syncthreads();
      // second half kick of the massive bodies, then the radii of the next
      // step's first half kick from the kicked velocities
      if (tid < nm) {
        d3 a = kick_one(tid, TB);
        V[tid] = fma(a.x, hdt, V[tid]);
        V[nmax + tid] = fma(a.y, hdt, V[nmax + tid]);
        V[2 * nmax + tid] = fma(a.z, hdt, V[2 * nmax + tid]);
      }
      __syncthreads();
      if (tid < nm) {
        d3 x = {X[tid], X[nmax + tid], X[2 * nmax + tid]}, v = {V[tid], V[nmax + tid], V[2 * nmax + tid]};
        rc_entry(TA, tid, x, v, M[tid], A.hill);
      }
      __syncthreads();
      // test particles: the second half kick of this step and (unless this is
      // the last step of the call) the first of the next, in one pass;
      // massive bodies: the first half kick of the next step
      for (int j = tid; j < n; j += T) {
        const int self = self_index(j, A.compat_block);
        d3 pos = {X[j], X[nmax + j], X[2 * nmax + j]};
        d3 vel = {V[j], V[nmax + j], V[2 * nmax + j]};
        if (j < nm) {
          if (!last) {
            d3 a = kick_one(j, TA);
            vel.x = fma(a.x, hdt, vel.x);
            vel.y = fma(a.y, hdt, vel.y);
            vel.z = fma(a.z, hdt, vel.z);
          }
        } else {
          d3 accB = {0.0, 0.0, 0.0}, accA = {0.0, 0.0, 0.0};  // this step's second, next step's first
          for (int i = 0; i < nm; i++) {
            FastSrc SB = smem_src(X, M, TB, nmax, i);
            const int thrA = thr_unpack(TA[4 * i + 3]);
            double dx = SB.x - pos.x, dy = SB.y - pos.y, dz = SB.z - pos.z;
            double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
            if (!last && hi_word(r2) > max(SB.rc2_hi, thrA) && i != self && seed_in_range(r2)) {
              double w = SB.m * inv_softened_r3(r2, r2 + A.soft2);
              accB.x = fma(w, dx, accB.x);
              accB.y = fma(w, dy, accB.y);
              accB.z = fma(w, dz, accB.z);
              accA.x = fma(w, dx, accA.x);
              accA.y = fma(w, dy, accA.y);
              accA.z = fma(w, dz, accA.z);
            } else {
              pair_fast<false>(pos, self, i, SB, A.soft2, accB);
              if (!last) pair_fast<false>(pos, self, i, smem_src(X, M, TA, nmax, i), A.soft2, accA);
            }
          }
          vel.x = fma(accB.x, hdt, vel.x);
          vel.y = fma(accB.y, hdt, vel.y);
          vel.z = fma(accB.z, hdt, vel.z);
          if (!last) {
            vel.x = fma(accA.x, hdt, vel.x);
            vel.y = fma(accA.y, hdt, vel.y);
            vel.z = fma(accA.z, hdt, vel.z);
          }
        }
        // flags of the step (positions are the step's final ones)
        uint32_t f = F[j];
        if (A.eject_r2 > 0.0 && mag2(pos) > A.eject_r2) f |= MERC_FLAG_EJECTED;
        // the state checked is the one after the second half kick
        bool fin = mm::isfinite_(pos.x) && mm::isfinite_(pos.y) && mm::isfinite_(pos.z) && mm::isfinite_(vel.x) &&
                   mm::isfinite_(vel.y) && mm::isfinite_(vel.z);
        if (!fin) f |= MERC_FLAG_NONFINITE;
        F[j] = f;
        V[j] = vel.x;
        V[nmax + j] = vel.y;
        V[2 * nmax + j] = vel.z;
      }
      __syncthreads();
    }
    // write the system back, and the radii the next call's first kick uses
    for (int j = tid; j < n; j += T) {
      D.x[b0 + j] = X[j];
      D.x[D.n + b0 + j] = X[nmax + j];
      D.x[2 * D.n + b0 + j] = X[2 * nmax + j];
      D.v[b0 + j] = V[j];
      D.v[D.n + b0 + j] = V[nmax + j];
      D.v[2 * D.n + b0 + j] = V[2 * nmax + j];
      D.flags[b0 + j] = F[j];
      D.ce[b0 + j] = (F[j] & MERC_FLAG_CE_LAST) ? 1 : 0;
    }
    if (tid < nm) {
      for (int k = 0; k < 4; k++) A.rc_final[4 * (size_t)(b0 + tid) + k] = TA[4 * tid + k];
    }
    atomicAdd(&tally[0], my_ce);
    atomicAdd(&tally[1], my_it);
    atomicAdd(&tally[2], my_sol);
    atomicAdd(&tally[3], my_nc);
    __syncthreads();
    if (tid < 4 && tally[tid]) atomicAdd(&D.counters[tid], tally[tid]);
    __syncthreads();
  }
}

}  // namespace
