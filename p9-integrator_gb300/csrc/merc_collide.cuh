// merc_collide.cuh - physical collisions (optional, merc_set_radii).
//
// No counterpart in the reference: its encounter test only chooses the
// sub-stepper (src/sim.cuh:589-613, 699-730).  Once per step, after the drift
// and the encounter sub-step and before the second solar jump, every body in
// close encounter that step (the two encounter lists) is tested against the
// massive bodies of its system in the drift outputs xo: |x_a - x_b| <
// R_a + R_b.  One warp per listed body, lanes over the sources; a hit appends
// the pair (a < b) to a candidate list.  One thread then sorts the step's
// candidates, drops duplicates (a massive pair is found from both sides) and
// merges them in ascending order while both bodies are unmerged, so the
// result does not depend on the order the warps found them in:
//   survivor s = the heavier (the lower index on a tie), other body o;
//   if o is massive: M = m_s + m_o, x_s = (m_s x_s + m_o x_o) / M,
//     v_s likewise (momentum and centre of mass kept), m_s = M, hc_s anew;
//     m_o = MERC_MERGED_MASS (a source keeps a non-zero critical radius, which
//     the reference's changeover formula divides by);
//   o is parked on a circular orbit at MERC_PARK_R + 64 x (its index in the
//   system) AU on the x axis (a_lag set to that radius), flags GREW on s and
//   MERGED on o, and the event (step, s, o) is logged.
// Collisions are rare, so the single resolving thread costs nothing; a step
// without candidates returns at once.  The CPU oracle restates the same rule
// (oracle/merc_oracle.cpp, collide()).

constexpr int kColPairCap = 4096;     // candidate pairs per step
constexpr int kColEventCap = 65536;   // logged events per context

struct Collide {
  const double* radius = nullptr;  // n
  double* m = nullptr;             // n, the context's masses (writable)
  int* n_pairs = nullptr;          // [0] candidates of this step, [1] candidates lost to a full list (sticky)
  int2* pairs = nullptr;           // kColPairCap
  long long* step = nullptr;       // steps since load, advanced by k_collide_resolve
  long long* n_events = nullptr;   // events since merc_set_radii
  long long* events = nullptr;     // 3 x kColEventCap: step, survivor, absorbed
};

__global__ void k_collide_find(Dev D, Collide C) {
  griddep_enter();
  const int lane = (int)(threadIdx.x & 31);
  const int warps = (int)(gridDim.x * (blockDim.x >> 5));
  const int n0 = D.ce_count[0], n1 = D.ce_count[1], n = D.n;
  for (int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); e < n0 + n1; e += warps) {
    const int j = e < n0 ? D.ce_list[e] : D.ce_list_big[e - n0];
    if (D.flags[j] & MERC_FLAG_MERGED) continue;
    const int s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    for (int i = b0 + lane; i < b0 + nm; i += 32) {
      if (i == j || (D.flags[i] & MERC_FLAG_MERGED)) continue;
      const int a = min(i, j), b = max(i, j);
      const double dx = D.xo[b] - D.xo[a], dy = D.xo[n + b] - D.xo[n + a], dz = D.xo[2 * n + b] - D.xo[2 * n + a];
      const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
      const double rs = C.radius[a] + C.radius[b];
      if (d2 < rs * rs) {
        const int k = atomicAdd(C.n_pairs, 1);
        if (k < kColPairCap)
          C.pairs[k] = make_int2(a, b);
        else
          atomicExch(C.n_pairs + 1, 1);
      }
    }
  }
}

__device__ __forceinline__ long long col_key(int2 p) { return ((long long)p.x << 32) | (unsigned)p.y; }

__global__ void k_collide_resolve(Dev D, Collide C, double hill) {
  griddep_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const long long step = ++(*C.step);
  const int found = *C.n_pairs;
  *C.n_pairs = 0;
  const int np = min(found, kColPairCap);
  if (np == 0) return;
  int2* P = C.pairs;
  for (int k = 1; k < np; k++) {  // insertion sort by (a, b)
    const int2 v = P[k];
    int q = k - 1;
    while (q >= 0 && col_key(P[q]) > col_key(v)) {
      P[q + 1] = P[q];
      q--;
    }
    P[q + 1] = v;
  }
  const int n = D.n;
  for (int k = 0; k < np; k++) {
    if (k > 0 && col_key(P[k]) == col_key(P[k - 1])) continue;
    const int a = P[k].x, b = P[k].y;
    if ((D.flags[a] | D.flags[b]) & MERC_FLAG_MERGED) continue;
    const int s = C.m[b] > C.m[a] ? b : a, o = s == a ? b : a;
    const int sys = D.sys[o], b0 = D.off[sys];
    if (o - b0 < D.nm[sys]) {
      const double ms = C.m[s], mo = C.m[o], M = ms + mo;
      for (int c = 0; c < 3; c++) {
        D.xo[c * n + s] = fma(ms, D.xo[c * n + s], mo * D.xo[c * n + o]) / M;
        D.vo[c * n + s] = fma(ms, D.vo[c * n + s], mo * D.vo[c * n + o]) / M;
      }
      C.m[s] = M;
      D.hc[s] = mm::cbrt(M / 3.0) * hill;
      C.m[o] = MERC_MERGED_MASS;
      D.hc[o] = mm::cbrt(MERC_MERGED_MASS / 3.0) * hill;
    }
    const double r = MERC_PARK_R + 64.0 * (double)(o - b0);
    D.xo[o] = r;
    D.xo[n + o] = 0.0;
    D.xo[2 * n + o] = 0.0;
    D.vo[o] = 0.0;
    D.vo[n + o] = 1.0 / sqrt(r);
    D.vo[2 * n + o] = 0.0;
    D.alag[o] = r;
    D.flags[s] |= MERC_FLAG_GREW;
    D.flags[o] |= MERC_FLAG_MERGED;
    const long long ev = (*C.n_events)++;
    if (ev < kColEventCap) {
      C.events[3 * ev] = step;
      C.events[3 * ev + 1] = s;
      C.events[3 * ev + 2] = o;
    }
  }
}
