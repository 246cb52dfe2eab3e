// merc_engine.cu - the Mercurius step on the GPU and the C ABI of libmerc.so.
//
// State layout in HBM (structure of arrays, binary64):
//   x[3][n], v[3][n]   heliocentric positions, democratic-heliocentric velocities
//   m[n], a_lag[n]     masses, semi-major axis of the previous element evaluation
//   flags[n]           MERC_FLAG_* per body
// for all systems concatenated body-wise (system s owns [off[s], off[s+1])).
//
// One step (the loop body of mercurius_solver, reference src/sim.cuh:679-742)
// is a fixed sequence of kernels, captured once into a CUDA graph and
// replayed:
//   kick(dt/2) -> momentum -> jump(dt/2) -> encounter test + drift ->
//   encounter sub-step of the compacted encounter list -> momentum ->
//   jump(dt/2) -> kick(dt/2)
// Each kernel reads the state the previous one wrote, so the phases that the
// reference separates with cluster.sync() are separated by kernel boundaries;
// every source is read before any body is written (the race-free order of the
// reference's racy kicks, sim.cuh:684-685, 740-741).
//
// Two arithmetic paths share this sequence:
//  - drift = MERC_DRIFT_ELEMENTS reproduces the reference's operation order
//    (sequential source sums per body, sequential momentum sums, merc_math
//    functions), bit for bit with the CPU check, because that drift
//    amplifies rounding differences by ~1e6 in 100 steps;
//  - drift = MERC_DRIFT_UNIVERSAL uses the universal-variable solve, whose
//    rounding sensitivity is ~100x smaller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/merc.h"
#include "../../include/merc_diag.h"
#include "merc_device.cuh"

using namespace merc;

namespace {

constexpr int kThreads = 128;

struct Dev {
  int n = 0;     // bodies, all systems
  int nsys = 0;  // systems
  const int* off = nullptr;
  const int* nm = nullptr;
  const int* sys = nullptr;  // system of each body
  double* x = nullptr;       // 3 n
  double* v = nullptr;       // 3 n
  double* xo = nullptr;      // 3 n, drift output
  double* vo = nullptr;      // 3 n
  const double* m = nullptr;
  double* alag = nullptr;
  uint32_t* flags = nullptr;
  unsigned char* ce = nullptr;  // encounter flag of the current step
  double* rc[2] = {nullptr, nullptr};  // 3 per body: rc, 0.1 rc, 0.9 rc (massive bodies only)
  double* P = nullptr;               // 3 per system
  int* ce_list = nullptr;
  int* ce_count = nullptr;
  unsigned long long* counters = nullptr;  // CE body-steps, Kepler iterations, solves, non-converged
};

__device__ __forceinline__ SrcView src_view(const Dev& D, const double* rc, int b0) {
  SrcView S;
  S.x = D.x + b0;
  S.y = D.x + D.n + b0;
  S.z = D.x + 2 * D.n + b0;
  S.m = D.m + b0;
  S.rc = rc + 3 * (size_t)b0;
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

__device__ __forceinline__ void write_rc(double* rc, int j, const d3& x, const d3& v, double m, double hill) {
  double r = rcrit(x, v, m, hill);
  rc[3 * (size_t)j] = r;
  rc[3 * (size_t)j + 1] = 0.1 * r;
  rc[3 * (size_t)j + 2] = 0.9 * r;
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
  write_rc(rc_out, j, load3(D.x, D.n, j), load3(D.v, D.n, j), D.m[j], hill);
}

// ---------------------------------------------------------------------------
// step kernels
// ---------------------------------------------------------------------------
// Half kick of every body (sim.cuh:683-685, 739-741).  When rc_out is given,
// each massive body also writes the changeover radius of its new state for
// the next phase; when `last` is set the step's flags are updated.
__global__ void k_kick(Dev D, const double* __restrict__ rc_in, double* __restrict__ rc_out, double hdt,
                       double soft2, int compat_block, double hill, double eject_r2, int last) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
  const int local = j - b0;
  SrcView S = src_view(D, rc_in, b0);
  d3 pos = load3(D.x, n, j);
  d3 vel = kick_exact<false>(pos, load3(D.v, n, j), self_index(local, compat_block), S, nm, hdt, soft2);
  store3(D.v, n, j, vel);
  if (rc_out && local < nm) write_rc(rc_out, j, pos, vel, D.m[j], hill);
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

// sum_i m_i v_i of each system in the reference order (main_body_kinetic,
// sim.cuh:394-399); `vsrc` is the velocity array to sum.
__global__ void k_momentum(Dev D, const double* __restrict__ vsrc) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= D.nsys) return;
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
__global__ void k_jump(Dev D, const double* __restrict__ xsrc, const double* __restrict__ vsrc, double* rc_out,
                       double hdt, double hill) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.n) return;
  const int n = D.n, s = D.sys[j];
  const double px = D.P[3 * s], py = D.P[3 * s + 1], pz = D.P[3 * s + 2];
  d3 x = load3(xsrc, n, j);
  x.x = fma(px, hdt, x.x);
  x.y = fma(py, hdt, x.y);
  x.z = fma(pz, hdt, x.z);
  store3(D.x, n, j, x);
  d3 v;
  if (vsrc) {
    v = load3(vsrc, n, j);
    store3(D.v, n, j, v);
  } else {
    v = load3(D.v, n, j);
  }
  if (j - D.off[s] < D.nm[s]) write_rc(rc_out, j, x, v, D.m[j], hill);
}

// Encounter test and Kepler drift of every body (sim.cuh:692-713).  Bodies in
// encounter are appended to the encounter list (warp ballot + prefix count);
// the rest write their drifted state to xo/vo.  The element drift keeps the
// reference's lagged mean motion (sim.cuh:692 uses a from the previous step).
template <int DRIFT>
__global__ void k_drift(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, int kep_iters,
                        double tol, int max_iter) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = j < D.n;
  const int lane = threadIdx.x & 31;
  bool is_ce = false;
  int its = 0, nonconv = 0;
  if (active) {
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    const int self = self_index(j - b0, compat_block);
    SrcView S = src_view(D, rc_in, b0);
    d3 pos = load3(D.x, n, j), vel = load3(D.v, n, j);
    is_ce = close_encounter(pos, self, S, nm);
    D.ce[j] = is_ce;
    if (DRIFT == MERC_DRIFT_ELEMENTS) {
      const double tp = 6.283185307179586476925286766559005768394338798750211641949;
      double a = D.alag[j];
      double nmot = rsqrt_ieee(a * a * a);
      Elem el = elem_from_cart(pos, vel);
      D.alag[j] = el.a;
      double Mn = (double)(!is_ce) * fmod(fma(nmot, dt, el.M), tp) + (double)(is_ce)*el.M;
      PV kep = cart_from_elem(el.inc, el.node, el.peri, Mn, el.e, el.a, kep_iters);
      // for encounter bodies the Kepler result still enters the blend
      // fma(0, kep, bs) of sim.cuh:718-730; the sub-step kernel completes it
      store3(D.xo, n, j, kep.pos);
      store3(D.vo, n, j, kep.vel);
    } else if (!is_ce) {
      double s0 = dt / sqrt(mag2(pos));
      UD u = universal_drift(pos, vel, dt, s0, tol, max_iter);
      store3(D.xo, n, j, u.out.pos);
      store3(D.vo, n, j, u.out.vel);
      its = u.iters;
      nonconv = !u.converged;
    }
  }
  // compaction of the encounter list
  unsigned mask = __ballot_sync(0xffffffffu, is_ce);
  if (mask) {
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(D.ce_count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (is_ce) D.ce_list[base + __popc(mask & ((1u << lane) - 1u))] = j;
    if (lane == leader) atomicAdd(&D.counters[0], (unsigned long long)__popc(mask));
  }
  if (DRIFT == MERC_DRIFT_UNIVERSAL) {
    int wits = __reduce_add_sync(0xffffffffu, its);
    int wsol = __reduce_add_sync(0xffffffffu, (active && !is_ce) ? 1 : 0);
    int wnc = __reduce_add_sync(0xffffffffu, nonconv);
    if (lane == 0 && wsol) {
      atomicAdd(&D.counters[1], (unsigned long long)wits);
      atomicAdd(&D.counters[2], (unsigned long long)wsol);
      if (wnc) atomicAdd(&D.counters[3], (unsigned long long)wnc);
    }
  }
}

// Encounter sub-step (Richardson extrapolation of modified-midpoint steps
// against sources frozen at the start of the drift, sim.cuh:701-702) of every
// body on the encounter list; grid-stride over the list.
template <int DRIFT>
__global__ void k_encounter(Dev D, const double* __restrict__ rc_in, double dt, int compat_block, int rows,
                            double soft2) {
  const int count = *D.ce_count;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int j = D.ce_list[k];
    const int n = D.n, s = D.sys[j], b0 = D.off[s], nm = D.nm[s];
    SrcView S = src_view(D, rc_in, b0);
    PV c = {load3(D.x, n, j), load3(D.v, n, j)};
    PV bs = richardson(c, self_index(j - b0, compat_block), S, nm, dt, rows, soft2);
    if (DRIFT == MERC_DRIFT_ELEMENTS) {
      d3 kp = load3(D.xo, n, j), kv = load3(D.vo, n, j);
      bs.pos = {fma(0.0, kp.x, bs.pos.x), fma(0.0, kp.y, bs.pos.y), fma(0.0, kp.z, bs.pos.z)};
      bs.vel = {fma(0.0, kv.x, bs.vel.x), fma(0.0, kv.y, bs.vel.y), fma(0.0, kv.z, bs.vel.z)};
    }
    store3(D.xo, n, j, bs.pos);
    store3(D.vo, n, j, bs.vel);
  }
}

// Energy of each system's massive bodies with the Sun (unsoftened, DH
// variables): one block per system, compensated block sums.
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

// ---- diagnostics ----
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

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct merc_ctx {
  int device = 0;
  merc_params p{};
  cudaStream_t stream = nullptr;
  std::string err;
  Dev D;
  int* d_off = nullptr;
  int* d_nm = nullptr;
  int* d_sys = nullptr;
  double* d_m = nullptr;
  std::vector<void*> allocs;
  std::vector<int> h_off, h_nm;
  bool loaded = false;
  int rc_cur = 0;  // buffer holding r_crit for the next first kick
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int enc_blocks = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> kick_ev;  // start/end pairs recorded around kicks inside the graph
  bool time_kicks = false;
  int64_t steps_done = 0;
  int64_t launches = 0;
  int64_t graph_launch_kernels = 0;
  double last_ms = 0.0;
};

namespace {

int fail(merc_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                                      \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                           \
  } while (0)

int check_params(merc_ctx* ctx, const merc_params* p) {
  if (!(p->dt > 0.0) || !(p->softening2 >= 0.0) || !(p->hill_factor > 0.0) || !(p->kepler_tol >= 0.0))
    return fail(ctx, MERC_ERR_CONFIG, "invalid parameter: dt, softening2, hill_factor, kepler_tol");
  if (p->kepler_iters < 1 || p->kepler_iters > 64) return fail(ctx, MERC_ERR_CONFIG, "kepler_iters out of 1..64");
  if (p->bs_rows < 1 || p->bs_rows > 4) return fail(ctx, MERC_ERR_CONFIG, "bs_rows out of 1..4");
  if (p->compat_block < 0) return fail(ctx, MERC_ERR_CONFIG, "compat_block < 0");
  if (p->drift != MERC_DRIFT_ELEMENTS && p->drift != MERC_DRIFT_UNIVERSAL)
    return fail(ctx, MERC_ERR_CONFIG, "unknown drift %d", p->drift);
  if (p->kepler_max_iter < 1 || p->kepler_max_iter > 1000)
    return fail(ctx, MERC_ERR_CONFIG, "kepler_max_iter out of 1..1000");
  if (p->warm_start != MERC_WARM_PLAIN && p->warm_start != MERC_WARM_MLP)
    return fail(ctx, MERC_ERR_CONFIG, "unknown warm_start %d", p->warm_start);
  return MERC_OK;
}

void free_all(merc_ctx* ctx) {
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  ctx->graph = nullptr;
  ctx->graph_steps = 0;
  for (void* a : ctx->allocs) cudaFree(a);
  ctx->allocs.clear();
  ctx->D = Dev();
  ctx->loaded = false;
}

template <class T> int dalloc(merc_ctx* ctx, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                                    cudaGetErrorString(e));
  ctx->allocs.push_back(q);
  *p = (T*)q;
  return MERC_OK;
}

int validate_layout(merc_ctx* ctx, int32_t n_systems, const int64_t* off, const int32_t* nm, const double* mass) {
  if (n_systems <= 0 || !off || !nm || !mass) return fail(ctx, MERC_ERR_CONFIG, "empty or NULL system layout");
  if (off[0] != 0) return fail(ctx, MERC_ERR_CONFIG, "body_offset[0] must be 0");
  for (int s = 0; s < n_systems; s++) {
    int64_t n = off[s + 1] - off[s];
    if (n <= 0) return fail(ctx, MERC_ERR_CONFIG, "system %d has no bodies", s);
    if (nm[s] < 0 || nm[s] > n) return fail(ctx, MERC_ERR_CONFIG, "system %d: n_massive %d out of 0..%lld", s, nm[s],
                                            (long long)n);
  }
  if (off[n_systems] > (int64_t)INT32_MAX / 3) return fail(ctx, MERC_ERR_CONFIG, "too many bodies");
  return MERC_OK;
}

int alloc_state(merc_ctx* ctx, int32_t n_systems, const int64_t* off, const int32_t* nm, const double* mass) {
  free_all(ctx);
  const int n = (int)off[n_systems];
  ctx->h_off.assign(n_systems + 1, 0);
  ctx->h_nm.assign(nm, nm + n_systems);
  std::vector<int> sys(n);
  for (int s = 0; s < n_systems; s++) {
    ctx->h_off[s + 1] = (int)off[s + 1];
    for (int64_t j = off[s]; j < off[s + 1]; j++) sys[j] = s;
  }
  Dev& D = ctx->D;
  D.n = n;
  D.nsys = n_systems;
  int st;
  if ((st = dalloc(ctx, &ctx->d_off, n_systems + 1)) || (st = dalloc(ctx, &ctx->d_nm, n_systems)) ||
      (st = dalloc(ctx, &ctx->d_sys, n)) || (st = dalloc(ctx, &ctx->d_m, n)) || (st = dalloc(ctx, &D.x, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.v, 3 * (size_t)n)) || (st = dalloc(ctx, &D.xo, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.vo, 3 * (size_t)n)) || (st = dalloc(ctx, &D.alag, n)) || (st = dalloc(ctx, &D.flags, n)) ||
      (st = dalloc(ctx, &D.ce, n)) || (st = dalloc(ctx, &D.rc[0], 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.rc[1], 3 * (size_t)n)) || (st = dalloc(ctx, &D.P, 3 * (size_t)n_systems)) ||
      (st = dalloc(ctx, &D.ce_list, n)) || (st = dalloc(ctx, &D.ce_count, 1)) || (st = dalloc(ctx, &D.counters, 4)))
    return st;
  D.off = ctx->d_off;
  D.nm = ctx->d_nm;
  D.sys = ctx->d_sys;
  D.m = ctx->d_m;
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_off, ctx->h_off.data(), sizeof(int) * (n_systems + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_nm, nm, sizeof(int) * n_systems, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_sys, sys.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(D.flags, 0, sizeof(uint32_t) * n, s));
  CK(cudaMemsetAsync(D.ce, 0, n, s));
  CK(cudaMemsetAsync(D.counters, 0, sizeof(unsigned long long) * 4, s));
  CK(cudaMemsetAsync(D.rc[0], 0, sizeof(double) * 3 * n, s));
  CK(cudaMemsetAsync(D.rc[1], 0, sizeof(double) * 3 * n, s));
  CK(cudaStreamSynchronize(s));  // the host vectors above are temporaries
  int dev_sms = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  ctx->enc_blocks = std::max(1, dev_sms) * 4;
  ctx->steps_done = 0;
  return MERC_OK;
}

// r_crit of the current state into the buffer the first kick reads
int compute_rc(merc_ctx* ctx) {
  Dev& D = ctx->D;
  k_rc<<<blocks_for(D.n), kThreads, 0, ctx->stream>>>(D, D.rc[ctx->rc_cur], ctx->p.hill_factor);
  ctx->launches++;
  CK(cudaGetLastError());
  return MERC_OK;
}

int dh_convert(merc_ctx* ctx, bool reverse) {
  Dev& D = ctx->D;
  k_dh_sums<<<blocks_for(D.nsys), kThreads, 0, ctx->stream>>>(D, reverse);
  k_dh_apply<<<blocks_for(D.n), kThreads, 0, ctx->stream>>>(D, reverse ? 1.0 : -1.0);
  ctx->launches += 2;
  CK(cudaGetLastError());
  return MERC_OK;
}

// Enqueue one step on the stream (also used while capturing the graph).
int enqueue_step(merc_ctx* ctx, bool record_kick_events, int step_in_graph) {
  Dev& D = ctx->D;
  const merc_params& p = ctx->p;
  cudaStream_t s = ctx->stream;
  const double hdt = 0.5 * p.dt;
  const unsigned nb = blocks_for(D.n), sb = blocks_for(D.nsys);
  const double ej2 = p.eject_r > 0 ? p.eject_r * p.eject_r : 0.0;
  double* rcA = D.rc[ctx->rc_cur];
  double* rcB = D.rc[ctx->rc_cur ^ 1];
  auto kick_ev = [&](int k) {
    if (record_kick_events) CK(cudaEventRecord(ctx->kick_ev[4 * step_in_graph + k], s));
    return MERC_OK;
  };
  int st;
  if ((st = kick_ev(0))) return st;
  k_kick<<<nb, kThreads, 0, s>>>(D, rcA, nullptr, hdt, p.softening2, p.compat_block, p.hill_factor, ej2, 0);
  if ((st = kick_ev(1))) return st;
  k_momentum<<<sb, kThreads, 0, s>>>(D, D.v);
  k_jump<<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt, p.hill_factor);
  CK(cudaMemsetAsync(D.ce_count, 0, sizeof(int), s));
  if (p.drift == MERC_DRIFT_ELEMENTS) {
    k_drift<MERC_DRIFT_ELEMENTS><<<nb, kThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.kepler_iters,
                                                         p.kepler_tol, p.kepler_max_iter);
    k_encounter<MERC_DRIFT_ELEMENTS><<<ctx->enc_blocks, 64, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows,
                                                                    p.softening2);
  } else {
    k_drift<MERC_DRIFT_UNIVERSAL><<<nb, kThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.kepler_iters,
                                                          p.kepler_tol, p.kepler_max_iter);
    k_encounter<MERC_DRIFT_UNIVERSAL><<<ctx->enc_blocks, 64, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows,
                                                                     p.softening2);
  }
  k_momentum<<<sb, kThreads, 0, s>>>(D, D.vo);
  k_jump<<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt, p.hill_factor);
  if ((st = kick_ev(2))) return st;
  k_kick<<<nb, kThreads, 0, s>>>(D, rcB, rcA, hdt, p.softening2, p.compat_block, p.hill_factor, ej2, 1);
  if ((st = kick_ev(3))) return st;
  CK(cudaGetLastError());
  return MERC_OK;
}
constexpr int kKernelsPerStep = 8;

int build_graph(merc_ctx* ctx, int steps) {
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  if (ctx->time_kicks) {
    size_t need = 4 * (size_t)steps;
    while (ctx->kick_ev.size() < need) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->kick_ev.push_back(e);
    }
  }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < steps; k++) {
    int st = enqueue_step(ctx, ctx->time_kicks, k);
    if (st) {
      cudaStreamEndCapture(ctx->stream, &g);
      return st;
    }
  }
  CK(cudaStreamEndCapture(ctx->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&ctx->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  ctx->graph_steps = steps;
  return MERC_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void merc_default_params(merc_params* p) {
  p->dt = 0.8219;
  p->softening2 = 1e-8;
  p->hill_factor = 1.0;
  p->kepler_tol = 1e-13;
  p->eject_r = 0.0;
  p->kepler_iters = 8;
  p->bs_rows = 3;
  p->compat_block = 0;
  p->drift = MERC_DRIFT_ELEMENTS;
  p->kepler_max_iter = 30;
  p->warm_start = MERC_WARM_PLAIN;
}

int merc_create(int device, const merc_params* p, merc_ctx** out) {
  if (!out) return MERC_ERR_CONFIG;
  *out = nullptr;
  merc_ctx* ctx = new merc_ctx();
  ctx->device = device;
  if (p) {
    int st = check_params(ctx, p);
    if (st) {
      delete ctx;
      return st;
    }
    ctx->p = *p;
  } else {
    merc_default_params(&ctx->p);
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e != cudaSuccess) {
    delete ctx;
    return MERC_ERR_CUDA;
  }
  *out = ctx;
  return MERC_OK;
}

int merc_destroy(merc_ctx* ctx) {
  if (!ctx) return MERC_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  for (cudaEvent_t e : ctx->kick_ev) cudaEventDestroy(e);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MERC_OK;
}

const char* merc_last_error(const merc_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int merc_set_params(merc_ctx* ctx, const merc_params* p) {
  if (!ctx || !p) return MERC_ERR_CONFIG;
  int st = check_params(ctx, p);
  if (st) return st;
  ctx->p = *p;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
    ctx->graph_steps = 0;
  }
  if (ctx->loaded) {
    CK(cudaSetDevice(ctx->device));
    return compute_rc(ctx);  // r_crit depends on hill_factor
  }
  return MERC_OK;
}

int merc_load_elements(merc_ctx* ctx, int32_t n_systems, const int64_t* body_offset, const int32_t* n_massive,
                       const double* mass, const double* elements) {
  if (!ctx) return MERC_ERR_CONFIG;
  int st = validate_layout(ctx, n_systems, body_offset, n_massive, mass);
  if (st) return st;
  if (!elements) return fail(ctx, MERC_ERR_CONFIG, "elements is NULL");
  CK(cudaSetDevice(ctx->device));
  if ((st = alloc_state(ctx, n_systems, body_offset, n_massive, mass))) return st;
  const int n = ctx->D.n;
  double* d_el = nullptr;
  if ((st = dalloc(ctx, &d_el, 6 * (size_t)n))) return st;
  CK(cudaMemcpyAsync(d_el, elements, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, ctx->stream));
  k_from_elements<<<blocks_for(n), kThreads, 0, ctx->stream>>>(ctx->D, d_el, ctx->p.kepler_iters);
  ctx->launches++;
  CK(cudaGetLastError());
  if ((st = dh_convert(ctx, false))) return st;
  if ((st = compute_rc(ctx))) return st;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->loaded = true;
  return MERC_OK;
}

int merc_load_state(merc_ctx* ctx, int32_t n_systems, const int64_t* body_offset, const int32_t* n_massive,
                    const double* mass, const double* pos, const double* vel, const double* a_lag) {
  if (!ctx) return MERC_ERR_CONFIG;
  int st = validate_layout(ctx, n_systems, body_offset, n_massive, mass);
  if (st) return st;
  if (!pos || !vel) return fail(ctx, MERC_ERR_CONFIG, "pos or vel is NULL");
  CK(cudaSetDevice(ctx->device));
  if ((st = alloc_state(ctx, n_systems, body_offset, n_massive, mass))) return st;
  const int n = ctx->D.n;
  CK(cudaMemcpyAsync(ctx->D.x, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->D.v, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  if (a_lag) {
    CK(cudaMemcpyAsync(ctx->D.alag, a_lag, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    // a of the current state: elements of the heliocentric state
    double* d_el = nullptr;
    if ((st = dalloc(ctx, &d_el, 6 * (size_t)n))) return st;
    if ((st = dh_convert(ctx, true))) return st;
    k_to_elements<<<blocks_for(n), kThreads, 0, ctx->stream>>>(ctx->D, d_el);
    ctx->launches++;
    CK(cudaMemcpyAsync(ctx->D.alag, d_el + 5 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    if ((st = dh_convert(ctx, false))) return st;
  }
  if ((st = compute_rc(ctx))) return st;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->loaded = true;
  return MERC_OK;
}

int merc_step(merc_ctx* ctx, int64_t n_steps) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_step before a load");
  if (n_steps < 0) return fail(ctx, MERC_ERR_CONFIG, "n_steps < 0");
  if (n_steps == 0) return MERC_OK;
  CK(cudaSetDevice(ctx->device));
  const int G = 8;
  if (!ctx->graph || ctx->graph_steps != G) {
    int st = build_graph(ctx, G);
    if (st) return st;
  }
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  int64_t full = n_steps / G, rest = n_steps % G;
  for (int64_t k = 0; k < full; k++) {
    CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    ctx->launches += (int64_t)G * kKernelsPerStep;
  }
  for (int64_t k = 0; k < rest; k++) {
    int st = enqueue_step(ctx, false, 0);
    if (st) return st;
    ctx->launches += kKernelsPerStep;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->last_ms = ms;
  ctx->steps_done += n_steps;
  return MERC_OK;
}

int merc_roundtrip(merc_ctx* ctx) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_roundtrip before a load");
  CK(cudaSetDevice(ctx->device));
  int st;
  const int n = ctx->D.n;
  if ((st = dh_convert(ctx, true))) return st;
  double* tmp = nullptr;  // 6 element rows
  if ((st = dalloc(ctx, &tmp, 6 * (size_t)n))) return st;
  k_to_elements<<<blocks_for(n), kThreads, 0, ctx->stream>>>(ctx->D, tmp);
  k_from_elements<<<blocks_for(n), kThreads, 0, ctx->stream>>>(ctx->D, tmp, ctx->p.kepler_iters);
  ctx->launches += 2;
  CK(cudaGetLastError());
  if ((st = dh_convert(ctx, false))) return st;
  if ((st = compute_rc(ctx))) return st;
  CK(cudaStreamSynchronize(ctx->stream));
  // release the temporary
  cudaFree(tmp);
  ctx->allocs.pop_back();
  return MERC_OK;
}

int merc_get_state(merc_ctx* ctx, double* pos, double* vel, uint32_t* flags) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_get_state before a load");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->D.n;
  if (pos) CK(cudaMemcpyAsync(pos, ctx->D.x, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (vel) CK(cudaMemcpyAsync(vel, ctx->D.v, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (flags) CK(cudaMemcpyAsync(flags, ctx->D.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MERC_OK;
}

int merc_get_a_lag(merc_ctx* ctx, double* a_lag) {
  if (!ctx || !a_lag) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_get_a_lag before a load");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(a_lag, ctx->D.alag, sizeof(double) * ctx->D.n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MERC_OK;
}

int merc_get_elements(merc_ctx* ctx, double* elements) {
  if (!ctx || !elements) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_get_elements before a load");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->D.n;
  int st;
  double* tmp = nullptr;
  if ((st = dalloc(ctx, &tmp, 6 * (size_t)n))) return st;
  // elements of the heliocentric state: reverse DH on a copy of v
  CK(cudaMemcpyAsync(ctx->D.vo, ctx->D.v, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, ctx->stream));
  if ((st = dh_convert(ctx, true))) return st;
  k_to_elements<<<blocks_for(n), kThreads, 0, ctx->stream>>>(ctx->D, tmp);
  ctx->launches++;
  CK(cudaMemcpyAsync(ctx->D.v, ctx->D.vo, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaMemcpyAsync(elements, tmp, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(tmp);
  ctx->allocs.pop_back();
  return MERC_OK;
}

int merc_get_stats(merc_ctx* ctx, merc_stats* out) {
  if (!ctx || !out) return MERC_ERR_CONFIG;
  memset(out, 0, sizeof *out);
  out->steps_done = ctx->steps_done;
  out->n_bodies = ctx->D.n;
  out->n_systems = ctx->D.nsys;
  out->last_step_ms = ctx->last_ms;
  if (ctx->loaded) {
    CK(cudaSetDevice(ctx->device));
    unsigned long long c[4];
    CK(cudaMemcpyAsync(c, ctx->D.counters, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out->ce_body_steps = (int64_t)c[0];
    out->kepler_iterations = (int64_t)c[1];
    out->kepler_solves = (int64_t)c[2];
    out->kepler_nonconverged = (int64_t)c[3];
  }
  return MERC_OK;
}

int merc_energy(merc_ctx* ctx, double* energy) {
  if (!ctx || !energy) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_energy before a load");
  CK(cudaSetDevice(ctx->device));
  double* tmp = nullptr;
  int st;
  if ((st = dalloc(ctx, &tmp, ctx->D.nsys))) return st;
  k_energy<<<ctx->D.nsys, kThreads, 0, ctx->stream>>>(ctx->D, tmp);
  ctx->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(energy, tmp, sizeof(double) * ctx->D.nsys, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(tmp);
  ctx->allocs.pop_back();
  return MERC_OK;
}

int64_t merc_launch_count(const merc_ctx* ctx) { return ctx ? ctx->launches : 0; }

// ---- diagnostics (merc_diag.h) ----
int merc_diag_math(int device, int fn, int64_t n, const double* x, const double* y, double* out) {
  merc_ctx* ctx = nullptr;
  if (n <= 0 || !x || !out) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  double *dx = nullptr, *dy = nullptr, *dout = nullptr;
  CK(cudaMalloc(&dx, n * sizeof(double)));
  CK(cudaMalloc(&dy, n * sizeof(double)));
  CK(cudaMalloc(&dout, n * sizeof(double)));
  CK(cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dy, y ? y : x, n * sizeof(double), cudaMemcpyHostToDevice));
  k_mm_eval<<<(unsigned)((n + 255) / 256), 256>>>(fn, (int)n, dx, dy, dout);
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dout);
  return MERC_OK;
}

int merc_diag_fp64_peak(int device, double* tflops) {
  merc_ctx* ctx = nullptr;
  if (!tflops) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 4, tpb = 256, iters = 20000;
  double* d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * blocks * tpb));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  k_dfma_probe<<<blocks, tpb>>>(d, 200, 1.0000001, 1e-9);
  CK(cudaDeviceSynchronize());
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    CK(cudaEventRecord(a));
    k_dfma_probe<<<blocks, tpb>>>(d, iters, 1.0000001, 1e-9);
    CK(cudaEventRecord(b));
    CK(cudaEventSynchronize(b));
    float ms;
    CK(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * tpb / (best * 1e-3) / 1e12;
  return MERC_OK;
}

int merc_diag_time_kicks(merc_ctx* ctx, int on) {
  if (!ctx) return MERC_ERR_CONFIG;
  ctx->time_kicks = on != 0;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
    ctx->graph_steps = 0;
  }
  return MERC_OK;
}

int merc_diag_kick_ms(merc_ctx* ctx, double* avg_ms, int32_t* n_launches) {
  if (!ctx || !avg_ms) return MERC_ERR_CONFIG;
  if (!ctx->time_kicks || ctx->graph_steps == 0) return fail(ctx, MERC_ERR_STATE, "kick timing is off");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  int cnt = 0;
  for (int k = 0; k < ctx->graph_steps; k++) {
    for (int h = 0; h < 2; h++) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->kick_ev[4 * k + 2 * h], ctx->kick_ev[4 * k + 2 * h + 1]));
      sum += ms;
      cnt++;
    }
  }
  *avg_ms = sum / cnt;
  if (n_launches) *n_launches = cnt;
  return MERC_OK;
}

}  // extern "C"
