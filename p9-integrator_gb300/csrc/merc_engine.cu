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
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/merc.h"
#include "../../include/merc_diag.h"
#include "merc_device.cuh"
#include "merc_fast.cuh"

using namespace merc;

#include "merc_kernels.cuh"

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
  unsigned char* d_big = nullptr;
  int* d_nchunk = nullptr;
  Work* d_work = nullptr;     // all targets of the big systems
  Work* d_work_tp = nullptr;  // test-particle targets of the big systems
  SymTask* d_sym = nullptr;   // massive block pairs of the big systems
  long long* d_sym_base = nullptr;
  int* d_big_ids = nullptr;
  int n_work = 0, n_work_tp = 0, n_sym = 0, n_big = 0, max_big_nm = 0;
  bool has_small = false, has_big = false, any_multi = false;
  std::vector<void*> allocs;
  std::vector<int> h_off, h_nm;
  bool loaded = false;
  int rc_cur = 0;  // buffer holding r_crit for the next first kick
  cudaGraphExec_t graph = nullptr;  // kGraphSteps steps
  cudaGraphExec_t graph1 = nullptr;  // one step
  int graph_steps = 0;
  int last_graph_steps = 0;  // steps of the graph replayed last
  double* flush_buf = nullptr;
  size_t flush_bytes = 0;
  int enc_blocks = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> kick_ev;  // start/end pairs recorded around kicks inside the graph
  bool time_kicks = false;
  int64_t steps_done = 0;
  int64_t launches = 0;
  int kernels_per_step = 0;
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
  if (p->softening2 > 1.0) return fail(ctx, MERC_ERR_CONFIG, "softening2 > 1 AU^2 is not supported");
  if (p->kepler_max_iter < 1 || p->kepler_max_iter > 1000)
    return fail(ctx, MERC_ERR_CONFIG, "kepler_max_iter out of 1..1000");
  if (p->warm_start != MERC_WARM_PLAIN && p->warm_start != MERC_WARM_MLP)
    return fail(ctx, MERC_ERR_CONFIG, "unknown warm_start %d", p->warm_start);
  return MERC_OK;
}

void drop_graphs(merc_ctx* ctx) {
  ctx->last_graph_steps = 0;
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->graph1) cudaGraphExecDestroy(ctx->graph1);
  ctx->graph = nullptr;
  ctx->graph1 = nullptr;
  ctx->graph_steps = 0;
}

void free_all(merc_ctx* ctx) {
  drop_graphs(ctx);
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
  // classification: systems with more than kSmallNm sources use the tiled
  // kernels; their work items split targets into kTile tiles and sources
  // into chunks so that about four blocks per SM are in flight
  int dev_sms = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  dev_sms = std::max(1, dev_sms);
  std::vector<unsigned char> big(n_systems, 0);
  std::vector<int> nchunk(n_systems, 0), big_ids;
  std::vector<Work> work;
  int64_t total_tiles = 0;
  for (int s = 0; s < n_systems; s++) {
    if (nm[s] > kSmallNm) {
      big[s] = 1;
      big_ids.push_back(s);
      total_tiles += (off[s + 1] - off[s] + kTile - 1) / kTile;
    }
  }
  const int64_t target_blocks = 4 * (int64_t)dev_sms;
  int max_chunks = 1;
  std::vector<Work> work_tp;
  std::vector<SymTask> sym;
  std::vector<long long> sym_base(n_systems, -1);
  long long sym_total = 0;
  ctx->max_big_nm = 0;
  for (int s : big_ids) {
    int ns = (int)(off[s + 1] - off[s]);
    int64_t want = (target_blocks + total_tiles - 1) / std::max<int64_t>(total_tiles, 1);
    int C = (int)std::max<int64_t>(1, std::min<int64_t>(want, (nm[s] + 15) / 16));
    nchunk[s] = C;
    max_chunks = std::max(max_chunks, C);
    ctx->max_big_nm = std::max(ctx->max_big_nm, (int)nm[s]);
    for (int t0 = 0; t0 < ns; t0 += kTile)
      for (int c = 0; c < C; c++) {
        Work w;
        w.sys = s;
        w.t0 = (int)off[s] + t0;
        w.c0 = (int)((int64_t)c * nm[s] / C);
        w.c1 = (int)((int64_t)(c + 1) * nm[s] / C);
        w.chunk = c;
        work.push_back(w);
      }
    for (int t0 = nm[s]; t0 < ns; t0 += kTile)
      for (int c = 0; c < C; c++) {
        Work w;
        w.sys = s;
        w.t0 = (int)off[s] + t0;
        w.c0 = (int)((int64_t)c * nm[s] / C);
        w.c1 = (int)((int64_t)(c + 1) * nm[s] / C);
        w.chunk = c;
        work_tp.push_back(w);
      }
    const int NB = (nm[s] + 31) / 32;
    for (int I = 0; I < NB; I++)
      for (int J = I; J < NB; J++) sym.push_back(SymTask{s, I, J});
    sym_base[s] = sym_total;
    sym_total += (long long)NB * 3 * nm[s];
  }
  ctx->n_work_tp = (int)work_tp.size();
  ctx->n_sym = (int)sym.size();
  ctx->n_work = (int)work.size();
  ctx->n_big = (int)big_ids.size();
  ctx->has_big = !big_ids.empty();
  ctx->has_small = (int)big_ids.size() < n_systems;
  ctx->any_multi = max_chunks > 1;
  Dev& D = ctx->D;
  D.n = n;
  D.nsys = n_systems;
  int st;
  if ((st = dalloc(ctx, &ctx->d_big, n_systems)) || (st = dalloc(ctx, &ctx->d_nchunk, n_systems)) ||
      (st = dalloc(ctx, &ctx->d_work, std::max(1, ctx->n_work))) ||
      (st = dalloc(ctx, &ctx->d_big_ids, std::max(1, ctx->n_big))) ||
      (st = dalloc(ctx, &D.part, ctx->any_multi ? (size_t)max_chunks * 3 * n : 1)) ||
      (st = dalloc(ctx, &D.ce_list_big, n)) || (st = dalloc(ctx, &ctx->d_work_tp, std::max(1, ctx->n_work_tp))) ||
      (st = dalloc(ctx, &ctx->d_sym, std::max(1, ctx->n_sym))) ||
      (st = dalloc(ctx, &ctx->d_sym_base, n_systems)) || (st = dalloc(ctx, &D.part_sym, std::max<long long>(1, sym_total))))
    return st;
  if ((st = dalloc(ctx, &ctx->d_off, n_systems + 1)) || (st = dalloc(ctx, &ctx->d_nm, n_systems)) ||
      (st = dalloc(ctx, &ctx->d_sys, n)) || (st = dalloc(ctx, &ctx->d_m, n)) || (st = dalloc(ctx, &D.x, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.v, 3 * (size_t)n)) || (st = dalloc(ctx, &D.xo, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.vo, 3 * (size_t)n)) || (st = dalloc(ctx, &D.alag, n)) || (st = dalloc(ctx, &D.flags, n)) ||
      (st = dalloc(ctx, &D.ce, n)) || (st = dalloc(ctx, &D.rc[0], 4 * (size_t)n)) ||
      (st = dalloc(ctx, &D.rc[1], 4 * (size_t)n)) || (st = dalloc(ctx, &D.P, 3 * (size_t)n_systems)) ||
      (st = dalloc(ctx, &D.ce_list, n)) || (st = dalloc(ctx, &D.ce_count, 2)) || (st = dalloc(ctx, &D.counters, 4)))
    return st;
  D.off = ctx->d_off;
  D.nm = ctx->d_nm;
  D.sys = ctx->d_sys;
  D.m = ctx->d_m;
  D.big = ctx->d_big;
  D.nchunk = ctx->d_nchunk;
  D.sym_base = ctx->d_sym_base;
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_off, ctx->h_off.data(), sizeof(int) * (n_systems + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_nm, nm, sizeof(int) * n_systems, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_sys, sys.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_big, big.data(), n_systems, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_nchunk, nchunk.data(), sizeof(int) * n_systems, cudaMemcpyHostToDevice, s));
  if (ctx->n_work)
    CK(cudaMemcpyAsync(ctx->d_work, work.data(), sizeof(Work) * ctx->n_work, cudaMemcpyHostToDevice, s));
  if (ctx->n_big)
    CK(cudaMemcpyAsync(ctx->d_big_ids, big_ids.data(), sizeof(int) * ctx->n_big, cudaMemcpyHostToDevice, s));
  if (ctx->n_work_tp)
    CK(cudaMemcpyAsync(ctx->d_work_tp, work_tp.data(), sizeof(Work) * ctx->n_work_tp, cudaMemcpyHostToDevice, s));
  if (ctx->n_sym) CK(cudaMemcpyAsync(ctx->d_sym, sym.data(), sizeof(SymTask) * ctx->n_sym, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_sym_base, sym_base.data(), sizeof(long long) * n_systems, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(D.flags, 0, sizeof(uint32_t) * n, s));
  CK(cudaMemsetAsync(D.ce, 0, n, s));
  CK(cudaMemsetAsync(D.counters, 0, sizeof(unsigned long long) * 4, s));
  CK(cudaMemsetAsync(D.rc[0], 0, sizeof(double) * 4 * n, s));
  CK(cudaMemsetAsync(D.rc[1], 0, sizeof(double) * 4 * n, s));
  CK(cudaStreamSynchronize(s));  // the host vectors above are temporaries
  ctx->enc_blocks = dev_sms * 4;
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

// Enqueue one step on the stream (also used while capturing the graph);
// returns the number of kernels it launched through *kernels.
int enqueue_step(merc_ctx* ctx, bool record_kick_events, int step_in_graph, int* kernels) {
  Dev& D = ctx->D;
  const merc_params& p = ctx->p;
  cudaStream_t s = ctx->stream;
  const double hdt = 0.5 * p.dt;
  const unsigned nb = blocks_for(D.n), sb = blocks_for(D.nsys);
  const double ej2 = p.eject_r > 0 ? p.eject_r * p.eject_r : 0.0;
  double* rcA = D.rc[ctx->rc_cur];
  double* rcB = D.rc[ctx->rc_cur ^ 1];
  int nk = 0;
  auto kick_ev = [&](int k) {
    if (record_kick_events)
      CK(cudaEventRecordWithFlags(ctx->kick_ev[4 * (size_t)step_in_graph + k], s, cudaEventRecordExternal));
    return MERC_OK;
  };
  int st;
  if (p.drift == MERC_DRIFT_ELEMENTS) {
    // exact path: the reference operation order for every system
    if ((st = kick_ev(0))) return st;
    k_kick<<<nb, kThreads, 0, s>>>(D, rcA, nullptr, hdt, p.softening2, p.compat_block, p.hill_factor, ej2, 0);
    if ((st = kick_ev(1))) return st;
    k_momentum<<<sb, kThreads, 0, s>>>(D, D.v, 0);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt, p.hill_factor);
    CK(cudaMemsetAsync(D.ce_count, 0, 2 * sizeof(int), s));
    k_drift_elements<<<nb, kThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.kepler_iters);
    k_encounter_elements<<<ctx->enc_blocks, 64, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows, p.softening2);
    k_momentum<<<sb, kThreads, 0, s>>>(D, D.vo, 0);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt, p.hill_factor);
    if ((st = kick_ev(2))) return st;
    k_kick<<<nb, kThreads, 0, s>>>(D, rcB, rcA, hdt, p.softening2, p.compat_block, p.hill_factor, ej2, 1);
    if ((st = kick_ev(3))) return st;
    nk = 8;
  } else {
    // the symmetric pair kernels assume a massive body excludes exactly itself
    const bool use_sym = p.compat_block == 0 || p.compat_block >= ctx->max_big_nm;
    auto kick = [&](const double* rc_in, double* rc_out, int last, int ev) {
      int st2;
      if ((st2 = kick_ev(ev))) return st2;
      if (ctx->has_small) {
        k_kick_small<<<nb, kThreads, 0, s>>>(D, rc_in, rc_out, hdt, p.softening2, p.compat_block, p.hill_factor,
                                             ej2, last);
        nk++;
      }
      if (ctx->has_big && use_sym) {
        // massive targets: symmetric block pairs; test particles: tiled
        k_sym<true><<<ctx->n_sym, 32, 0, s>>>(D, ctx->d_sym, ctx->n_sym, rc_in, p.softening2);
        nk++;
        if (ctx->n_work_tp) {
          k_kick_tiled<<<ctx->n_work_tp, kTile, 0, s>>>(D, ctx->d_work_tp, rc_in, rc_out, hdt, p.softening2,
                                                        p.compat_block, p.hill_factor, ej2, last);
          nk++;
        }
        k_kick_reduce_sym<<<nb, kThreads, 0, s>>>(D, rc_out, hdt, p.hill_factor, ej2, last);
        nk++;
      } else if (ctx->has_big) {
        k_kick_tiled<<<ctx->n_work, kTile, 0, s>>>(D, ctx->d_work, rc_in, rc_out, hdt, p.softening2, p.compat_block,
                                                   p.hill_factor, ej2, last);
        nk++;
        if (ctx->any_multi) {
          k_kick_reduce<<<nb, kThreads, 0, s>>>(D, rc_out, hdt, p.hill_factor, ej2, last);
          nk++;
        }
      }
      return kick_ev(ev + 1);
    };
    auto momentum = [&](const double* vsrc) {
      if (ctx->has_small) {
        k_momentum<<<sb, kThreads, 0, s>>>(D, vsrc, 1);
        nk++;
      }
      if (ctx->has_big) {
        k_momentum_big<<<ctx->n_big, kThreads, 0, s>>>(D, ctx->d_big_ids, vsrc);
        nk++;
      }
    };
    if ((st = kick(rcA, nullptr, 0, 0))) return st;
    momentum(D.v);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt, p.hill_factor);
    nk++;
    if (ctx->has_big) {
      CK(cudaMemsetAsync(D.ce, 0, D.n, s));
      if (use_sym) {
        k_sym<false><<<ctx->n_sym, 32, 0, s>>>(D, ctx->d_sym, ctx->n_sym, rcB, p.softening2);
        nk++;
        if (ctx->n_work_tp) {
          k_ce_tiled<<<ctx->n_work_tp, kTile, 0, s>>>(D, ctx->d_work_tp, rcB, p.compat_block);
          nk++;
        }
      } else {
        k_ce_tiled<<<ctx->n_work, kTile, 0, s>>>(D, ctx->d_work, rcB, p.compat_block);
        nk++;
      }
    }
    CK(cudaMemsetAsync(D.ce_count, 0, 2 * sizeof(int), s));
    k_drift_universal<<<nb, kThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.kepler_tol, p.kepler_max_iter);
    nk++;
    if (ctx->has_small) {
      k_encounter_small<<<ctx->enc_blocks, 64, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows, p.softening2);
      nk++;
    }
    if (ctx->has_big) {
      k_encounter_cluster<<<ctx->enc_blocks, kEncThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows,
                                                                   p.softening2);
      nk++;
    }
    momentum(D.vo);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt, p.hill_factor);
    nk++;
    if ((st = kick(rcB, rcA, 1, 2))) return st;
  }
  CK(cudaGetLastError());
  if (kernels) *kernels = nk;
  return MERC_OK;
}

// Capture `steps` steps; with timing on, kick events use slots first_slot..
int capture(merc_ctx* ctx, int steps, bool timed, int first_slot, cudaGraphExec_t* out) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < steps; k++) {
    int nk = 0;
    int st = enqueue_step(ctx, timed, first_slot + k, &nk);
    ctx->kernels_per_step = nk;
    if (st) {
      cudaStreamEndCapture(ctx->stream, &g);
      cudaGraphDestroy(g);
      return st;
    }
  }
  CK(cudaStreamEndCapture(ctx->stream, &g));
  cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  return MERC_OK;
}

constexpr int kGraphSteps = 8;

// The step graphs: kGraphSteps steps (kick events recorded when timing is on)
// and a single step.
int build_graphs(merc_ctx* ctx) {
  drop_graphs(ctx);
  if (ctx->time_kicks) {
    size_t need = 4 * (size_t)(kGraphSteps + 1);
    while (ctx->kick_ev.size() < need) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->kick_ev.push_back(e);
    }
  }
  int st;
  if ((st = capture(ctx, kGraphSteps, ctx->time_kicks, 0, &ctx->graph))) return st;
  if ((st = capture(ctx, 1, ctx->time_kicks, kGraphSteps, &ctx->graph1))) return st;
  ctx->graph_steps = kGraphSteps;
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
  if (ctx->flush_buf) cudaFree(ctx->flush_buf);
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
  drop_graphs(ctx);
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

int merc_set_state(merc_ctx* ctx, const double* pos, const double* vel, const double* a_lag) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_set_state before a load");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->D.n;
  if (pos) CK(cudaMemcpyAsync(ctx->D.x, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  if (vel) CK(cudaMemcpyAsync(ctx->D.v, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
  if (a_lag) CK(cudaMemcpyAsync(ctx->D.alag, a_lag, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int st = compute_rc(ctx);
  if (st) return st;
  CK(cudaStreamSynchronize(ctx->stream));
  return MERC_OK;
}

int merc_step(merc_ctx* ctx, int64_t n_steps) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_step before a load");
  if (n_steps < 0) return fail(ctx, MERC_ERR_CONFIG, "n_steps < 0");
  if (n_steps == 0) return MERC_OK;
  CK(cudaSetDevice(ctx->device));
  if (!ctx->graph) {
    int st = build_graphs(ctx);
    if (st) return st;
  }
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  const int64_t full = n_steps / kGraphSteps, rest = n_steps % kGraphSteps;
  for (int64_t k = 0; k < full; k++) CK(cudaGraphLaunch(ctx->graph, ctx->stream));
  for (int64_t k = 0; k < rest; k++) CK(cudaGraphLaunch(ctx->graph1, ctx->stream));
  ctx->last_graph_steps = rest > 0 ? 1 : kGraphSteps;
  ctx->launches += n_steps * ctx->kernels_per_step;
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

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free stepping (merc_step_static)
// ---------------------------------------------------------------------------
// Some callers cannot call cudaMalloc: a host application that hands this
// library device memory it manages itself (a memory pool or a framework
// allocator that must see every allocation), a runtime that forbids
// allocation after start-up, or a caller that must not add allocator traffic
// while it is recording CUDA work.  For them merc_step_static integrates one
// system held in caller-owned device buffers and takes every scratch buffer of
// the step (r_crit tables, the kick's per-chunk partial sums, drift outputs,
// encounter lists, per-step momentum) from this fixed device array.  Every GPU
// that loads the library holds it until the process exits.
constexpr size_t kStaticScratchBytes = (size_t)MERC_STATIC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device `dev`: in host
// code the symbol names a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, once per device, with that device current.
cudaError_t static_scratch_on(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_ptr[dev] = (unsigned char*)p;
  }
  *out = g_static_ptr[dev];
  return cudaSuccess;
}

// bump allocator over the static array (offsets only; nothing is allocated)
struct Carve {
  unsigned char* base;
  size_t used = 0;
  template <class T> T* take(size_t count) {
    size_t bytes = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~(size_t)255;
    T* p = base ? (T*)(base + used) : nullptr;
    used += bytes;
    return p;
  }
};

}  // namespace

extern "C" int merc_step_static(int device, const merc_params* p, int32_t n_bodies, int32_t n_massive, double* pos,
                                double* vel, const double* mass, uint32_t* flags, int64_t n_steps, void* stream) {
  merc_ctx* ctx = nullptr;  // errors are reported by status code only
  if (!p || !pos || !vel || !mass) return MERC_ERR_CONFIG;
  if (n_bodies <= 0 || n_massive < 0 || n_massive > n_bodies || n_steps < 0) return MERC_ERR_CONFIG;
  if (device < 0 || device >= kMaxDevices) return MERC_ERR_CONFIG;
  if (p->drift != MERC_DRIFT_UNIVERSAL || check_params(nullptr, p) != MERC_OK) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  sms = std::max(1, sms);
  const int n = n_bodies, nm = n_massive;
  const bool big = nm > kSmallNm;
  // chunks of the tiled kick, as in the context path
  int C = 1;
  std::vector<Work> work;
  if (big) {
    int64_t tiles = (n + kTile - 1) / kTile;
    int64_t want = (4 * (int64_t)sms + tiles - 1) / tiles;
    C = (int)std::max<int64_t>(1, std::min<int64_t>(want, (nm + 15) / 16));
  }
  // layout of the scratch; sizes checked before anything is launched
  Carve lay{nullptr};
  auto plan = [&](Carve& c, Dev& D, int** off, int** nmv, unsigned char** bigv, int** nch, Work** wk, int** ids,
                  uint32_t** fl) {
    *off = c.take<int>(2);
    *nmv = c.take<int>(1);
    *bigv = c.take<unsigned char>(1);
    *nch = c.take<int>(1);
    *ids = c.take<int>(1);
    *wk = c.take<Work>(big ? (size_t)((n + kTile - 1) / kTile) * C : 1);
    D.sys = c.take<int>(n);
    D.xo = c.take<double>(3 * (size_t)n);
    D.vo = c.take<double>(3 * (size_t)n);
    D.alag = c.take<double>(n);
    D.ce = c.take<unsigned char>(n);
    D.rc[0] = c.take<double>(4 * (size_t)n);
    D.rc[1] = c.take<double>(4 * (size_t)n);
    D.P = c.take<double>(3);
    D.part = c.take<double>(C > 1 ? (size_t)C * 3 * n : 1);
    D.ce_list = c.take<int>(n);
    D.ce_list_big = c.take<int>(n);
    D.ce_count = c.take<int>(2);
    D.counters = c.take<unsigned long long>(4);
    *fl = c.take<uint32_t>(n);
  };
  {
    Dev tmp;
    int *a, *b, *d, *f;
    unsigned char* e;
    Work* w;
    uint32_t* g;
    plan(lay, tmp, &a, &b, &e, &d, &w, &f, &g);
    if (lay.used > kStaticScratchBytes) return MERC_ERR_CONFIG;  // too many bodies for the static scratch
  }
  if (n_steps == 0) return MERC_OK;
  unsigned char* base = nullptr;
  CK(static_scratch_on(device, &base));
  Carve cv{base};
  Dev D;
  int *d_off, *d_nm, *d_nchunk, *d_ids;
  unsigned char* d_big;
  Work* d_work;
  uint32_t* d_flags_scratch;
  plan(cv, D, &d_off, &d_nm, &d_big, &d_nchunk, &d_work, &d_ids, &d_flags_scratch);
  D.n = n;
  D.nsys = 1;
  D.off = d_off;
  D.nm = d_nm;
  D.big = d_big;
  D.nchunk = d_nchunk;
  D.x = pos;
  D.v = vel;
  D.m = mass;
  D.flags = flags ? flags : d_flags_scratch;
  cudaStream_t s = (cudaStream_t)stream;
  if (big)
    for (int t0 = 0; t0 < n; t0 += kTile)
      for (int c = 0; c < C; c++) work.push_back(Work{0, t0, (int)((int64_t)c * nm / C), (int)((int64_t)(c + 1) * nm / C), c});
  const int h_off[2] = {0, n};
  const int h_nchunk = big ? C : 0, h_ids = 0;
  const unsigned char h_big = big ? 1 : 0;
  // the tables of this call, and every region that must start at zero
  CK(cudaMemcpyAsync(d_off, h_off, sizeof h_off, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_nm, &nm, sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_big, &h_big, 1, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_nchunk, &h_nchunk, sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_ids, &h_ids, sizeof(int), cudaMemcpyHostToDevice, s));
  if (big) CK(cudaMemcpyAsync(d_work, work.data(), sizeof(Work) * work.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync((void*)D.sys, 0, sizeof(int) * n, s));
  CK(cudaMemsetAsync(D.ce, 0, n, s));
  CK(cudaMemsetAsync(D.counters, 0, 4 * sizeof(unsigned long long), s));
  if (!flags) CK(cudaMemsetAsync(d_flags_scratch, 0, sizeof(uint32_t) * n, s));
  // the kernel sequence of the universal path, on the caller's stream
  const double hdt = 0.5 * p->dt;
  const double ej2 = p->eject_r > 0 ? p->eject_r * p->eject_r : 0.0;
  const unsigned nb = blocks_for(n);
  double *rcA = D.rc[0], *rcB = D.rc[1];
  k_rc<<<nb, kThreads, 0, s>>>(D, rcA, p->hill_factor);
  auto kick = [&](const double* rc_in, double* rc_out, int last) {
    if (!big) {
      k_kick_small<<<nb, kThreads, 0, s>>>(D, rc_in, rc_out, hdt, p->softening2, p->compat_block, p->hill_factor,
                                           ej2, last);
    } else {
      k_kick_tiled<<<(unsigned)work.size(), kTile, 0, s>>>(D, d_work, rc_in, rc_out, hdt, p->softening2,
                                                          p->compat_block, p->hill_factor, ej2, last);
      if (C > 1) k_kick_reduce<<<nb, kThreads, 0, s>>>(D, rc_out, hdt, p->hill_factor, ej2, last);
    }
  };
  auto momentum = [&](const double* vsrc) {
    if (!big)
      k_momentum<<<1, kThreads, 0, s>>>(D, vsrc, 1);
    else
      k_momentum_big<<<1, kThreads, 0, s>>>(D, d_ids, vsrc);
  };
  for (int64_t k = 0; k < n_steps; k++) {
    kick(rcA, nullptr, 0);
    momentum(D.v);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt, p->hill_factor);
    if (big) {
      CK(cudaMemsetAsync(D.ce, 0, n, s));
      k_ce_tiled<<<(unsigned)work.size(), kTile, 0, s>>>(D, d_work, rcB, p->compat_block);
    }
    CK(cudaMemsetAsync(D.ce_count, 0, 2 * sizeof(int), s));
    k_drift_universal<<<nb, kThreads, 0, s>>>(D, rcB, p->dt, p->compat_block, p->kepler_tol, p->kepler_max_iter);
    if (!big)
      k_encounter_small<<<sms * 4, 64, 0, s>>>(D, rcB, p->dt, p->compat_block, p->bs_rows, p->softening2);
    else
      k_encounter_big<<<sms * 4, kEncThreads, 0, s>>>(D, rcB, p->dt, p->compat_block, p->bs_rows, p->softening2);
    momentum(D.vo);
    k_jump<<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt, p->hill_factor);
    kick(rcB, rcA, 1);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(s));
  return MERC_OK;
}

extern "C" {

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

int merc_diag_flush_l2(merc_ctx* ctx, int64_t bytes) {
  if (!ctx || bytes <= 0) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(ctx->device));
  if (ctx->flush_bytes < (size_t)bytes) {
    if (ctx->flush_buf) cudaFree(ctx->flush_buf);
    ctx->flush_buf = nullptr;
    ctx->flush_bytes = 0;
    CK(cudaMalloc(&ctx->flush_buf, (size_t)bytes));
    ctx->flush_bytes = (size_t)bytes;
  }
  CK(cudaMemsetAsync(ctx->flush_buf, (int)(ctx->steps_done & 0xff), (size_t)bytes, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MERC_OK;
}

int merc_diag_time_kicks(merc_ctx* ctx, int on) {
  if (!ctx) return MERC_ERR_CONFIG;
  ctx->time_kicks = on != 0;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_diag_kick_ms(merc_ctx* ctx, double* avg_ms, int32_t* n_launches) {
  if (!ctx || !avg_ms) return MERC_ERR_CONFIG;
  if (!ctx->time_kicks || ctx->graph_steps == 0 || ctx->last_graph_steps == 0)
    return fail(ctx, MERC_ERR_STATE, "kick timing is off or no step ran since it was turned on");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  int cnt = 0;
  const int first = ctx->last_graph_steps == 1 ? kGraphSteps : 0;
  const int steps = ctx->last_graph_steps == 1 ? 1 : kGraphSteps;
  for (int k = first; k < first + steps; k++) {
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
