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
#include <cmath>
#include <cstdarg>
#include <array>
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

#include "merc_mlp.cuh"
#include "merc_kernels.cuh"
#include "merc_sweep.cuh"
#include "merc_collide.cuh"

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
  int2* d_exact_groups = nullptr;  // element path: (first body, count) of each block of the exact kick
  int n_exact_groups = 0;
  int n_work = 0, n_work_tp = 0, n_sym = 0, n_big = 0, max_big_nm = 0;
  bool has_small = false, has_big = false, any_multi = false;
  std::vector<void*> allocs;
  std::vector<int> h_off, h_nm;
  bool loaded = false;
  int rc_cur = 0;  // buffer holding r_crit for the next first kick
  // step graphs by kind (GraphKind): executable, kernels per replay
  cudaGraphExec_t graphs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int graph_kernels[5] = {0, 0, 0, 0, 0};
  unsigned last_kinds = 0;  // bit k: graphs of kind k replayed by the last merc_step
  int graph_steps = 0;
  int last_graph_steps = 0;  // steps of the graph replayed last
  double* flush_buf = nullptr;
  size_t flush_bytes = 0;
  int enc_blocks = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> kick_ev;  // start/end pairs recorded around kicks inside the graph
  std::vector<char> kick_ev_used;    // slots recorded by the captured graphs
  bool time_kicks = false;
  std::vector<cudaEvent_t> enc_ev;  // start/end pairs around the big systems' encounter sub-step
  bool time_encounter = false;
  bool pdl = true;  // programmatic dependent launches inside the step graphs
  int smem_optin = 0;  // largest dynamic shared memory per block (opt-in)
  int sms = 0;         // multiprocessors of the device
  int64_t steps_done = 0;
  int64_t launches = 0;

  // persistent small-system path: size order, work counter, tuned block size
  std::vector<int> h_order;  // systems, largest first
  SweepItem* d_items = nullptr;
  int items_cap = 0, n_items = 0, items_threads = 0, items_grid = 0;  // item list and what it was built for
  int* d_queue = nullptr;
  int* d_moff = nullptr;           // per system: first staging slot of its massive bodies
  int* d_mbody = nullptr;          // staging slot -> global body
  double* d_stage = nullptr;       // 6 per massive body
  uint32_t* d_stage_f = nullptr;   // 1 per massive body
  int n_mass = 0;
  int nmax_sys = 0;
  int sweep_threads = 0;   // 0: not tuned yet
  int sweep_grid = 0;
  unsigned long long* d_tune_counters = nullptr;
  uint32_t* d_tune_flags = nullptr;
  // learned warm start: parameter blob, drift log, training state
  float* d_mlp = nullptr;
  bool mlp_ready = false;
  float* d_log = nullptr;
  unsigned long long* d_log_count = nullptr;
  long long log_cap = 0;
  double last_ms = 0.0;
  // physical collisions (merc_set_radii): buffers allocated with the state
  Collide col;
  bool collide_on = false;
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
  if (p->warm_start != MERC_WARM_PLAIN && p->warm_start != MERC_WARM_MLP && p->warm_start != MERC_WARM_SERIES)
    return fail(ctx, MERC_ERR_CONFIG, "unknown warm_start %d", p->warm_start);
  return MERC_OK;
}

void drop_graphs(merc_ctx* ctx) {
  ctx->last_graph_steps = 0;
  ctx->last_kinds = 0;
  for (auto& g : ctx->graphs) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  ctx->graph_steps = 0;
}

void free_all(merc_ctx* ctx) {
  drop_graphs(ctx);
  for (void* a : ctx->allocs) cudaFree(a);
  ctx->allocs.clear();
  ctx->D = Dev();
  ctx->col = Collide();
  ctx->collide_on = false;
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
    // off-diagonal block pairs (full 32x32) first, the half-length diagonal
    // ones last: blocks start in index order, so the short tasks fill the tail
    const int NB = (nm[s] + 31) / 32;
    for (int I = 0; I < NB; I++)
      for (int J = I + 1; J < NB; J++) sym.push_back(SymTask{s, I, J});
    for (int I = 0; I < NB; I++) sym.push_back(SymTask{s, I, I});
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
  D.nm0 = n_systems == 1 ? nm[0] : 0;
  D.gate_words = std::max(1, ((D.nm0 + 31) / 32 + 63) / 64);
  const long long sym_set = std::max<long long>(3, sym_total);  // a multiple of 3 (NB * 3 * nm per system)
  int st;
  if ((st = dalloc(ctx, &ctx->d_big, n_systems)) || (st = dalloc(ctx, &ctx->d_nchunk, n_systems)) ||
      (st = dalloc(ctx, &ctx->d_work, std::max(1, ctx->n_work))) ||
      (st = dalloc(ctx, &ctx->d_big_ids, std::max(1, ctx->n_big))) ||
      (st = dalloc(ctx, &D.part, ctx->any_multi ? (size_t)max_chunks * 3 * n : 1)) ||
      (st = dalloc(ctx, &D.ce_list_big, n)) || (st = dalloc(ctx, &ctx->d_work_tp, std::max(1, ctx->n_work_tp))) ||
      (st = dalloc(ctx, &ctx->d_sym, std::max(1, ctx->n_sym))) ||
      (st = dalloc(ctx, &ctx->d_sym_base, n_systems)) ||
      (st = dalloc(ctx, &D.part_sym, 2 * (size_t)sym_set)) || (st = dalloc(ctx, &D.near_mask, 2 * (size_t)(sym_set / 3))) ||
      (st = dalloc(ctx, &D.gate, 1)) || (st = dalloc(ctx, &D.far_recomputes, 1)) ||
      (st = dalloc(ctx, &D.gate_blocks, (size_t)D.gate_words)) ||
      (st = dalloc(ctx, &D.far_acc, ctx->has_big ? 3 * (size_t)n : 1)))
    return st;
  {
    // encounter task kernel state (every body of a big system may be listed)
    const size_t ne = ctx->has_big ? (size_t)n : 1;
    if ((st = dalloc(ctx, &D.enc_q, kEncQ * ne)) || (st = dalloc(ctx, &D.enc_st, 27 * ne)) ||
        (st = dalloc(ctx, &D.enc_res, 18 * ne)) || (st = dalloc(ctx, &D.enc_cnt, 11 * ne)) ||
        (st = dalloc(ctx, &D.enc_head, 2)))
      return st;
    CK(cudaMemsetAsync(D.enc_cnt, 0, sizeof(int) * 11 * ne, ctx->stream));
    CK(cudaMemsetAsync(D.enc_head, 0, sizeof(int) * 2, ctx->stream));
  }
  D.sym_set = sym_set;
  CK(cudaMemsetAsync(D.gate, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(D.gate_blocks, 0, sizeof(unsigned long long) * (size_t)D.gate_words, ctx->stream));
  CK(cudaMemsetAsync(D.far_recomputes, 0, sizeof(unsigned long long), ctx->stream));
  if ((st = dalloc(ctx, &ctx->d_off, n_systems + 1)) || (st = dalloc(ctx, &ctx->d_nm, n_systems)) ||
      (st = dalloc(ctx, &ctx->d_sys, n)) || (st = dalloc(ctx, &ctx->d_m, n)) || (st = dalloc(ctx, &D.hc, n)) ||
      (st = dalloc(ctx, &D.x, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.v, 3 * (size_t)n)) || (st = dalloc(ctx, &D.xo, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.xf, 3 * (size_t)n)) ||
      (st = dalloc(ctx, &D.vo, 3 * (size_t)n)) || (st = dalloc(ctx, &D.alag, n)) || (st = dalloc(ctx, &D.flags, n)) ||
      (st = dalloc(ctx, &D.ce, ((size_t)n + 3) & ~(size_t)3)) || (st = dalloc(ctx, &D.rc[0], rc_table_doubles(n))) ||
      (st = dalloc(ctx, &D.rc[1], rc_table_doubles(n))) || (st = dalloc(ctx, &D.P, 3 * (size_t)n_systems)) ||
      (st = dalloc(ctx, &D.ce_list, n)) || (st = dalloc(ctx, &D.ce_count, 2)) || (st = dalloc(ctx, &D.counters, kNumCounters)))
    return st;
  {
    // systems by size, largest first: the persistent kernel's work order
    std::vector<int> order(n_systems);
    for (int q = 0; q < n_systems; q++) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return (off[a + 1] - off[a]) > (off[b + 1] - off[b]);
    });
    ctx->nmax_sys = n_systems ? (int)(off[order[0] + 1] - off[order[0]]) : 0;
    ctx->h_order = order;
    // staging slots of the massive bodies, and the item capacity (items of at
    // least 64 test particles, one or more per system)
    std::vector<int> moff(n_systems), mbody;
    int64_t tps = 0;
    for (int q = 0; q < n_systems; q++) {
      moff[q] = (int)mbody.size();
      for (int i = 0; i < nm[q]; i++) mbody.push_back((int)off[q] + i);
      tps += (off[q + 1] - off[q]) - nm[q];
    }
    ctx->n_mass = (int)mbody.size();
    ctx->items_cap = n_systems + (int)(tps / 64) + 1;
    ctx->n_items = ctx->items_threads = ctx->items_grid = 0;
    if ((st = dalloc(ctx, &ctx->d_items, ctx->items_cap)) || (st = dalloc(ctx, &ctx->d_queue, 1)) ||
        (st = dalloc(ctx, &ctx->d_moff, n_systems)) || (st = dalloc(ctx, &ctx->d_mbody, std::max(1, ctx->n_mass))) ||
        (st = dalloc(ctx, &ctx->d_stage, 6 * (size_t)std::max(1, ctx->n_mass))) ||
        (st = dalloc(ctx, &ctx->d_stage_f, std::max(1, ctx->n_mass))) ||
        (st = dalloc(ctx, &ctx->d_tune_counters, kNumCounters)) || (st = dalloc(ctx, &ctx->d_tune_flags, n)))
      return st;
    CK(cudaMemcpy(ctx->d_moff, moff.data(), sizeof(int) * n_systems, cudaMemcpyHostToDevice));
    if (ctx->n_mass)
      CK(cudaMemcpy(ctx->d_mbody, mbody.data(), sizeof(int) * ctx->n_mass, cudaMemcpyHostToDevice));
    ctx->sweep_threads = 0;
  }
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
  {
    // the element path's pipelined exact kick: G bodies of one big system per
    // block, G chosen so that there are about two blocks per SM
    int64_t nbig = 0;
    for (int sb : big_ids) nbig += off[sb + 1] - off[sb];
    // measured on the 2002-body disk (ms per step): G = 7 (286 blocks) 1.561,
    // 5 1.571, 9 1.685, 4 1.638; one body per one-warp block without the
    // pipeline 1.972, two 1.638
    const int64_t cover = 2 * (int64_t)dev_sms;
    const int G = (int)std::max<int64_t>(1, std::min<int64_t>(kPipeGroupMax, (nbig + cover - 1) / cover));
    std::vector<int2> groups;
    for (int sb : big_ids)
      for (int64_t j0 = off[sb]; j0 < off[sb + 1]; j0 += G)
        groups.push_back(make_int2((int)j0, (int)std::min<int64_t>(G, off[sb + 1] - j0)));
    ctx->n_exact_groups = (int)groups.size();
    if ((st = dalloc(ctx, &ctx->d_exact_groups, std::max<size_t>(1, groups.size())))) return st;
    if (!groups.empty())
      CK(cudaMemcpyAsync(ctx->d_exact_groups, groups.data(), sizeof(int2) * groups.size(), cudaMemcpyHostToDevice,
                         s));
    CK(cudaStreamSynchronize(s));  // `groups` is a temporary
  }
  if (ctx->n_work_tp)
    CK(cudaMemcpyAsync(ctx->d_work_tp, work_tp.data(), sizeof(Work) * ctx->n_work_tp, cudaMemcpyHostToDevice, s));
  if (ctx->n_sym) CK(cudaMemcpyAsync(ctx->d_sym, sym.data(), sizeof(SymTask) * ctx->n_sym, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->d_sym_base, sym_base.data(), sizeof(long long) * n_systems, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(D.flags, 0, sizeof(uint32_t) * n, s));
  CK(cudaMemsetAsync(D.ce, 0, n, s));
  CK(cudaMemsetAsync(D.counters, 0, sizeof(unsigned long long) * kNumCounters, s));
  CK(cudaMemsetAsync(D.rc[0], 0, sizeof(double) * rc_table_doubles(n), s));
  CK(cudaMemsetAsync(D.rc[1], 0, sizeof(double) * rc_table_doubles(n), s));
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

// initial guess of the universal drift for the parameters (the network's
// fallback outside its box is the plain guess)
// the guess of a solve the network does not serve (MERC_WARM_MLP outside its
// feature box) is the series guess
double guess_of(const merc_params& p) { return p.warm_start == MERC_WARM_PLAIN ? kGuessPlain : kGuessSeries; }

// Launch on the step stream.  With pdl (programmatic dependent launch) the
// kernel may be scheduled while its predecessor is still running; every kernel
// of the step waits for its predecessor in griddep_wait() before it touches
// memory, so only the launch latency overlaps.
template <typename... P, typename... A>
cudaError_t step_launch(bool pdl, cudaStream_t s, void (*k)(P...), dim3 grid, dim3 block, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// Enqueue one step on the stream (also used while capturing the graph);
// returns the number of kernels it launched through *kernels.
int enqueue_step(merc_ctx* ctx, bool record_kick_events, int step_in_graph, int* kernels, bool first_in_graph,
                 bool last_in_graph) {
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
    if (record_kick_events) {
      const size_t slot = 4 * (size_t)step_in_graph + k;
      CK(cudaEventRecordWithFlags(ctx->kick_ev[slot], s, cudaEventRecordExternal));
      ctx->kick_ev_used[slot] = 1;
    }
    return MERC_OK;
  };
  int st;
  if (p.drift == MERC_DRIFT_ELEMENTS) {
    // exact path: the reference operation order for every system
    // the bodies of big systems by one warp each (same bits, same order)
    const int bx = ctx->has_big ? 1 : 0;
    const unsigned nbx =
        (unsigned)std::min<int64_t>((D.n + kExactWarps - 1) / kExactWarps, (int64_t)ctx->sms * 16);
    // without small systems the small-system kernels have nothing to do
    const bool small = ctx->has_small || !bx;
    auto kick_exact_all = [&](const double* rc_in, double* rc_out, int last) {
      if (small)
        k_kick<<<nb, kThreads, 0, s>>>(D, rc_in, rc_out, hdt, p.softening2, p.compat_block, p.hill_factor, ej2,
                                       last, bx);
      if (bx)
        k_kick_big_exact_pipe<<<(unsigned)std::max(1, ctx->n_exact_groups), 32 * (1 + kPipeTermWarps), 0, s>>>(
            D, ctx->d_exact_groups, ctx->n_exact_groups, rc_in, rc_out, hdt, p.softening2, p.compat_block,
            p.hill_factor, ej2, last);
    };
    if ((st = kick_ev(0))) return st;
    kick_exact_all(rcA, nullptr, 0);
    if ((st = kick_ev(1))) return st;
    auto momentum_exact = [&](const double* vsrc) {
      if (small) k_momentum<<<sb, kThreads, 0, s>>>(D, vsrc, bx);
      if (bx)
        k_momentum_big_exact<<<(unsigned)((D.nsys + kExactWarps - 1) / kExactWarps), 32 * kExactWarps, 0, s>>>(
            D, vsrc);
    };
    momentum_exact(D.v);
    // the symmetric encounter test of the big systems (each unordered pair
    // once, the same exact decisions as k_ce_big_exact: 34 -> ~8 us on the
    // 2002-body disk) sets flags only, so this jump clears them first; with
    // the reference's local-index self test (compat_block), or with test
    // particles in big systems (the symmetric test covers massive pairs), the
    // warp-per-body test stays
    const bool sym_ce =
        bx && ctx->n_work_tp == 0 && (p.compat_block == 0 || p.compat_block >= ctx->max_big_nm);
    if (sym_ce)
      k_jump<false, true><<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt);
    else
      k_jump<false, false><<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt);
    CK(cudaMemsetAsync(D.ce_count, 0, 2 * sizeof(int), s));
    if (sym_ce && D.nsys == 1)
      k_sym<false, true><<<ctx->n_sym, 32 * kSymSplit, 0, s>>>(D, ctx->d_sym, ctx->n_sym, rcB, p.softening2, 1,
                                                               nullptr);
    else if (sym_ce)
      k_sym<false, false><<<ctx->n_sym, 32 * kSymSplit, 0, s>>>(D, ctx->d_sym, ctx->n_sym, rcB, p.softening2, 1,
                                                                nullptr);
    else if (bx)
      k_ce_big_exact<<<nbx, 32 * kExactWarps, 0, s>>>(D, rcB, p.compat_block);
    // big systems only: the encounter sub-step runs beside the drift (the
    // drift lets it launch at once and it waits for the drift before its
    // stores; the bodies they integrate are disjoint, the stores blend the
    // drift's result as the reference does)
    const bool beside = bx && !small && ctx->pdl;
    k_drift_elements<<<nb, kThreads, 0, s>>>(D, rcB, p.dt, p.compat_block, p.kepler_iters, bx, beside ? 1 : 0);
    if (small)
      k_encounter_elements<<<ctx->enc_blocks, 64, 0, s>>>(D, rcB, p.dt, p.compat_block, p.bs_rows, p.softening2,
                                                           bx);
    if (bx) {
      cudaError_t le = step_launch(beside, s, k_encounter_big_pipe, dim3((unsigned)(kExactEncBlocksPerSM * ctx->sms)),
                                   dim3((unsigned)(32 + kExactRowThreads * p.bs_rows)), D, (const double*)rcB,
                                   p.dt, p.compat_block, p.bs_rows, p.softening2, beside ? 1 : 0);
      if (le != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(le));
    }
    if (ctx->collide_on) {
      k_collide_find<<<ctx->sms * 4, 256, 0, s>>>(D, ctx->col);
      k_collide_resolve<<<1, 32, 0, s>>>(D, ctx->col, p.hill_factor);
      nk += 2;
    }
    momentum_exact(D.vo);
    k_jump<false, false><<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt);
    if ((st = kick_ev(2))) return st;
    kick_exact_all(rcB, rcA, 1);
    if ((st = kick_ev(3))) return st;
    nk += 3 + (small ? 5 : 0) + 6 * bx;  // jumps and drift; small-system kick, momentum, encounter; big systems
  } else {
    // programmatic dependent launches: a kernel may be scheduled while its
    // predecessor finishes; every kernel here waits for it (griddep_wait)
    // before touching memory
    cudaError_t lerr = cudaSuccess;
    auto launch = [&](auto k, auto grid, auto block, auto... args) {
      cudaError_t e = step_launch(ctx->pdl, s, k, dim3((unsigned)grid), dim3((unsigned)block), args...);
      if (e != cudaSuccess && lerr == cudaSuccess) lerr = e;
    };
    // the symmetric pair kernels assume a massive body excludes exactly itself
    const bool use_sym = p.compat_block == 0 || p.compat_block >= ctx->max_big_nm;
    // test particles of big systems: adjacent half kicks merged inside a graph
    const bool merge_tp = ctx->has_big && use_sym && ctx->n_work_tp > 0 && !ctx->any_multi;
    const unsigned nred = (unsigned)((kRedThreads * (int64_t)D.n + kThreads - 1) / kThreads);
    auto tp_kick = [&](const double* rc_in, double* rc_out, int last) {
      launch(k_kick_tiled, ctx->n_work_tp, kTile, D, ctx->d_work_tp, rc_in, rc_out, hdt, p.softening2,
             p.compat_block, p.hill_factor, ej2, last);
      nk++;
    };
    auto reduce = [&](const double* rc_in, const int* gate, double* rc_out, int last, int massive_only, int check,
                      int far_mode) {
      if (D.nsys == 1)
        launch(k_kick_reduce_sym<true>, nred, kThreads, D, rc_in, gate, rc_out, hdt, p.softening2, p.hill_factor,
               ej2, last, massive_only, check, far_mode);
      else
        launch(k_kick_reduce_sym<false>, nred, kThreads, D, rc_in, gate, rc_out, hdt, p.softening2, p.hill_factor,
               ej2, last, massive_only, check, far_mode);
      nk++;
    };
    // far-field pass of the massive bodies (timed as the kick kernel)
    auto far = [&](const double* rc_in, int set, const int* gate, int ev) {
      int st2;
      if (ev >= 0 && (st2 = kick_ev(ev))) return st2;
      // the gated pass (usually empty) in fewer blocks, each looping over tasks
      const int nfar = gate ? (ctx->n_sym + kSymGatedDiv - 1) / kSymGatedDiv : ctx->n_sym;
      if (D.nsys == 1)
        launch(k_sym<true, true>, nfar, 32 * kSymSplit, D, ctx->d_sym, ctx->n_sym, rc_in, p.softening2, set, gate);
      else
        launch(k_sym<true, false>, nfar, 32 * kSymSplit, D, ctx->d_sym, ctx->n_sym, rc_in, p.softening2, set, gate);
      nk++;
      return ev >= 0 ? kick_ev(ev + 1) : MERC_OK;
    };
    auto kick = [&](const double* rc_in, double* rc_out, int last, int ev) {
      int st2;
      if (ctx->has_small) {
        if (!(ctx->has_big && use_sym) && (st2 = kick_ev(ev))) return st2;
        launch(k_kick_small, nb, kThreads, D, rc_in, rc_out, hdt, p.softening2, p.compat_block, p.hill_factor,
               ej2, last);
        nk++;
      } else if (!use_sym || !ctx->has_big) {
        if ((st2 = kick_ev(ev))) return st2;
      }
      if (ctx->has_big && use_sym) {
        if (!last) {
          // inside a graph the first kick of a step was done by the merged
          // kick that ended the step before
          if (!first_in_graph) return MERC_OK;
          if ((st2 = far(rc_in, 0, nullptr, ev))) return st2;
          if (ctx->n_work_tp) tp_kick(rc_in, nullptr, 0);
          reduce(rc_in, nullptr, nullptr, 0, 0, 0, 0);
        } else if (last_in_graph) {
          if ((st2 = far(rc_in, 0, nullptr, ev))) return st2;
          if (ctx->n_work_tp) tp_kick(rc_in, rc_out, 1);
          reduce(rc_in, nullptr, rc_out, 1, 0, 0, 0);
        } else {
          // this kick and the next step's first kick (same positions): the
          // far field is summed once unless a far-field threshold moved
          // between them (the reduce sets the gate, the second pass runs)
          if ((st2 = far(rc_in, 0, nullptr, ev))) return st2;
          if (ctx->n_work_tp && !merge_tp) tp_kick(rc_in, rc_out, 1);
          reduce(rc_in, nullptr, rc_out, 1, merge_tp ? 1 : 0, 1, 1);
          if ((st2 = far(rc_out, 1, D.gate, -1))) return st2;
          if (merge_tp) {
            // rc_out holds the next step's radii (written by the reduce)
            launch(k_kick_tiled_merged, ctx->n_work_tp, kTile, D, ctx->d_work_tp, rc_in, rc_out, hdt,
                   p.softening2, p.compat_block, ej2);
            nk++;
          } else if (ctx->n_work_tp) {
            tp_kick(rc_out, nullptr, 0);
          }
          reduce(rc_out, D.gate, nullptr, 0, merge_tp ? 1 : 0, 0, 2);
        }
        return MERC_OK;
      } else if (ctx->has_big) {
        launch(k_kick_tiled, ctx->n_work, kTile, D, ctx->d_work, rc_in, rc_out, hdt, p.softening2, p.compat_block,
               p.hill_factor, ej2, last);
        nk++;
        if (ctx->any_multi) {
          launch(k_kick_reduce, nb, kThreads, D, rc_out, hdt, p.hill_factor, ej2, last);
          nk++;
        }
      }
      return kick_ev(ev + 1);
    };
    // momentum of the small systems (the big systems' is summed inside k_jump)
    auto momentum = [&](const double* vsrc) {
      if (ctx->has_small) {
        launch(k_momentum, sb, kThreads, D, vsrc, 1);
        nk++;
      }
    };
    if ((st = kick(rcA, nullptr, 0, 0))) return st;
    momentum(D.v);
    // also clears the encounter flags and list counts of this step
    const unsigned njb = (unsigned)((D.n + kJumpThreads - 1) / kJumpThreads);
    // one big system: the momentum is split over the blocks of a cluster
    const bool jump_cl = D.nsys == 1 && ctx->has_big;
    const unsigned njc = (njb + kJumpCluster - 1) / kJumpCluster * kJumpCluster;
    if (jump_cl)
      launch(k_jump_cluster<true>, njc, kJumpThreads, D, D.x, (const double*)nullptr, rcB, hdt);
    else
      launch(k_jump<true, true>, njb, kJumpThreads, D, D.x, nullptr, rcB, hdt);
    nk++;
    if (ctx->has_big) {
      if (use_sym) {
        if (D.nsys == 1)
          launch(k_sym<false, true>, ctx->n_sym, 32 * kSymSplit, D, ctx->d_sym, ctx->n_sym, rcB, p.softening2, 0,
                 nullptr);
        else
          launch(k_sym<false, false>, ctx->n_sym, 32 * kSymSplit, D, ctx->d_sym, ctx->n_sym, rcB, p.softening2, 0,
                 nullptr);
        nk++;
        if (ctx->n_work_tp) {
          launch(k_ce_tiled, ctx->n_work_tp, kTile, D, ctx->d_work_tp, rcB, p.compat_block);
          nk++;
        }
      } else {
        launch(k_ce_tiled, ctx->n_work, kTile, D, ctx->d_work, rcB, p.compat_block);
        nk++;
      }
    }
    const float* mlp = (p.warm_start == MERC_WARM_MLP && ctx->mlp_ready) ? ctx->d_mlp : nullptr;
    // one-warp blocks when kDriftThreads-blocks would leave SMs idle
    const int dthr = (D.n + kDriftThreads - 1) / kDriftThreads < ctx->sms ? 32 : kDriftThreads;
    // Without small systems the drift (bodies not in encounter) and the big
    // systems' encounter sub-step (the list built by the encounter test) are
    // independent, and they run side by side: the drift lets the next kernel
    // launch as soon as it starts (its own dependency wait has returned, so
    // the encounter test is complete), and the encounter task kernel skips
    // its dependency wait at the start and waits for the drift at its end, so
    // its completion still implies the drift's.  (Placed on a second graph
    // branch instead, the drift's blocks were not scheduled until the
    // encounter kernel's warps began to exit: a %globaltimer timeline showed
    // it starting 108 us into a 130 us encounter sub-step and ending after it.)
    const bool overlap = !ctx->has_small && ctx->has_big && ctx->pdl && p.bs_rows == 3;
    launch(k_drift_universal, (unsigned)((D.n + dthr - 1) / dthr), dthr, D, rcB, p.dt, p.compat_block,
           p.kepler_tol, p.kepler_max_iter, guess_of(p), mlp, ctx->d_log, ctx->d_log_count, ctx->log_cap,
           overlap ? 1 : 0);
    nk++;
    if (ctx->has_small) {
      launch(k_encounter_small, ctx->enc_blocks, 64, D, rcB, p.dt, p.compat_block, p.bs_rows, p.softening2);
      nk++;
    }
    if (ctx->has_big) {
      // (encounter timing: events on the step stream around the launch; the
      // event between the drift and this kernel makes them run one after the
      // other, so the interval holds the encounter sub-step alone)
      const bool enc_ev = ctx->time_encounter && !ctx->enc_ev.empty();
      if (enc_ev) CK(cudaEventRecordWithFlags(ctx->enc_ev[2 * step_in_graph], s, cudaEventRecordExternal));
      if (p.bs_rows == 3 && D.nsys == 1)
        launch(k_encounter_tasks<true>, ctx->sms * kEncBlocksPerSM, 32 * kEncTaskWarps, D, rcB, p.dt,
               p.compat_block, p.softening2, kEncSpin, overlap ? 1 : 0);
      else if (p.bs_rows == 3)
        launch(k_encounter_tasks<false>, ctx->sms * kEncBlocksPerSM, 32 * kEncTaskWarps, D, rcB, p.dt,
               p.compat_block, p.softening2, kEncSpin, overlap ? 1 : 0);
      else
        launch(k_encounter_cluster, ctx->enc_blocks * 2, 32, D, rcB, p.dt, p.compat_block, p.bs_rows,
               p.softening2);
      if (enc_ev) CK(cudaEventRecordWithFlags(ctx->enc_ev[2 * step_in_graph + 1], s, cudaEventRecordExternal));
      nk++;
    }
    if (ctx->collide_on) {
      launch(k_collide_find, ctx->sms * 4, 256, D, ctx->col);
      launch(k_collide_resolve, 1, 32, D, ctx->col, p.hill_factor);
      nk += 2;
    }
    momentum(D.vo);
    if (jump_cl)
      launch(k_jump_cluster<false>, njc, kJumpThreads, D, (const double*)D.xo, (const double*)D.vo, rcB, hdt);
    else
      launch(k_jump<true, false>, njb, kJumpThreads, D, D.xo, D.vo, rcB, hdt);
    nk++;
    if ((st = kick(rcB, rcA, 1, 2))) return st;
    if (lerr != cudaSuccess) return fail(ctx, MERC_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(lerr));
  }
  CK(cudaGetLastError());
  if (kernels) *kernels = nk;
  return MERC_OK;
}

// Capture `steps` steps; with timing on, kick events use slots first_slot..
int capture(merc_ctx* ctx, int steps, bool timed, int first_slot, bool first_alone, bool last_alone,
            cudaGraphExec_t* out, int* kernels) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  *kernels = 0;
  for (int k = 0; k < steps; k++) {
    int nk = 0;
    int st = enqueue_step(ctx, timed, first_slot / 4 + k, &nk, k == 0 && first_alone, k == steps - 1 && last_alone);
    *kernels += nk;
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

// Kinds of step graphs.  Inside a graph the kick that ends a step and the
// kick that starts the next share their far field (merged); at a graph's ends
// a kick is either merged with the neighbouring graph's (when merc_step
// replays another graph right after it) or done alone.  A call of k >= 2
// full graphs replays HEAD, MID x (k - 2), TAIL; one full graph replays
// ALONE; the remaining steps replay ONE.  The merged and the separate forms
// give the same bits.
enum GraphKind { G_ALONE = 0, G_ONE = 1, G_HEAD = 2, G_MID = 3, G_TAIL = 4 };
constexpr int kKindSteps[5] = {kGraphSteps, 1, kGraphSteps, kGraphSteps, kGraphSteps};
constexpr bool kKindFirstAlone[5] = {true, true, true, false, false};  // start kick done in the graph
constexpr bool kKindLastAlone[5] = {true, true, false, false, true};   // end kick not merged onward
constexpr int kKindSlot[5] = {0, 4 * kGraphSteps, 4 * (kGraphSteps + 1), 4 * (2 * kGraphSteps + 1),
                              4 * (3 * kGraphSteps + 1)};
constexpr int kKickSlots = 4 * (4 * kGraphSteps + 1);

int build_graphs(merc_ctx* ctx) {
  drop_graphs(ctx);
  if (ctx->time_kicks) {
    while (ctx->kick_ev.size() < (size_t)kKickSlots) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->kick_ev.push_back(e);
    }
    ctx->kick_ev_used.assign(kKickSlots, 0);
  }
  if (ctx->time_encounter) {
    while (ctx->enc_ev.size() < (size_t)(kKickSlots / 2)) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->enc_ev.push_back(e);
    }
  }
  for (int k = 0; k < 5; k++) {
    int st = capture(ctx, kKindSteps[k], ctx->time_kicks, kKindSlot[k], kKindFirstAlone[k], kKindLastAlone[k],
                     &ctx->graphs[k], &ctx->graph_kernels[k]);
    if (st) return st;
  }
  ctx->graph_steps = kGraphSteps;
  return MERC_OK;
}

// ---- persistent path for batches of small systems ----
constexpr int kSweepChunk = 16;  // steps of massive-body history per chunk

int sweep_nh(const merc_ctx* ctx) {
  int nh = 1;
  for (int v : ctx->h_nm) nh = std::max(nh, v);
  return nh;
}

size_t sweep_smem_bytes(const merc_ctx* ctx) {
  return 2 * 8 * hist_step_doubles(sweep_nh(ctx)) * kSweepChunk;  // two history buffers
}

// The persistent kernel keeps only the massive bodies and their history in
// shared memory, so any batch of small systems fits.
// A block integrates one work item at a time: the test particles of a slice of
// one system; a system with many test particles is cut into several items,
// so a few large systems (the reference's Planet Nine sweep: 4 to 32 systems
// of 10240 bodies) fill the GPU as well as thousands of small ones.
bool use_persistent(const merc_ctx* ctx) {
  return ctx->p.drift == MERC_DRIFT_UNIVERSAL && !ctx->has_big && ctx->log_cap == 0 && !ctx->collide_on &&
         ctx->nmax_sys > 0 && sweep_smem_bytes(ctx) <= (size_t)ctx->smem_optin;
}

// Work items for blocks of `threads` and a grid of at most `grid` blocks:
// about one item per block, of at least `threads` test particles, systems
// largest first with their slices together; the first slice is the primary.
// Every item integrates its system's massive bodies in one warp before its
// test particles, so fewer, larger items pay that phase less often (the
// reference's Planet Nine sweep, 32 x 10240 bodies: 0.216 ms per step with
// one item per block, 0.241 with two, 0.307 with four).
int build_items(merc_ctx* ctx, int threads, int grid) {
  if (ctx->items_threads == threads && ctx->items_grid == grid) return MERC_OK;
  const int nsys = ctx->D.nsys;
  int64_t tps = 0;
  for (int q = 0; q < nsys; q++) tps += (ctx->h_off[q + 1] - ctx->h_off[q]) - ctx->h_nm[q];
  const int64_t slice = std::max<int64_t>(threads, (tps + grid - 1) / grid);
  std::vector<SweepItem> items;
  for (int q : ctx->h_order) {
    const int nm = ctx->h_nm[q], ntp = (ctx->h_off[q + 1] - ctx->h_off[q]) - nm;
    const int k = (int)std::max<int64_t>(1, (ntp + slice - 1) / slice);
    for (int i = 0; i < k; i++)
      items.push_back(SweepItem{q, nm + (int)((int64_t)i * ntp / k), nm + (int)((int64_t)(i + 1) * ntp / k), i == 0});
  }
  if ((int)items.size() > ctx->items_cap) return fail(ctx, MERC_ERR_CONFIG, "sweep items exceed their capacity");
  CK(cudaMemcpy(ctx->d_items, items.data(), sizeof(SweepItem) * items.size(), cudaMemcpyHostToDevice));
  ctx->n_items = (int)items.size();
  ctx->items_threads = threads;
  ctx->items_grid = grid;
  return MERC_OK;
}

SweepArgs sweep_args(merc_ctx* ctx, int steps, bool trial) {
  SweepArgs a;
  a.D = ctx->D;
  const merc_params& p = ctx->p;
  if (trial) {  // a timing trial integrates a copy of the state into scratch
    a.D.x = ctx->D.xo;
    a.D.v = ctx->D.vo;
    a.D.flags = ctx->d_tune_flags;
    a.D.counters = ctx->d_tune_counters;
  }
  a.items = ctx->d_items;
  a.queue = ctx->d_queue;
  a.nitems = ctx->n_items;
  a.nmax = ctx->nmax_sys;
  a.moff = ctx->d_moff;
  a.stage = ctx->d_stage;
  a.stage_f = ctx->d_stage_f;
  a.nh = sweep_nh(ctx);
  a.chunk = kSweepChunk;
  a.steps = steps;
  a.dt = p.dt;
  a.soft2 = p.softening2;
  a.hill = p.hill_factor;
  a.tol = p.kepler_tol;
  a.eject_r2 = p.eject_r > 0 ? p.eject_r * p.eject_r : 0.0;
  a.compat_block = p.compat_block;
  a.rows = p.bs_rows;
  a.max_iter = p.kepler_max_iter;
  a.mlp = (p.warm_start == MERC_WARM_MLP && ctx->mlp_ready) ? ctx->d_mlp : nullptr;
  a.guess = guess_of(p);
  a.rc_final = trial ? ctx->D.rc[ctx->rc_cur ^ 1] : ctx->D.rc[ctx->rc_cur];
  return a;
}

// One persistent launch over the work items built for (threads, grid); after
// a launch that is not a timing trial the staged massive bodies are written back.
int launch_sweep(merc_ctx* ctx, int threads, int grid, int steps, bool trial) {
  const size_t smem = sweep_smem_bytes(ctx);
  int st = build_items(ctx, threads, grid);
  if (st) return st;
  CK(cudaMemsetAsync(ctx->d_queue, 0, sizeof(int), ctx->stream));
  k_sweep_persistent<<<std::min(grid, ctx->n_items), threads, smem, ctx->stream>>>(sweep_args(ctx, steps, trial));
  CK(cudaGetLastError());
  if (!trial && ctx->n_mass) {
    k_sweep_commit<<<(ctx->n_mass + kThreads - 1) / kThreads, kThreads, 0, ctx->stream>>>(
        ctx->D, ctx->d_mbody, ctx->d_stage, ctx->d_stage_f, ctx->n_mass);
    CK(cudaGetLastError());
  }
  return MERC_OK;
}

// Tuner of the persistent kernel: the block size (bodies per thread) is
// chosen by timing a 2-step trial of each candidate on a copy of the state;
// the choice is cached per (largest system, massive count, systems) bucket.
std::mutex g_tune_mu;
std::vector<std::pair<std::array<int, 3>, std::pair<int, int>>> g_tune_cache;

int tune_sweep(merc_ctx* ctx) {
  const size_t smem = sweep_smem_bytes(ctx);
  CK(cudaFuncSetAttribute(k_sweep_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int max_nm = 0;
  for (int v : ctx->h_nm) max_nm = std::max(max_nm, v);
  int lg = 0;
  while ((1 << lg) < ctx->nmax_sys) lg++;
  int sl = 0;
  while ((1 << sl) < ctx->D.nsys) sl++;
  std::array<int, 3> key = {lg, max_nm, sl};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto& e : g_tune_cache)
      if (e.first == key) {
        ctx->sweep_threads = e.second.first;
        ctx->sweep_grid = e.second.second;
        return MERC_OK;
      }
  }
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int cands[3] = {64, 128, 256};
  float best = 1e30f;
  int best_t = 128, best_g = sms;
  for (int t : cands) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_persistent, t, smem));
    if (per_sm < 1) continue;
    const int grid = per_sm * sms;
    const size_t n3 = 3 * (size_t)ctx->D.n;
    CK(cudaMemcpyAsync(ctx->D.xo, ctx->D.x, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->D.vo, ctx->D.v, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_tune_flags, 0, sizeof(uint32_t) * ctx->D.n, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    int st = launch_sweep(ctx, t, grid, 2, true);
    if (st) return st;
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (ms < best) {
      best = ms;
      best_t = t;
      best_g = grid;
    }
  }
  ctx->sweep_threads = best_t;
  ctx->sweep_grid = best_g;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache.push_back({key, {best_t, best_g}});
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
  p->warm_start = MERC_WARM_SERIES;
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
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
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
  if (ctx->d_mlp) cudaFree(ctx->d_mlp);
  if (ctx->d_log) cudaFree(ctx->d_log);
  if (ctx->d_log_count) cudaFree(ctx->d_log_count);
  for (cudaEvent_t e : ctx->kick_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->enc_ev) cudaEventDestroy(e);
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
  if (use_persistent(ctx)) {
    if (!ctx->sweep_threads) {
      int st = tune_sweep(ctx);
      if (st) return st;
    }
    CK(cudaFuncSetAttribute(k_sweep_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)sweep_smem_bytes(ctx)));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    const int64_t chunk = 1 << 20;  // steps per launch
    for (int64_t done = 0; done < n_steps; done += chunk) {
      int st = launch_sweep(ctx, ctx->sweep_threads, ctx->sweep_grid, (int)std::min(chunk, n_steps - done), false);
      if (st) return st;
      ctx->launches += ctx->n_mass ? 2 : 1;  // the persistent kernel and the commit of the massive bodies
    }
    ctx->last_graph_steps = 0;
  } else {
    if (!ctx->graphs[G_ALONE]) {
      int st = build_graphs(ctx);
      if (st) return st;
    }
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    const int64_t full = n_steps / kGraphSteps, rest = n_steps % kGraphSteps;
    unsigned kinds = 0;
    auto replay = [&](int kind, int64_t times) -> int {
      for (int64_t k = 0; k < times; k++) CK(cudaGraphLaunch(ctx->graphs[kind], ctx->stream));
      if (times > 0) kinds |= 1u << kind;
      ctx->launches += times * ctx->graph_kernels[kind];
      return MERC_OK;
    };
    int st = MERC_OK;
    if (full == 1) {
      st = replay(G_ALONE, 1);
    } else if (full >= 2) {
      if (!(st = replay(G_HEAD, 1)) && !(st = replay(G_MID, full - 2))) st = replay(G_TAIL, 1);
    }
    if (!st) st = replay(G_ONE, rest);
    if (st) return st;
    ctx->last_kinds = kinds;
    ctx->last_graph_steps = rest > 0 ? 1 : kGraphSteps;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->last_ms = ms;
  ctx->steps_done += n_steps;
  if (ctx->has_big && ctx->D.enc_head) {
    int gave_up = 0;
    CK(cudaMemcpy(&gave_up, ctx->D.enc_head + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (gave_up) {
      ctx->loaded = false;  // the encounter state is incomplete: load again
      return fail(ctx, MERC_ERR_TIMEOUT, "encounter sub-step: a bounded device wait gave up");
    }
  }
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

int merc_set_radii(merc_ctx* ctx, const double* radius) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_set_radii before a load");
  CK(cudaSetDevice(ctx->device));
  drop_graphs(ctx);  // the step graphs gain or lose the collision kernels
  if (!radius) {
    ctx->collide_on = false;
    return MERC_OK;
  }
  const int n = ctx->D.n;
  for (int j = 0; j < n; j++)
    if (!(radius[j] >= 0.0) || !std::isfinite(radius[j]))
      return fail(ctx, MERC_ERR_CONFIG, "radius[%d] must be finite and >= 0", j);
  Collide& C = ctx->col;
  int st;
  if (!C.radius) {
    double* r = nullptr;
    if ((st = dalloc(ctx, &r, n)) || (st = dalloc(ctx, &C.n_pairs, 2)) || (st = dalloc(ctx, &C.pairs, kColPairCap)) ||
        (st = dalloc(ctx, &C.step, 1)) || (st = dalloc(ctx, &C.n_events, 1)) ||
        (st = dalloc(ctx, &C.events, 3 * (size_t)kColEventCap)))
      return st;
    C.radius = r;
    C.m = ctx->d_m;
  }
  const long long step0 = ctx->steps_done, zero = 0;
  CK(cudaMemcpyAsync((void*)C.radius, radius, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(C.n_pairs, 0, 2 * sizeof(int), ctx->stream));
  CK(cudaMemcpyAsync(C.step, &step0, sizeof step0, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(C.n_events, &zero, sizeof zero, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->collide_on = true;
  return MERC_OK;
}

int merc_get_collisions(merc_ctx* ctx, merc_collision* out, int64_t max, int64_t* count) {
  if (!ctx || max < 0 || (max > 0 && !out)) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_get_collisions before a load");
  long long total = 0;
  int lost = 0;
  if (ctx->col.n_events) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpy(&total, ctx->col.n_events, sizeof total, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&lost, ctx->col.n_pairs + 1, sizeof lost, cudaMemcpyDeviceToHost));
  }
  if (count) *count = total;
  const int64_t k = std::min<int64_t>(std::min<int64_t>(total, kColEventCap), max);
  if (k > 0) {
    std::vector<long long> ev(3 * (size_t)k);
    CK(cudaMemcpy(ev.data(), ctx->col.events, sizeof(long long) * ev.size(), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < k; i++) out[i] = merc_collision{ev[3 * i], ev[3 * i + 1], ev[3 * i + 2]};
  }
  if (lost) return fail(ctx, MERC_ERR_STATE, "more than %d collision candidates in one step: some were dropped",
                        kColPairCap);
  return MERC_OK;
}

int merc_get_masses(merc_ctx* ctx, double* mass) {
  if (!ctx || !mass) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_get_masses before a load");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(mass, ctx->d_m, sizeof(double) * ctx->D.n, cudaMemcpyDeviceToHost, ctx->stream));
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
    unsigned long long c[kNumCounters];
    CK(cudaMemcpyAsync(c, ctx->D.counters, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out->ce_body_steps = (int64_t)c[0];
    out->kepler_iterations = (int64_t)c[1];
    out->kepler_solves = (int64_t)c[2];
    out->kepler_nonconverged = (int64_t)c[3];
    out->kepler_simt_iterations = (int64_t)c[4];
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

int merc_angular_momentum(merc_ctx* ctx, double* L) {
  if (!ctx || !L) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_angular_momentum before a load");
  CK(cudaSetDevice(ctx->device));
  double* tmp = nullptr;
  int st;
  if ((st = dalloc(ctx, &tmp, 3 * (size_t)ctx->D.nsys))) return st;
  k_angmom<<<ctx->D.nsys, kThreads, 0, ctx->stream>>>(ctx->D, tmp);
  ctx->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(L, tmp, sizeof(double) * 3 * ctx->D.nsys, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(tmp);
  ctx->allocs.pop_back();
  return MERC_OK;
}

int64_t merc_launch_count(const merc_ctx* ctx) { return ctx ? ctx->launches : 0; }

// ---- learned warm start ----
int merc_mlp_log(merc_ctx* ctx, int64_t capacity) {
  if (!ctx || capacity < 0) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->d_log) cudaFree(ctx->d_log);
  ctx->d_log = nullptr;
  ctx->log_cap = 0;
  if (!ctx->d_log_count) CK(cudaMalloc(&ctx->d_log_count, sizeof(unsigned long long)));
  CK(cudaMemset(ctx->d_log_count, 0, sizeof(unsigned long long)));
  if (capacity > 0) {
    CK(cudaMalloc(&ctx->d_log, sizeof(float) * 5 * (size_t)capacity));
    ctx->log_cap = capacity;
  }
  drop_graphs(ctx);  // the graphs hold the log pointer
  return MERC_OK;
}

int64_t merc_mlp_log_count(merc_ctx* ctx) {
  if (!ctx || !ctx->d_log_count) return 0;
  unsigned long long c = 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return 0;
  cudaStreamSynchronize(ctx->stream);
  if (cudaMemcpy(&c, ctx->d_log_count, sizeof c, cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  return (int64_t)std::min<unsigned long long>(c, (unsigned long long)ctx->log_cap);
}

int merc_mlp_get_log(merc_ctx* ctx, float* out, int64_t max_samples) {
  if (!ctx || !out || max_samples < 0) return MERC_ERR_CONFIG;
  int64_t n = std::min<int64_t>(merc_mlp_log_count(ctx), max_samples);
  if (n > 0) CK(cudaMemcpy(out, ctx->d_log, sizeof(float) * 5 * (size_t)n, cudaMemcpyDeviceToHost));
  return MERC_OK;
}

int merc_mlp_append_log(merc_ctx* ctx, const float* samples, int64_t n) {
  if (!ctx || !samples || n < 0) return MERC_ERR_CONFIG;
  if (!ctx->d_log) return fail(ctx, MERC_ERR_STATE, "no drift log: call merc_mlp_log first");
  int64_t have = merc_mlp_log_count(ctx);
  if (have + n > ctx->log_cap) return fail(ctx, MERC_ERR_CONFIG, "drift log full (%lld + %lld > %lld)",
                                          (long long)have, (long long)n, (long long)ctx->log_cap);
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpy(ctx->d_log + 5 * (size_t)have, samples, sizeof(float) * 5 * (size_t)n, cudaMemcpyHostToDevice));
  unsigned long long c = (unsigned long long)(have + n);
  CK(cudaMemcpy(ctx->d_log_count, &c, sizeof c, cudaMemcpyHostToDevice));
  return MERC_OK;
}

// ---- checkpoint file ----
// Little-endian binary: "MERCCKP1", uint32 version (3), uint32 sizeof(merc_params),
// merc_params, int32 n_systems, int64 n_bodies, int64 steps_done,
// int64 body_offset[n_systems + 1], int32 n_massive[n_systems], double
// mass[n], pos[3n], vel[3n], a_lag[n], uint32 flags[n], uint64 counters[5],
// uint32 has_mlp, float mlp[MERC_MLP_BLOB] (when has_mlp), uint32 has_radii and,
// when set, double radius[n], int64 collision step counter, int64 events,
// int64 event log[3 min(events, 65536)], then the FNV-1a 64-bit hash of every
// byte before it.  Version 2 files (no collision block) are read too.
struct CkptWriter {
  std::FILE* f;
  uint64_t h = 1469598103934665603ull;
  bool ok = true;
  void put(const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    ok = ok && std::fwrite(p, 1, n, f) == n;
  }
};

struct CkptReader {
  const std::vector<unsigned char>& buf;
  size_t pos = 0;
  bool ok = true;
  void get(void* p, size_t n) {
    if (pos + n > buf.size()) {
      ok = false;
      return;
    }
    std::memcpy(p, buf.data() + pos, n);
    pos += n;
  }
};

int merc_save_checkpoint(merc_ctx* ctx, const char* path) {
  if (!ctx || !path) return MERC_ERR_CONFIG;
  if (!ctx->loaded) return fail(ctx, MERC_ERR_STATE, "merc_save_checkpoint before a load");
  CK(cudaSetDevice(ctx->device));
  const int32_t nsys = ctx->D.nsys;
  const int64_t n = ctx->D.n;
  std::vector<int64_t> off(ctx->h_off.begin(), ctx->h_off.end());
  std::vector<int32_t> nm(ctx->h_nm.begin(), ctx->h_nm.end());
  std::vector<double> mass(n), pos(3 * n), vel(3 * n), alag(n);
  std::vector<uint32_t> flags(n);
  unsigned long long counters[kNumCounters];
  CK(cudaMemcpyAsync(mass.data(), ctx->D.m, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(counters, ctx->D.counters, sizeof counters, cudaMemcpyDeviceToHost, ctx->stream));
  int st;
  if ((st = merc_get_state(ctx, pos.data(), vel.data(), flags.data())) ||
      (st = merc_get_a_lag(ctx, alag.data())))
    return st;
  std::vector<float> mlp;
  if (ctx->mlp_ready) {
    mlp.resize(kBlob);
    if ((st = merc_mlp_get_weights(ctx, mlp.data()))) return st;
  }
  const uint32_t has_radii = ctx->collide_on ? 1u : 0u;
  std::vector<double> radii;
  long long col_step = 0, col_events = 0;
  std::vector<long long> events;
  if (has_radii) {
    radii.resize(n);
    CK(cudaMemcpy(radii.data(), ctx->col.radius, sizeof(double) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&col_step, ctx->col.step, sizeof col_step, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&col_events, ctx->col.n_events, sizeof col_events, cudaMemcpyDeviceToHost));
    events.resize(3 * (size_t)std::min<long long>(col_events, kColEventCap));
    if (!events.empty())
      CK(cudaMemcpy(events.data(), ctx->col.events, sizeof(long long) * events.size(), cudaMemcpyDeviceToHost));
  }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return fail(ctx, MERC_ERR_CONFIG, "cannot open %s for writing", path);
  CkptWriter w{f};
  const uint32_t version = 3, psize = sizeof(merc_params), has_mlp = ctx->mlp_ready ? 1u : 0u;
  const int64_t steps = ctx->steps_done;
  w.put("MERCCKP1", 8);
  w.put(&version, 4);
  w.put(&psize, 4);
  w.put(&ctx->p, sizeof(merc_params));
  w.put(&nsys, 4);
  w.put(&n, 8);
  w.put(&steps, 8);
  w.put(off.data(), 8 * off.size());
  w.put(nm.data(), 4 * nm.size());
  w.put(mass.data(), 8 * mass.size());
  w.put(pos.data(), 8 * pos.size());
  w.put(vel.data(), 8 * vel.size());
  w.put(alag.data(), 8 * alag.size());
  w.put(flags.data(), 4 * flags.size());
  w.put(counters, sizeof counters);
  w.put(&has_mlp, 4);
  if (has_mlp) w.put(mlp.data(), 4 * mlp.size());
  w.put(&has_radii, 4);
  if (has_radii) {
    w.put(radii.data(), 8 * radii.size());
    w.put(&col_step, 8);
    w.put(&col_events, 8);
    w.put(events.data(), 8 * events.size());
  }
  const uint64_t hash = w.h;
  w.put(&hash, 8);
  const bool ok = w.ok && std::fclose(f) == 0;
  if (!ok) return fail(ctx, MERC_ERR_CONFIG, "writing %s failed", path);
  return MERC_OK;
}

int merc_load_checkpoint(merc_ctx* ctx, const char* path) {
  if (!ctx || !path) return MERC_ERR_CONFIG;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, MERC_ERR_CONFIG, "cannot open %s", path);
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  std::fclose(f);
  if (buf.size() < 8 + 8) return fail(ctx, MERC_ERR_CONFIG, "%s: not a checkpoint", path);
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i + 8 < buf.size(); i++) h = (h ^ buf[i]) * 1099511628211ull;
  uint64_t stored;
  std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
  if (std::memcmp(buf.data(), "MERCCKP1", 8) != 0 || stored != h)
    return fail(ctx, MERC_ERR_CONFIG, "%s: not a checkpoint or damaged (hash mismatch)", path);
  CkptReader r{buf};
  char magic[8];
  uint32_t version = 0, psize = 0, has_mlp = 0;
  merc_params p;
  int32_t nsys = 0;
  int64_t n = 0, steps = 0;
  r.get(magic, 8);
  r.get(&version, 4);
  r.get(&psize, 4);
  if ((version != 2 && version != 3) || psize != sizeof(merc_params))
    return fail(ctx, MERC_ERR_CONFIG, "%s: checkpoint version %u not supported", path, version);
  r.get(&p, sizeof p);
  r.get(&nsys, 4);
  r.get(&n, 8);
  r.get(&steps, 8);
  if (!r.ok || nsys <= 0 || n <= 0 || n > ((int64_t)1 << 31) || (size_t)n > buf.size() / 8)
    return fail(ctx, MERC_ERR_CONFIG, "%s: bad sizes", path);
  std::vector<int64_t> off(nsys + 1);
  std::vector<int32_t> nm(nsys);
  std::vector<double> mass(n), pos(3 * n), vel(3 * n), alag(n);
  std::vector<uint32_t> flags(n);
  unsigned long long counters[kNumCounters];
  r.get(off.data(), 8 * off.size());
  r.get(nm.data(), 4 * nm.size());
  r.get(mass.data(), 8 * mass.size());
  r.get(pos.data(), 8 * pos.size());
  r.get(vel.data(), 8 * vel.size());
  r.get(alag.data(), 8 * alag.size());
  r.get(flags.data(), 4 * flags.size());
  r.get(counters, sizeof counters);
  r.get(&has_mlp, 4);
  std::vector<float> mlp;
  if (has_mlp) {
    mlp.resize(kBlob);
    r.get(mlp.data(), 4 * mlp.size());
  }
  uint32_t has_radii = 0;
  std::vector<double> radii;
  long long col_step = 0, col_events = 0;
  std::vector<long long> events;
  if (version >= 3) {
    r.get(&has_radii, 4);
    if (has_radii) {
      radii.resize(n);
      r.get(radii.data(), 8 * radii.size());
      r.get(&col_step, 8);
      r.get(&col_events, 8);
      if (!r.ok || col_events < 0) return fail(ctx, MERC_ERR_CONFIG, "%s: bad collision block", path);
      events.resize(3 * (size_t)std::min<long long>(col_events, kColEventCap));
      r.get(events.data(), 8 * events.size());
    }
  }
  if (!r.ok || r.pos + 8 != buf.size()) return fail(ctx, MERC_ERR_CONFIG, "%s: truncated", path);
  int st;
  if ((st = merc_set_params(ctx, &p)) ||
      (st = merc_load_state(ctx, nsys, off.data(), nm.data(), mass.data(), pos.data(), vel.data(), alag.data())))
    return st;
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(ctx->D.flags, flags.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->D.counters, counters, sizeof counters, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->steps_done = steps;
  if (has_mlp && (st = merc_mlp_set_weights(ctx, mlp.data()))) return st;
  if (has_radii) {
    if ((st = merc_set_radii(ctx, radii.data()))) return st;
    CK(cudaMemcpy(ctx->col.step, &col_step, sizeof col_step, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->col.n_events, &col_events, sizeof col_events, cudaMemcpyHostToDevice));
    if (!events.empty())
      CK(cudaMemcpy(ctx->col.events, events.data(), sizeof(long long) * events.size(), cudaMemcpyHostToDevice));
  }
  return MERC_OK;
}

int merc_load_systems(merc_ctx* ctx, const merc_system_desc* systems, int32_t n_systems) {
  if (!ctx) return MERC_ERR_CONFIG;
  if (!systems || n_systems <= 0) return fail(ctx, MERC_ERR_CONFIG, "no systems");
  const bool by_elements = systems[0].elements != nullptr;
  std::vector<int64_t> off(n_systems + 1, 0);
  std::vector<int32_t> nm(n_systems);
  for (int s = 0; s < n_systems; s++) {
    const merc_system_desc& d = systems[s];
    if (d.n_bodies <= 0 || !d.mass) return fail(ctx, MERC_ERR_CONFIG, "system %d: no bodies or no masses", s);
    if ((d.elements != nullptr) != by_elements || (!by_elements && (!d.pos || !d.vel)))
      return fail(ctx, MERC_ERR_CONFIG, "system %d: give elements for every system, or pos and vel for every one", s);
    off[s + 1] = off[s] + d.n_bodies;
    nm[s] = d.n_massive;
  }
  const int64_t n = off[n_systems];
  std::vector<double> mass(n), a(by_elements ? 6 * n : 3 * n), b(by_elements ? 0 : 3 * n);
  for (int s = 0; s < n_systems; s++) {
    const merc_system_desc& d = systems[s];
    const int64_t b0 = off[s], ns = d.n_bodies;
    std::memcpy(mass.data() + b0, d.mass, sizeof(double) * ns);
    const int rows = by_elements ? 6 : 3;
    for (int k = 0; k < rows; k++) {
      std::memcpy(a.data() + k * n + b0, (by_elements ? d.elements : d.pos) + k * ns, sizeof(double) * ns);
      if (!by_elements) std::memcpy(b.data() + k * n + b0, d.vel + k * ns, sizeof(double) * ns);
    }
  }
  if (by_elements) return merc_load_elements(ctx, n_systems, off.data(), nm.data(), mass.data(), a.data());
  return merc_load_state(ctx, n_systems, off.data(), nm.data(), mass.data(), a.data(), b.data(), nullptr);
}

int merc_mlp_set_weights(merc_ctx* ctx, const float* w) {
  if (!ctx || !w) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(ctx->device));
  if (!ctx->d_mlp) CK(cudaMalloc(&ctx->d_mlp, sizeof(float) * kBlob));
  CK(cudaMemcpy(ctx->d_mlp, w, sizeof(float) * kBlob, cudaMemcpyHostToDevice));
  ctx->mlp_ready = true;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_mlp_get_weights(merc_ctx* ctx, float* w) {
  if (!ctx || !w) return MERC_ERR_CONFIG;
  if (!ctx->mlp_ready) return fail(ctx, MERC_ERR_STATE, "no warm-start network: train or set weights first");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpy(w, ctx->d_mlp, sizeof(float) * kBlob, cudaMemcpyDeviceToHost));
  return MERC_OK;
}

}  // extern "C"

namespace {

// Train the network on device data (5 floats per sample) with the
// hand-written kernels: k_mlp_grad -> k_mlp_reduce -> k_mlp_adam per batch.
int train_on(merc_ctx* ctx, int device, float* d_blob, const float* d_data, long long n_data, int epochs, int batch,
             float lr, unsigned long long seed, float* loss_out) {
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int nblocks = std::max(1, std::min(2 * sms, (batch + kMlpThreads - 1) / kMlpThreads));
  float *part = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  CK(cudaMalloc(&part, sizeof(float) * (size_t)nblocks * (kNet + 1)));
  CK(cudaMalloc(&grad, sizeof(float) * (kNet + 1)));
  CK(cudaMalloc(&m, sizeof(float) * kNet));
  CK(cudaMalloc(&v, sizeof(float) * kNet));
  CK(cudaMemset(m, 0, sizeof(float) * kNet));
  CK(cudaMemset(v, 0, sizeof(float) * kNet));
  const long long steps_per_epoch = std::max<long long>(1, n_data / batch);
  int step = 0;
  float lossv = 0.f;
  for (int ep = 0; ep < epochs; ep++) {
    double esum = 0.0;
    // cosine decay of the learning rate over the epochs
    const float lr_ep = lr * 0.5f * (1.0f + cosf(3.14159265f * ep / std::max(1, epochs)));
    for (long long st = 0; st < steps_per_epoch; st++) {
      step++;
      k_mlp_grad<<<nblocks, kMlpThreads, 0, ctx ? ctx->stream : 0>>>(d_blob, d_data, n_data, nullptr, batch,
                                                                     seed + 0x632BE59BD9B4E019ull * step, part);
      k_mlp_reduce<<<(kNet + 1 + 127) / 128, 128, 0, ctx ? ctx->stream : 0>>>(part, nblocks, batch, grad);
      k_mlp_adam<<<(kNet + 127) / 128, 128, 0, ctx ? ctx->stream : 0>>>(d_blob, grad, m, v, lr_ep, 0.9f, 0.999f,
                                                                        1e-8f, step);
      if (st == steps_per_epoch - 1 || (st & 63) == 0) {
        CK(cudaMemcpyAsync(&lossv, grad + kNet, sizeof(float), cudaMemcpyDeviceToHost, ctx ? ctx->stream : 0));
        CK(cudaStreamSynchronize(ctx ? ctx->stream : 0));
        esum = lossv;
      }
    }
    CK(cudaGetLastError());
    if (loss_out) loss_out[ep] = (float)esum;
  }
  cudaFree(part);
  cudaFree(grad);
  cudaFree(m);
  cudaFree(v);
  return MERC_OK;
}

// normalisation and feature box of a sample set (host side, double sums)
void fit_normalisation(const std::vector<float>& h, long long n, float* blob) {
  double mean[5] = {0, 0, 0, 0, 0}, sq[5] = {0, 0, 0, 0, 0};
  float lo[4], hi[4];
  for (int k = 0; k < 4; k++) {
    lo[k] = 3.4e38f;
    hi[k] = -3.4e38f;
  }
  for (long long i = 0; i < n; i++)
    for (int k = 0; k < 5; k++) {
      double x = h[5 * i + k];
      mean[k] += x;
      sq[k] += x * x;
      if (k < 4) {
        lo[k] = std::min(lo[k], h[5 * i + k]);
        hi[k] = std::max(hi[k], h[5 * i + k]);
      }
    }
  for (int k = 0; k < 5; k++) {
    mean[k] /= (double)n;
    double var = std::max(sq[k] / (double)n - mean[k] * mean[k], 1e-30);
    double sc = 1.0 / std::sqrt(var);
    if (k < 4) {
      blob[kInMean + k] = (float)mean[k];
      blob[kInScale + k] = (float)std::min(sc, 1e6);
      blob[kBoxLo + k] = lo[k];
      blob[kBoxHi + k] = hi[k];
    } else {
      blob[kOutMean] = (float)mean[k];
      blob[kOutScale] = (float)std::min(sc, 1e12);
    }
  }
  // the sign feature is +-1: keep it as it is
  blob[kInMean + 3] = 0.0f;
  blob[kInScale + 3] = 1.0f;
  blob[kBoxLo + 3] = -1.0f;
  blob[kBoxHi + 3] = 1.0f;
}

void init_weights(float* blob, unsigned long long seed) {
  unsigned long long z = seed ^ 0x2545F4914F6CDD1Dull;
  auto uni = [&]() {  // xorshift64*
    z ^= z >> 12;
    z ^= z << 25;
    z ^= z >> 27;
    return (double)((z * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int count, double bound) {
    for (int k = 0; k < count; k++) blob[off + k] = (float)((2.0 * uni() - 1.0) * bound);
  };
  fill(kW1, kH * 4, std::sqrt(6.0 / (4 + kH)));
  fill(kB1, kH, 0.0);
  fill(kW2, kH * kH, std::sqrt(6.0 / (kH + kH)));
  fill(kB2, kH, 0.0);
  fill(kW3, kH, std::sqrt(6.0 / (kH + 1)));
  blob[kB3] = 0.0f;
}

}  // namespace

extern "C" {

int merc_mlp_train(merc_ctx* ctx, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_per_epoch) {
  if (!ctx || epochs < 1 || batch < 32 || !(lr > 0.f)) return MERC_ERR_CONFIG;
  const long long n = merc_mlp_log_count(ctx);
  if (n < 1024) return fail(ctx, MERC_ERR_STATE, "warm-start training needs logged drifts (have %lld)", n);
  CK(cudaSetDevice(ctx->device));
  std::vector<float> h((size_t)5 * n);
  CK(cudaMemcpy(h.data(), ctx->d_log, sizeof(float) * 5 * (size_t)n, cudaMemcpyDeviceToHost));
  std::vector<float> blob(kBlob, 0.f);
  fit_normalisation(h, n, blob.data());
  init_weights(blob.data(), seed);
  if (!ctx->d_mlp) CK(cudaMalloc(&ctx->d_mlp, sizeof(float) * kBlob));
  CK(cudaMemcpy(ctx->d_mlp, blob.data(), sizeof(float) * kBlob, cudaMemcpyHostToDevice));
  int st = train_on(ctx, ctx->device, ctx->d_mlp, ctx->d_log, n, epochs, batch, lr, seed, loss_per_epoch);
  if (st) return st;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->mlp_ready = true;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_diag_mlp_grad(int device, int64_t n, const float* samples, const float* blob, float* loss, float* grad) {
  merc_ctx* ctx = nullptr;
  if (n <= 0 || !samples || !blob || !grad) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  float *d_s = nullptr, *d_b = nullptr, *d_part = nullptr, *d_g = nullptr;
  long long* d_idx = nullptr;
  std::vector<long long> idx(n);
  for (int64_t i = 0; i < n; i++) idx[i] = i;
  const int nblocks = (int)std::min<int64_t>(8, (n + kMlpThreads - 1) / kMlpThreads);
  CK(cudaMalloc(&d_s, sizeof(float) * 5 * n));
  CK(cudaMalloc(&d_b, sizeof(float) * kBlob));
  CK(cudaMalloc(&d_idx, sizeof(long long) * n));
  CK(cudaMalloc(&d_part, sizeof(float) * nblocks * (kNet + 1)));
  CK(cudaMalloc(&d_g, sizeof(float) * (kNet + 1)));
  CK(cudaMemcpy(d_s, samples, sizeof(float) * 5 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_b, blob, sizeof(float) * kBlob, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_idx, idx.data(), sizeof(long long) * n, cudaMemcpyHostToDevice));
  k_mlp_grad<<<nblocks, kMlpThreads>>>(d_b, d_s, n, d_idx, (int)n, 0, d_part);
  k_mlp_reduce<<<(kNet + 1 + 127) / 128, 128>>>(d_part, nblocks, (int)n, d_g);
  CK(cudaGetLastError());
  std::vector<float> g(kNet + 1);
  CK(cudaMemcpy(g.data(), d_g, sizeof(float) * (kNet + 1), cudaMemcpyDeviceToHost));
  memcpy(grad, g.data(), sizeof(float) * kNet);
  if (loss) *loss = g[kNet];
  cudaFree(d_s);
  cudaFree(d_b);
  cudaFree(d_idx);
  cudaFree(d_part);
  cudaFree(d_g);
  return MERC_OK;
}

// Evaluate the warm-start guess for n drift inputs on the GPU (diagnostic):
// pos/vel 3 x n component-major, returns s_guess (n) and, if s_solved is
// given, the converged s and iterations of the solve from that guess.
__global__ void k_mlp_probe(int n, const double* pos, const double* vel, double dt, const float* blob, double tol,
                            int max_iter, double* guess, double* solved, int* iters) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  d3 x = {pos[j], pos[n + j], pos[2 * n + j]}, v = {vel[j], vel[n + j], vel[2 * n + j]};
  // as the drift kernels: FP32 features, the network's relative correction
  double s0 = kGuessPlain;
  float rel = 0.0f;
  if (blob) {
    float f[4];
    if (warm_long(x, f32_trunc(dt))) {
      warm_features_f32(x, v, f32_trunc(dt), f);
      const float d = warm_delta(blob, f);
      if (d == d) {
        s0 = kGuessRel;
        rel = d;
      }
    }
  }
  const double p0 = dt / sqrt(mag2(x));
  guess[j] = s0 == kGuessRel ? p0 * (1.0 + (double)rel) : p0;
  UD u = universal_drift(FU{1.0, -0.0}, x, v, dt, s0, tol, max_iter, rel);
  solved[j] = u.s;
  iters[j] = u.iters;
}

int merc_diag_warm_start(int device, int64_t n, const double* pos, const double* vel, double dt, const float* blob,
                         double tol, int32_t max_iter, double* guess, double* solved, int32_t* iters) {
  merc_ctx* ctx = nullptr;
  if (n <= 0 || !pos || !vel || !guess || !solved || !iters) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  double *dp, *dv, *dg, *ds;
  int* di;
  float* db = nullptr;
  CK(cudaMalloc(&dp, sizeof(double) * 3 * n));
  CK(cudaMalloc(&dv, sizeof(double) * 3 * n));
  CK(cudaMalloc(&dg, sizeof(double) * n));
  CK(cudaMalloc(&ds, sizeof(double) * n));
  CK(cudaMalloc(&di, sizeof(int) * n));
  if (blob) {
    CK(cudaMalloc(&db, sizeof(float) * kBlob));
    CK(cudaMemcpy(db, blob, sizeof(float) * kBlob, cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(dp, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dv, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
  k_mlp_probe<<<(unsigned)((n + 127) / 128), 128>>>((int)n, dp, dv, dt, db, tol, max_iter, dg, ds, di);
  CK(cudaGetLastError());
  CK(cudaMemcpy(guess, dg, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(solved, ds, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(iters, di, sizeof(int) * n, cudaMemcpyDeviceToHost));
  cudaFree(dp);
  cudaFree(dv);
  cudaFree(dg);
  cudaFree(ds);
  cudaFree(di);
  if (db) cudaFree(db);
  return MERC_OK;
}

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

static int step_static(int device, const merc_params* p, int32_t n_bodies, int32_t n_massive, double* pos,
                       double* vel, const double* mass, uint32_t* flags, int64_t n_steps, void* stream) {
  merc_ctx* ctx = nullptr;  // errors are reported by status code only
  if (!p || !pos || !vel || !mass) return MERC_ERR_CONFIG;
  if (n_bodies <= 0 || n_massive < 0 || n_massive > n_bodies || n_steps < 0) return MERC_ERR_CONFIG;
  if (device < 0 || device >= kMaxDevices) return MERC_ERR_CONFIG;
  if (p->drift != MERC_DRIFT_UNIVERSAL || check_params(nullptr, p) != MERC_OK) return MERC_ERR_CONFIG;
  CK(cudaSetDevice(device));
  {
    // the call copies small tables from its own stack and waits for the
    // stream at the end: neither may be recorded into a graph
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
    if (e == cudaErrorStreamCaptureImplicit || (e == cudaSuccess && cap != cudaStreamCaptureStatusNone))
      return MERC_ERR_STATE;
    CK(e);
  }
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
    D.xf = c.take<float>(3 * (size_t)n);
    D.xo = c.take<double>(3 * (size_t)n);
    D.vo = c.take<double>(3 * (size_t)n);
    D.alag = c.take<double>(n);
    D.hc = c.take<double>(n);
    D.ce = c.take<unsigned char>(n);
    D.rc[0] = c.take<double>(rc_table_doubles(n));
    D.rc[1] = c.take<double>(rc_table_doubles(n));
    D.P = c.take<double>(3);
    D.part = c.take<double>(C > 1 ? (size_t)C * 3 * n : 1);
    D.ce_list = c.take<int>(n);
    D.ce_list_big = c.take<int>(n);
    D.ce_count = c.take<int>(2);
    D.counters = c.take<unsigned long long>(kNumCounters);
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
  D.nm0 = nm;
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
  CK(cudaMemsetAsync(D.counters, 0, kNumCounters * sizeof(unsigned long long), s));
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
      k_momentum_big<<<1, kMomThreads, 0, s>>>(D, d_ids, vsrc);
  };
  for (int64_t k = 0; k < n_steps; k++) {
    kick(rcA, nullptr, 0);
    momentum(D.v);
    k_jump<false, false><<<nb, kThreads, 0, s>>>(D, D.x, nullptr, rcB, hdt);
    CK(cudaMemsetAsync(D.ce_count, 0, 2 * sizeof(int), s));
    if (big) {
      CK(cudaMemsetAsync(D.ce, 0, n, s));
      k_ce_tiled<<<(unsigned)work.size(), kTile, 0, s>>>(D, d_work, rcB, p->compat_block);
    }
    k_drift_universal<<<nb, kThreads, 0, s>>>(D, rcB, p->dt, p->compat_block, p->kepler_tol, p->kepler_max_iter,
                                              guess_of(*p), nullptr, nullptr, nullptr, 0, 0);
    if (!big)
      k_encounter_small<<<sms * 4, 64, 0, s>>>(D, rcB, p->dt, p->compat_block, p->bs_rows, p->softening2);
    else
      k_encounter_big<<<sms * 4, kEncThreads, 0, s>>>(D, rcB, p->dt, p->compat_block, p->bs_rows, p->softening2);
    momentum(D.vo);
    k_jump<false, false><<<nb, kThreads, 0, s>>>(D, D.xo, D.vo, rcB, hdt);
    kick(rcB, rcA, 1);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(s));
  return MERC_OK;
}

extern "C" int merc_step_static(int device, const merc_params* p, int32_t n_bodies, int32_t n_massive, double* pos,
                                double* vel, const double* mass, uint32_t* flags, int64_t n_steps, void* stream) {
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  const int st = step_static(device, p, n_bodies, n_massive, pos, vel, mass, flags, n_steps, stream);
  if (prev >= 0) cudaSetDevice(prev);  // the caller's current device, as it was
  return st;
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

int merc_diag_far_recomputes(merc_ctx* ctx, int64_t* count) {
  if (!ctx || !count) return MERC_ERR_CONFIG;
  *count = 0;
  if (!ctx->loaded || !ctx->D.far_recomputes) return MERC_OK;
  CK(cudaSetDevice(ctx->device));
  unsigned long long c = 0;
  CK(cudaMemcpyAsync(&c, ctx->D.far_recomputes, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *count = (int64_t)c;
  return MERC_OK;
}

int merc_diag_pdl(merc_ctx* ctx, int on) {
  if (!ctx) return MERC_ERR_CONFIG;
  ctx->pdl = on != 0;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_diag_encounter_wait(merc_ctx* ctx, int32_t* gave_up) {
  if (!ctx || !gave_up) return MERC_ERR_CONFIG;
  if (!ctx->loaded || !ctx->has_big) return fail(ctx, MERC_ERR_STATE, "no big system loaded");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  Dev& D = ctx->D;
  int body = 0;
  for (int s = 0; s < D.nsys; s++)
    if (ctx->h_nm[s] > kSmallNm) {
      body = (int)ctx->h_off[s];
      break;
    }
  // one listed body; tasks start at the second unit (the first unit, row 2's
  // evaluation 0 of every listed body, is skipped)
  const int one = 1, head[2] = {enc_parts_slot(0), 0};
  CK(cudaMemcpy(D.ce_list_big, &body, sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(D.ce_count + 1, &one, sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(D.enc_head, head, sizeof head, cudaMemcpyHostToDevice));
  CK(cudaMemset(D.enc_cnt, 0, 11 * sizeof(int)));
  k_encounter_tasks<false><<<ctx->sms * kEncBlocksPerSM, 32 * kEncTaskWarps, 0, ctx->stream>>>(
      D, D.rc[ctx->rc_cur], ctx->p.dt, ctx->p.compat_block, ctx->p.softening2, 4096, 0);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  int h[2] = {0, 0};
  CK(cudaMemcpy(h, D.enc_head, sizeof h, cudaMemcpyDeviceToHost));
  *gave_up = h[1] != 0;
  // the step state of the encounter kernel back to zero
  CK(cudaMemset(D.enc_cnt, 0, 11 * sizeof(int)));
  CK(cudaMemset(D.enc_head, 0, 2 * sizeof(int)));
  CK(cudaMemset(D.ce_count, 0, 2 * sizeof(int)));
  return MERC_OK;
}

int merc_diag_time_kicks(merc_ctx* ctx, int on) {
  if (!ctx) return MERC_ERR_CONFIG;
  ctx->time_kicks = on != 0;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_diag_time_encounter(merc_ctx* ctx, int on) {
  if (!ctx) return MERC_ERR_CONFIG;
  ctx->time_encounter = on != 0;
  drop_graphs(ctx);
  return MERC_OK;
}

int merc_diag_encounter_ms(merc_ctx* ctx, double* avg_ms, int32_t* n_launches) {
  if (!ctx || !avg_ms) return MERC_ERR_CONFIG;
  if (!ctx->time_encounter || !ctx->has_big || ctx->graph_steps == 0 || ctx->last_graph_steps == 0)
    return fail(ctx, MERC_ERR_STATE, "encounter timing is off, no big system, or no step ran since it was turned on");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  int cnt = 0;
  // the last replay of every graph kind that the last call used
  for (int kind = 0; kind < 5; kind++) {
    if (!(ctx->last_kinds & (1u << kind))) continue;
    for (int k = 0; k < kKindSteps[kind]; k++) {
      const int slot = 2 * (kKindSlot[kind] / 4 + k);
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->enc_ev[slot], ctx->enc_ev[slot + 1]));
      sum += ms;
      cnt++;
    }
  }
  *avg_ms = cnt ? sum / cnt : 0.0;
  if (n_launches) *n_launches = cnt;
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
  // the last replay of every graph kind that the last call used
  for (int kind = 0; kind < 5; kind++) {
    if (!(ctx->last_kinds & (1u << kind))) continue;
    for (int k = 0; k < kKindSteps[kind]; k++) {
      for (int h = 0; h < 2; h++) {
        const int slot = kKindSlot[kind] + 4 * k + 2 * h;
        if (!ctx->kick_ev_used[slot]) continue;  // a kick merged into the one before
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->kick_ev[slot], ctx->kick_ev[slot + 1]));
        sum += ms;
        cnt++;
      }
    }
  }
  *avg_ms = cnt ? sum / cnt : 0.0;
  if (n_launches) *n_launches = cnt;
  return MERC_OK;
}

}  // extern "C"
