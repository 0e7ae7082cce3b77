// server.cu -- continuous-batching identification server (spi_server_* in spi_engine.h).
//
// Slots hold admitted jobs (windows in SoA layout, population, cost partials, CEM state).
// A tick advances every active slot by one CEM iteration:
//   cem_sample_kernel (grid row per slot) -> the rollout kernel of items.cu (one warp per
//   (slot, theta, 8-window group) work item, items ordered longest horizon first; the
//   single-job engine launches the same kernel on a one-slot table) -> server_finalize_kernel
//   -> cem_refit_kernel.
// The tick is captured once as a CUDA graph: every per-tick quantity (slot table, work
// order, item count) lives in device buffers that the host refreshes before each launch, and
// each round's rollout grid (one warp per work item) is set on the instantiated graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cem.cuh"
#include "common.h"
#include "items.h"
#include "model.h"
#include "rollout.cuh"

using namespace spi;

namespace {

// A tick runs up to kMaxRounds rounds of one CEM iteration each (sample, rollout, finalize,
// refit); slot j takes part in rounds 0 .. rounds[j] - 1, so jobs with less work per
// iteration advance several iterations per tick. Per round the rollout's work items are
// laid out slot after slot (begin[round][slot]) in the order order[round][0 .. n_order).
constexpr int kMaxRounds = 8;

struct SlotHost {
  bool used = false;      // holds a job (or its unread result)
  bool active = false;    // takes part in ticks
  bool retiring = false;  // result copy in flight
  int remaining = 0;
  int iterations = 0;
  int job_id = 0;
  int dim = 0;
  size_t bytes = 0;
  void* mem = nullptr;
  cudaEvent_t done = nullptr;
  SlotDesc desc;
};

__global__ void srv_rows_to_soa(const float* __restrict__ src, float* __restrict__ dst, int W, int F) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)W * F) return;
  dst[(size_t)(i % F) * W + (i / F)] = src[i];
}
__global__ void srv_actions_to_hw(const float* __restrict__ src, float* __restrict__ dst, int W, int H) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)W * H * 12) return;
  const int j = (int)(i % 12);
  const long long wh = i / 12;
  const int h = (int)(wh % H), w = (int)(wh / H);
  dst[((size_t)h * W + w) * 12 + j] = src[i];
}
__global__ void srv_fill(float* p, float v, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void server_finalize_kernel(const SlotDesc* __restrict__ slots, const int* __restrict__ rounds, int round,
                                       int mode, float w0, float w1, float w2, float w3, float w4, float w5) {
  const SlotDesc& S = slots[blockIdx.y];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (!S.active || n >= S.N || round >= rounds[blockIdx.y]) return;
  const float w[6] = {w0, w1, w2, w3, w4, w5};
  finalize_one(S.partial, n, S.G, S.norm, mode, w, S.comp, S.cost);
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct JobLayout {
  size_t init, tgt, weight, act, theta, partial, comp, cost, total;
};
JobLayout layout_of(int W, int H, int N) {
  const int G = (W + 7) / 8;
  JobLayout L;
  size_t o = 0;
  L.init = o;    o += align256((size_t)W * SPI_STATE_DIM * 4);
  L.tgt = o;     o += align256((size_t)W * SPI_STATE_DIM * 4);
  L.weight = o;  o += align256((size_t)W * 4);
  L.act = o;     o += align256((size_t)W * H * 12 * 4);
  L.theta = o;   o += align256((size_t)N * SPI_THETA_DIM * 4);
  L.partial = o; o += align256((size_t)N * G * SPI_N_COMP * 4);
  L.comp = o;    o += align256((size_t)N * SPI_N_COMP * 4);
  L.cost = o;    o += align256((size_t)N * 4);
  L.total = o;
  return L;
}

}  // namespace

struct spi_server {
  DevModel host_model;
  DevModel* d_model = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t capture = nullptr;
  int max_slots = 0, max_samples = 0;
  size_t budget = 0, used = 0;
  std::vector<SlotHost> slots;
  SlotDesc* d_slots = nullptr;
  SlotDesc* h_slots = nullptr;     // pinned staging
  int* d_order = nullptr;          // [kMaxRounds][max_slots]
  int* h_order = nullptr;          // pinned
  long long* d_begin = nullptr;    // [kMaxRounds][max_slots]
  long long* h_begin = nullptr;    // pinned
  int* d_rounds = nullptr;         // [max_slots]
  int* h_rounds = nullptr;         // pinned
  TickInfo* d_info = nullptr;      // [kMaxRounds]
  TickInfo* h_info = nullptr;      // pinned
  unsigned long long* d_bad = nullptr;
  CemState* d_cem = nullptr;
  CemState* h_cem_in = nullptr;    // pinned, per slot
  CemState* h_cem_out = nullptr;   // pinned, per slot
  int* h_zero = nullptr;           // pinned 0 (clears CemState::active)
  cudaEvent_t staging_free = nullptr;
  cudaEvent_t tick_done[2] = {nullptr, nullptr};   // at most two ticks in flight
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_src = nullptr;          // the captured graph (its nodes address `graph`'s)
  cudaGraphNode_t roll_node[kMaxRounds] = {};
  cudaKernelNodeParams roll_params[kMaxRounds] = {};
  int grid_cap = 0;                         // CTAs of a rollout launch at most (0: no cap)
  int ctas_per_sm = 0, items_per_claim = 1;
  long long max_items = 0;         // admission cap on work items per tick (0: none)
  int min_blocks = 3;              // rollout kernel occupancy variant
  int layout = SPI_LAYOUT_QUAD;    // SPI_LAYOUT_QUAD or SPI_LAYOUT_LANE
  int rounds = 1;                  // CEM-iteration rounds per tick (1 .. kMaxRounds)
  int cost_mode = 1;
  float sq_w[6] = {10.f, 5.f, 0.1f, 0.1f, 1.f, 0.01f};
  long long ticks = 0;
};

namespace {

// Work items of one slot per tick: (theta, 8-window group) in the quad layout, four of them (a
// warp's worth) in the lane layout.
long long slot_items(const spi_server* s, const SlotDesc& d) { return items_of(s->layout, d.N, d.G); }

bool server_busy(const spi_server* s) {
  for (const auto& sl : s->slots)
    if (sl.used) return true;
  return false;
}

void drop_graph(spi_server* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph_src) cudaGraphDestroy(s->graph_src);
  s->graph = nullptr;
  s->graph_src = nullptr;
  for (auto& nd : s->roll_node) nd = nullptr;
}

void free_server(spi_server* s) {
  if (!s) return;
  if (s->stream || s->capture) cudaStreamSynchronize(s->stream);
  for (auto& sl : s->slots) {
    if (sl.mem) cudaFree(sl.mem);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  drop_graph(s);
  if (s->staging_free) cudaEventDestroy(s->staging_free);
  for (auto& ev : s->tick_done) if (ev) cudaEventDestroy(ev);
  if (s->capture) cudaStreamDestroy(s->capture);
  cudaFree(s->d_model); cudaFree(s->d_slots); cudaFree(s->d_order); cudaFree(s->d_info);
  cudaFree(s->d_begin); cudaFree(s->d_rounds);
  cudaFree(s->d_bad); cudaFree(s->d_cem);
  cudaFreeHost(s->h_slots); cudaFreeHost(s->h_order); cudaFreeHost(s->h_info);
  cudaFreeHost(s->h_begin); cudaFreeHost(s->h_rounds);
  cudaFreeHost(s->h_cem_in); cudaFreeHost(s->h_cem_out); cudaFreeHost(s->h_zero);
  delete s;
}

int enqueue_tick(spi_server* s) {
  const int rows = (s->max_samples + 127) / 128;
  cudaError_t ce = cudaSuccess;
  const float* w = s->sq_w;
  for (int r = 0; r < s->rounds; ++r) {
    cem_sample_kernel<<<dim3(rows, s->max_slots), 128, 0, s->stream>>>(s->d_cem, s->d_rounds, r);
    // grid 1 at capture; each tick sets the round's grid on the instantiated graph
    const ItemTables t{s->d_slots, s->d_order, s->d_begin, s->d_info, s->max_slots};
    ce = items_launch(s->layout, s->min_blocks, s->host_model, s->d_model, t, r, 1, s->d_bad, s->stream);
    if (ce != cudaSuccess) return cuda_error(ce, "tick: rollout launch");
    server_finalize_kernel<<<dim3(rows, s->max_slots), 128, 0, s->stream>>>(s->d_slots, s->d_rounds, r, s->cost_mode,
                                                                            w[0], w[1], w[2], w[3], w[4], w[5]);
    cem_refit_kernel<<<s->max_slots, 1024, cem_refit_smem(s->max_samples), s->stream>>>(s->d_cem, s->d_rounds, r);
  }
  ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "tick: launch");
}

int build_graph(spi_server* s) {
  if (s->graph) return SPI_OK;
  cudaStream_t user = s->stream;
  s->stream = s->capture;
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) { s->stream = user; return cuda_error(ce, "server: begin capture"); }
  int rc = enqueue_tick(s);
  ce = cudaStreamEndCapture(s->stream, &g);
  s->stream = user;
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (ce != cudaSuccess) return cuda_error(ce, "server: end capture");
  // the rollout node of each round, by its kernel's round argument
  size_t n = 0;
  ce = cudaGraphGetNodes(g, nullptr, &n);
  std::vector<cudaGraphNode_t> nodes(n);
  if (ce == cudaSuccess && n) ce = cudaGraphGetNodes(g, nodes.data(), &n);
  int found = 0;
  for (size_t i = 0; ce == cudaSuccess && i < n; ++i) {
    cudaGraphNodeType type;
    ce = cudaGraphNodeGetType(nodes[i], &type);
    if (ce != cudaSuccess || type != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams p;
    ce = cudaGraphKernelNodeGetParams(nodes[i], &p);
    if (ce != cudaSuccess || !items_is_rollout_kernel(p.func)) continue;
    const int r = *static_cast<const int*>(p.kernelParams[2]);
    if (r < 0 || r >= s->rounds || s->roll_node[r]) { ce = cudaErrorInvalidValue; break; }
    s->roll_node[r] = nodes[i];
    s->roll_params[r] = p;
    ++found;
  }
  if (ce == cudaSuccess && found != s->rounds) ce = cudaErrorInvalidValue;
  if (ce == cudaSuccess) ce = cudaGraphInstantiate(&s->graph, g, 0);
  if (ce != cudaSuccess) {
    s->graph = nullptr;
    cudaGraphDestroy(g);
    for (auto& nd : s->roll_node) nd = nullptr;
    return cuda_error(ce, "server: graph");
  }
  s->graph_src = g;
  return SPI_OK;
}

int resize_grid(spi_server* s) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const cudaError_t ce = items_occupancy(s->layout, s->min_blocks, &occ);
  if (ce != cudaSuccess) return cuda_error(ce, "server: occupancy");
  s->grid_cap = s->ctas_per_sm > 0 ? sms * std::min(s->ctas_per_sm, std::max(occ, 1)) : 0;
  drop_graph(s);
  return SPI_OK;
}

}  // namespace

extern "C" {

size_t spi_server_job_bytes(const spi_job* job) {
  if (!job || job->W <= 0 || job->H <= 0 || job->cem.n_samples <= 0) return 0;
  return layout_of(job->W, job->H, job->cem.n_samples).total;
}

int spi_server_create(const spi_robot* robot, int max_slots, int max_samples, size_t hbm_budget_bytes,
                      spi_server** out) {
  if (!robot || !out) return set_error(SPI_EINVAL, "spi_server_create: null argument");
  if (max_slots < 1 || max_slots > 4096) return set_error(SPI_EINVAL, "spi_server_create: max_slots %d", max_slots);
  if (max_samples < 2 || max_samples > CEM_MAX_SAMPLES)
    return set_error(SPI_EINVAL, "spi_server_create: max_samples %d outside [2, %d]", max_samples, CEM_MAX_SAMPLES);
  *out = nullptr;
  spi_server* s = new (std::nothrow) spi_server();
  if (!s) return set_error(SPI_ENOMEM, "spi_server_create: host allocation");
  const char* why = "";
  int rc = build_dev_model(*robot, &s->host_model, &why);
  if (rc) { delete s; return set_error(rc, "spi_server_create: %s", why); }
  s->max_slots = max_slots;
  s->max_samples = max_samples;
  s->budget = hbm_budget_bytes;
  s->slots.resize(max_slots);
  cudaError_t ce = cudaSuccess;
#define SRV_TRY(x) do { ce = (x); if (ce != cudaSuccess) { free_server(s); return cuda_error(ce, #x); } } while (0)
  SRV_TRY(cudaMalloc(&s->d_model, sizeof(DevModel)));
  SRV_TRY(cudaMemcpy(s->d_model, &s->host_model, sizeof(DevModel), cudaMemcpyHostToDevice));
  SRV_TRY(cudaMalloc(&s->d_slots, sizeof(SlotDesc) * max_slots));
  SRV_TRY(cudaMemset(s->d_slots, 0, sizeof(SlotDesc) * max_slots));
  SRV_TRY(cudaMalloc(&s->d_order, sizeof(int) * max_slots * kMaxRounds));
  SRV_TRY(cudaMalloc(&s->d_begin, sizeof(long long) * max_slots * kMaxRounds));
  SRV_TRY(cudaMalloc(&s->d_rounds, sizeof(int) * max_slots));
  SRV_TRY(cudaMemset(s->d_rounds, 0, sizeof(int) * max_slots));
  SRV_TRY(cudaMalloc(&s->d_info, sizeof(TickInfo) * kMaxRounds));
  SRV_TRY(cudaMemset(s->d_info, 0, sizeof(TickInfo) * kMaxRounds));
  SRV_TRY(cudaMalloc(&s->d_bad, sizeof(unsigned long long)));
  SRV_TRY(cudaMemset(s->d_bad, 0, sizeof(unsigned long long)));
  SRV_TRY(cudaMalloc(&s->d_cem, sizeof(CemState) * max_slots));
  SRV_TRY(cudaMemset(s->d_cem, 0, sizeof(CemState) * max_slots));
  SRV_TRY(cudaMallocHost(&s->h_slots, sizeof(SlotDesc) * max_slots));
  SRV_TRY(cudaMallocHost(&s->h_order, sizeof(int) * max_slots * kMaxRounds));
  SRV_TRY(cudaMallocHost(&s->h_begin, sizeof(long long) * max_slots * kMaxRounds));
  SRV_TRY(cudaMallocHost(&s->h_rounds, sizeof(int) * max_slots));
  SRV_TRY(cudaMallocHost(&s->h_info, sizeof(TickInfo) * kMaxRounds));
  SRV_TRY(cudaMallocHost(&s->h_cem_in, sizeof(CemState) * max_slots));
  SRV_TRY(cudaMallocHost(&s->h_cem_out, sizeof(CemState) * max_slots));
  SRV_TRY(cudaMallocHost(&s->h_zero, sizeof(int)));
  SRV_TRY(cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking));
  SRV_TRY(cudaEventCreateWithFlags(&s->staging_free, cudaEventDisableTiming));
  SRV_TRY(cudaEventCreateWithFlags(&s->tick_done[0], cudaEventDisableTiming));
  SRV_TRY(cudaEventCreateWithFlags(&s->tick_done[1], cudaEventDisableTiming));
  SRV_TRY(cudaFuncSetAttribute(cem_refit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kCemRefitMaxSmem));
  for (auto& sl : s->slots) SRV_TRY(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
#undef SRV_TRY
  memset(s->h_slots, 0, sizeof(SlotDesc) * max_slots);
  *s->h_zero = 0;
  if ((rc = resize_grid(s))) { free_server(s); return rc; }
  *out = s;
  return SPI_OK;
}

int spi_server_destroy(spi_server* s) {
  free_server(s);
  return SPI_OK;
}

int spi_server_set_stream(spi_server* s, void* stream) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  s->stream = (cudaStream_t)stream;
  return SPI_OK;
}

int spi_server_set_cost(spi_server* s, int mode, const float* sq_weights) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  if (mode != 0 && mode != 1) return set_error(SPI_EINVAL, "spi_server_set_cost: mode %d", mode);
  s->cost_mode = mode;
  if (sq_weights) memcpy(s->sq_w, sq_weights, sizeof(s->sq_w));
  drop_graph(s);
  return SPI_OK;
}

int spi_server_set_work_cap(spi_server* s, long long max_items) {
  if (!s || max_items < 0) return set_error(SPI_EINVAL, "spi_server_set_work_cap: bad argument");
  s->max_items = max_items;
  return SPI_OK;
}

int spi_server_config(spi_server* s, int ctas_per_sm, int items_per_claim) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  if (ctas_per_sm < 0 || items_per_claim < 1 || items_per_claim > 64)
    return set_error(SPI_EINVAL, "spi_server_config: ctas_per_sm %d items_per_claim %d", ctas_per_sm, items_per_claim);
  s->ctas_per_sm = ctas_per_sm;
  s->items_per_claim = items_per_claim;
  return resize_grid(s);
}

int spi_server_set_kernel_config(spi_server* s, int min_blocks) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  const int lo = s->layout == SPI_LAYOUT_LANE ? 2 : 3, hi = 4;
  if (min_blocks < lo || min_blocks > hi)
    return set_error(SPI_EINVAL, "spi_server_set_kernel_config: min_blocks %d outside [%d, %d]", min_blocks, lo, hi);
  s->min_blocks = min_blocks;
  return resize_grid(s);
}

int spi_server_set_rounds(spi_server* s, int rounds) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  if (rounds < 1 || rounds > kMaxRounds)
    return set_error(SPI_EINVAL, "spi_server_set_rounds: rounds %d outside [1, %d]", rounds, kMaxRounds);
  s->rounds = rounds;
  drop_graph(s);
  return SPI_OK;
}

int spi_server_set_kernel_layout(spi_server* s, int layout) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  if (layout != SPI_LAYOUT_QUAD && layout != SPI_LAYOUT_LANE)
    return set_error(SPI_EINVAL, "spi_server_set_kernel_layout: layout %d not 0/1", layout);
  if (server_busy(s))
    return set_error(SPI_ESTATE, "spi_server_set_kernel_layout: jobs in flight");
  if (layout == SPI_LAYOUT_LANE) {
    const cudaError_t ce = items_prepare_lane();
    if (ce != cudaSuccess) return cuda_error(ce, "spi_server_set_kernel_layout: shared-memory attribute");
    s->min_blocks = std::min(std::max(s->min_blocks, 2), 4);
  } else {
    s->min_blocks = std::min(std::max(s->min_blocks, 3), 4);
  }
  s->layout = layout;
  return resize_grid(s);
}

int spi_server_submit(spi_server* s, const spi_job* job, int32_t* slot_out) {
  if (!s || !job || !job->init || !job->actions || !job->target)
    return set_error(SPI_EINVAL, "spi_server_submit: null argument");
  const spi_cem_config& c = job->cem;
  if (job->W <= 0 || job->H <= 0 || job->iterations < 1)
    return set_error(SPI_EINVAL, "spi_server_submit: W=%d H=%d iterations=%d", job->W, job->H, job->iterations);
  if (c.n_samples < 2 || c.n_samples > s->max_samples)
    return set_error(SPI_EINVAL, "spi_server_submit: n_samples %d outside [2, %d]", c.n_samples, s->max_samples);
  if (c.dim < 1 || c.dim > CEM_MAX_DIM) return set_error(SPI_EINVAL, "spi_server_submit: dim %d", c.dim);
  if (!(c.elite_frac > 0.0 && c.elite_frac <= 1.0) || !(c.alpha > 0.0 && c.alpha <= 1.0))
    return set_error(SPI_EINVAL, "spi_server_submit: elite_frac / alpha");
  int slot = -1;
  for (int i = 0; i < s->max_slots; ++i)
    if (!s->slots[i].used) { slot = i; break; }
  const JobLayout L = layout_of(job->W, job->H, c.n_samples);
  if (slot < 0 || s->used + L.total > s->budget)
    return set_error(SPI_EBUDGET, "spi_server_submit: %s (need %zu bytes, %zu free)",
                     slot < 0 ? "no free slot" : "over the HBM budget", L.total, s->budget - s->used);
  CemState& h = s->h_cem_in[slot];
  memset(&h, 0, sizeof(h));
  unsigned seen = 0;
  for (int d = 0; d < c.dim; ++d) {
    const int p = c.param_ids[d];
    if (p < 0 || p >= SPI_THETA_DIM || ((seen >> p) & 1u) || !(c.hi[d] > c.lo[d]))
      return set_error(SPI_EINVAL, "spi_server_submit: parameter %d (slot %d)", d, p);
    seen |= 1u << p;
    h.param_ids[d] = p;
    h.lo[d] = c.lo[d];
    h.hi[d] = c.hi[d];
    h.min_std[d] = c.min_std_frac * (c.hi[d] - c.lo[d]);
    h.mu[d] = 0.5 * (c.lo[d] + c.hi[d]);
    const double w = c.hi[d] - c.lo[d];
    h.cov[d * CEM_MAX_DIM + d] = w * w / 12.0;
    h.L[d * CEM_MAX_DIM + d] = w / std::sqrt(12.0);
  }
  void* mem = nullptr;
  cudaError_t ce = cudaMallocAsync(&mem, L.total, s->stream);
  if (ce != cudaSuccess) { cudaGetLastError(); return set_error(SPI_ENOMEM, "spi_server_submit: %s", cudaGetErrorString(ce)); }
  char* base = static_cast<char*>(mem);
  SlotHost& sl = s->slots[slot];
  SlotDesc& d = sl.desc;
  memset(&d, 0, sizeof(d));
  d.win.init = (float*)(base + L.init);
  d.win.tgt = (float*)(base + L.tgt);
  d.win.weight = (float*)(base + L.weight);
  d.win.act = (float*)(base + L.act);
  d.win.W = job->W;
  d.win.H = job->H;
  d.theta = (float*)(base + L.theta);
  d.partial = (float*)(base + L.partial);
  d.comp = (float*)(base + L.comp);
  d.cost = (float*)(base + L.cost);
  d.N = c.n_samples;
  d.G = (job->W + 7) / 8;
  d.norm = job->norm > 0.f ? job->norm : (float)job->W;
  d.active = 1;
  const long long ns = (long long)job->W * SPI_STATE_DIM;
  srv_rows_to_soa<<<(unsigned)((ns + 255) / 256), 256, 0, s->stream>>>(job->init, (float*)d.win.init, job->W, SPI_STATE_DIM);
  srv_rows_to_soa<<<(unsigned)((ns + 255) / 256), 256, 0, s->stream>>>(job->target, (float*)d.win.tgt, job->W, SPI_STATE_DIM);
  const long long na = (long long)job->W * job->H * 12;
  srv_actions_to_hw<<<(unsigned)((na + 255) / 256), 256, 0, s->stream>>>(job->actions, (float*)d.win.act, job->W, job->H);
  if (job->weight)
    ce = cudaMemcpyAsync((void*)d.win.weight, job->weight, (size_t)job->W * 4, cudaMemcpyDeviceToDevice, s->stream);
  else
    srv_fill<<<(job->W + 255) / 256, 256, 0, s->stream>>>((float*)d.win.weight, 1.0f, job->W);
  memcpy(h.nominal, c.nominal, sizeof(h.nominal));
  memcpy(h.best_theta, c.nominal, sizeof(h.best_theta));
  h.best_cost = INFINITY;
  h.alpha = c.alpha;
  h.dim = c.dim;
  h.n_samples = c.n_samples;
  h.n_elite = std::max(2, (int)std::floor(c.elite_frac * c.n_samples + 0.5));
  h.seed = c.seed;
  h.job = c.job_id;
  h.active = 1;
  h.theta = d.theta;
  h.cost = d.cost;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(s->d_cem + slot, &h, sizeof(CemState), cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    cudaFreeAsync(mem, s->stream);
    return cuda_error(ce, "spi_server_submit: upload");
  }
  sl.used = true;
  sl.active = true;
  sl.retiring = false;
  sl.remaining = job->iterations;
  sl.iterations = job->iterations;
  sl.job_id = c.job_id;
  sl.dim = c.dim;
  sl.bytes = L.total;
  sl.mem = mem;
  s->used += L.total;
  if (slot_out) *slot_out = slot;
  return SPI_OK;
}

int spi_server_tick(spi_server* s) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  // keep the host at most two ticks ahead of the device, so retirements (decided from host
  // counts) and their result copies are observed within a tick of happening
  cudaError_t we = cudaEventSynchronize(s->tick_done[s->ticks & 1]);
  if (we != cudaSuccess) return cuda_error(we, "spi_server_tick: wait");
  // retire finished slots: copy the CEM state out, deactivate, free the slot memory
  for (int i = 0; i < s->max_slots; ++i) {
    SlotHost& sl = s->slots[i];
    if (!sl.active || sl.remaining > 0) continue;
    cudaError_t ce = cudaMemcpyAsync(s->h_cem_out + i, s->d_cem + i, sizeof(CemState), cudaMemcpyDeviceToHost, s->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&s->d_cem[i].active, s->h_zero, sizeof(int), cudaMemcpyHostToDevice, s->stream);
    if (ce == cudaSuccess) ce = cudaEventRecord(sl.done, s->stream);
    if (ce == cudaSuccess) ce = cudaFreeAsync(sl.mem, s->stream);
    if (ce != cudaSuccess) return cuda_error(ce, "spi_server_tick: retire");
    sl.mem = nullptr;
    sl.active = false;
    sl.retiring = true;
    s->used -= sl.bytes;
    sl.desc.active = 0;
  }
  // work layout of this tick: active slots, longest horizon first
  std::vector<int> act;
  for (int i = 0; i < s->max_slots; ++i)
    if (s->slots[i].active) act.push_back(i);
  if (act.empty()) return SPI_OK;
  std::stable_sort(act.begin(), act.end(), [&](int a, int b) {
    return s->slots[a].desc.win.H > s->slots[b].desc.win.H;
  });
  cudaError_t ce = cudaEventSynchronize(s->staging_free);   // previous tick's table copies are done
  if (ce != cudaSuccess) return cuda_error(ce, "spi_server_tick: staging");
  for (int i = 0; i < s->max_slots; ++i) {
    s->h_slots[i] = s->slots[i].desc;
    s->h_slots[i].active = s->slots[i].active ? 1 : 0;
    s->h_rounds[i] = 0;
  }
  // jobs of this tick: shortest remaining work first (remaining iterations x work items x
  // horizon), as many as fit the work cap (at least one); the others stay resident and wait
  auto work = [&](int i) { return slot_items(s, s->h_slots[i]) * (long long)s->h_slots[i].win.H; };
  std::vector<int> run = act;
  if (s->max_items > 0) {
    std::stable_sort(run.begin(), run.end(), [&](int a, int b) {
      return work(a) * (long long)s->slots[a].remaining < work(b) * (long long)s->slots[b].remaining;
    });
    long long items = 0;
    size_t keep = 0;
    for (; keep < run.size(); ++keep) {
      const long long mine = slot_items(s, s->h_slots[run[keep]]);
      if (keep > 0 && items + mine > s->max_items) break;
      items += mine;
    }
    run.resize(keep);
  }
  // rounds per job: the largest running job's work per iteration over its own, at most the
  // rounds of a tick and the iterations it has left
  long long most = 0;
  for (int i : run) most = std::max(most, work(i));
  for (int i : run) {
    const long long mine = std::max(work(i), 1LL);
    const long long share = std::max(most / mine, 1LL);
    s->h_rounds[i] = (int)std::min<long long>(std::min<long long>(share, s->rounds), s->slots[i].remaining);
  }
  for (int r = 0; r < s->rounds; ++r) {
    long long begin = 0;
    int n = 0;
    int* order = s->h_order + (size_t)r * s->max_slots;
    long long* beg = s->h_begin + (size_t)r * s->max_slots;
    for (size_t k = 0; k < act.size(); ++k) {
      const int i = act[k];
      beg[i] = begin;
      if (r >= s->h_rounds[i]) continue;
      begin += slot_items(s, s->h_slots[i]);
      order[n++] = i;
    }
    s->h_info[r].total = begin;
    s->h_info[r].n_order = n;
    // one claim per warp; under a CTA cap a warp's claim grows until the capped grid covers
    // the round
    long long per = s->items_per_claim;
    if (s->grid_cap > 0) per = std::max(per, (begin + 4LL * s->grid_cap - 1) / (4LL * s->grid_cap));
    if (per > 0x7fffffffLL) return set_error(SPI_EINVAL, "spi_server_tick: %lld work items", begin);
    s->h_info[r].items_per_claim = (int)per;
  }
  const size_t tab = (size_t)s->rounds * s->max_slots;
  ce = cudaMemcpyAsync(s->d_slots, s->h_slots, sizeof(SlotDesc) * s->max_slots, cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(s->d_order, s->h_order, sizeof(int) * tab, cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(s->d_begin, s->h_begin, sizeof(long long) * tab, cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(s->d_rounds, s->h_rounds, sizeof(int) * s->max_slots, cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(s->d_info, s->h_info, sizeof(TickInfo) * s->rounds, cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess) ce = cudaEventRecord(s->staging_free, s->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_server_tick: upload table");
  int rc = build_graph(s);
  if (rc) return rc;
  for (int r = 0; r < s->rounds; ++r) {   // one warp per claim of the round's work items
    const long long g = std::max(items_grid(s->h_info[r].total, s->h_info[r].items_per_claim), 1LL);
    if (g > 0x7fffffffLL) return set_error(SPI_EINVAL, "spi_server_tick: %lld work items", s->h_info[r].total);
    cudaKernelNodeParams& p = s->roll_params[r];
    if (p.gridDim.x == (unsigned)g) continue;
    p.gridDim = dim3((unsigned)g);
    ce = cudaGraphExecKernelNodeSetParams(s->graph, s->roll_node[r], &p);
    if (ce != cudaSuccess) return cuda_error(ce, "spi_server_tick: rollout grid");
  }
  ce = cudaGraphLaunch(s->graph, s->stream);
  if (ce == cudaSuccess) ce = cudaEventRecord(s->tick_done[s->ticks & 1], s->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_server_tick: launch");
  for (int i : act) s->slots[i].remaining -= s->h_rounds[i];
  ++s->ticks;
  return SPI_OK;
}

int spi_server_poll(spi_server* s, spi_job_result* results, int max, int32_t* n_done) {
  if (!s || (max > 0 && !results)) return set_error(SPI_EINVAL, "spi_server_poll: null argument");
  int n = 0;
  for (int i = 0; i < s->max_slots && n < max; ++i) {
    SlotHost& sl = s->slots[i];
    if (!sl.retiring) continue;
    cudaError_t q = cudaEventQuery(sl.done);
    if (q == cudaErrorNotReady) continue;
    if (q != cudaSuccess) return cuda_error(q, "spi_server_poll");
    const CemState& st = s->h_cem_out[i];
    spi_job_result& r = results[n++];
    memset(&r, 0, sizeof(r));
    r.job_id = sl.job_id;
    r.iterations = st.iter;
    r.best_cost = st.best_cost;
    memcpy(r.best_theta, st.best_theta, sizeof(r.best_theta));
    r.dim = st.dim;
    for (int d = 0; d < st.dim; ++d) r.mu[d] = st.mu[d];
    r.status = st.status;
    sl.retiring = false;
    sl.used = false;
  }
  if (n_done) *n_done = n;
  return SPI_OK;
}

int spi_server_wait(spi_server* s) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  cudaError_t ce = cudaStreamSynchronize(s->stream);
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_server_wait");
}

int spi_server_stats(spi_server* s, int32_t* active, size_t* bytes_free) {
  if (!s) return set_error(SPI_EINVAL, "null server");
  int a = 0;
  for (const auto& sl : s->slots) a += sl.active ? 1 : 0;
  if (active) *active = a;
  if (bytes_free) *bytes_free = s->budget - s->used;
  return SPI_OK;
}

}  // extern "C"
