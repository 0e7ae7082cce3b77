// engine.cu -- C ABI of the batched candidate-evaluation engine (declared in spi_engine.h).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "common.h"
#include "engine_impl.h"
#include "items.h"
#include "model.h"
#include "rollout.cuh"
#include "rollout_block.cuh"

using namespace spi;

namespace spi {
thread_local std::string g_last_error;
int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
int cuda_error(cudaError_t e, const char* what) {
  return set_error(SPI_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}
}  // namespace spi

namespace {

__global__ void rows_to_soa(const float* __restrict__ src, float* __restrict__ dst, int W, int F) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)W * F) return;
  const int w = (int)(i / F), f = (int)(i % F);
  dst[(size_t)f * W + w] = src[i];
}
__global__ void actions_to_hw(const float* __restrict__ src, float* __restrict__ dst, int W, int H) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)W * H * 12) return;
  const int j = (int)(i % 12);
  const long long wh = i / 12;
  const int h = (int)(wh % H), w = (int)(wh / H);
  dst[((size_t)h * W + w) * 12 + j] = src[i];
}
__global__ void fill_f32(float* p, float v, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}
}  // namespace

int spi::run_impl(spi_engine* e, float* trace) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  if (e->W <= 0 || e->H <= 0) return set_error(SPI_ESTATE, "spi_run before spi_load_windows");
  if (e->N <= 0) return set_error(SPI_ESTATE, "spi_run before spi_set_theta");
  const int G = (e->W + 7) / 8;
  int rc = e->partial.reserve((size_t)e->N * G * SPI_N_COMP * sizeof(float));
  if (rc) return rc;
  rc = e->comp.reserve((size_t)e->N * SPI_N_COMP * sizeof(float));
  if (rc) return rc;
  rc = e->cost.reserve((size_t)e->N * sizeof(float));
  if (rc) return rc;
  if ((rc = refresh_after_realloc(e))) return rc;
  WinView win{e->init.f(), e->act.f(), e->tgt.f(), e->weight.f(), e->W, e->H};
  const long long warps = (long long)e->N * G;
  const unsigned grid = blocks_for(warps, 4);
  unsigned long long* bad = (unsigned long long*)e->bad.p;
  if (!trace && (e->layout == SPI_LAYOUT_LANE || e->layout == SPI_LAYOUT_QUAD)) {
    // the server's rollout kernel on a table of one slot (items.h), one warp per work item
    SlotDesc d{};
    d.win = win;
    d.theta = e->theta.f();
    d.partial = e->partial.f();
    d.comp = e->comp.f();
    d.cost = e->cost.f();
    d.N = e->N;
    d.G = G;
    d.norm = e->norm;
    d.active = 1;
    const long long items = items_of(e->layout, e->N, G);
    const long long ctas = items_grid(items, 1);
    if (ctas > 0x7fffffffLL) return set_error(SPI_EINVAL, "spi_run: %lld work items", items);
    SingleTable* tab = static_cast<SingleTable*>(e->items.p);
    cudaError_t ce = items_fill_single(tab, d, items, 1, e->stream);
    if (ce == cudaSuccess)
      ce = items_launch(e->layout, e->min_blocks, e->host_model, e->d_model, single_tables(tab), 0, (int)ctas, bad,
                        e->stream);
    if (ce != cudaSuccess) return cuda_error(ce, "rollout launch");
  } else if (!trace && e->layout == SPI_LAYOUT_BLOCK) {
    if (e->min_blocks == 4)
      rollout_block_kernel<4><<<grid, 128, 0, e->stream>>>(e->d_model, win, e->theta.f(), e->N, G,
                                                            e->partial.f(), bad);
    else if (e->min_blocks == 5)
      rollout_block_kernel<5><<<grid, 128, 0, e->stream>>>(e->d_model, win, e->theta.f(), e->N, G,
                                                            e->partial.f(), bad);
    else
      rollout_block_kernel<3><<<grid, 128, 0, e->stream>>>(e->d_model, win, e->theta.f(), e->N, G,
                                                            e->partial.f(), bad);
  } else {
    rollout_kernel<true, 3><<<grid, 128, 0, e->stream>>>(e->d_model, win, e->theta.f(), e->N, G,
                                                         e->partial.f(), trace, bad);
  }
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "rollout_kernel launch");
  const float* w = e->sq_w;
  finalize_costs<<<blocks_for(e->N, 128), 128, 0, e->stream>>>(e->partial.f(), e->N, G, e->norm,
                                                               e->cost_mode, w[0], w[1], w[2], w[3],
                                                               w[4], w[5], e->comp.f(), e->cost.f());
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "finalize_costs launch");
  e->ran = true;
  return SPI_OK;
}

extern "C" {

int spi_abi_version(void) { return SPI_ABI_VERSION; }

const char* spi_last_error(void) { return g_last_error.c_str(); }

int spi_create(const spi_robot* robot, spi_engine** out) {
  if (!robot || !out) return set_error(SPI_EINVAL, "spi_create: null argument");
  *out = nullptr;
  spi_engine* e = new (std::nothrow) spi_engine();
  if (!e) return set_error(SPI_ENOMEM, "spi_create: host allocation failed");
  const char* why = "";
  int rc = build_dev_model(*robot, &e->host_model, &why);
  if (rc) { delete e; return set_error(rc, "spi_create: %s", why); }
  cudaError_t ce = cudaMalloc(&e->d_model, sizeof(DevModel));
  if (ce != cudaSuccess) { delete e; return cuda_error(ce, "spi_create: cudaMalloc(model)"); }
  ce = cudaMemcpy(e->d_model, &e->host_model, sizeof(DevModel), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) { cudaFree(e->d_model); delete e; return cuda_error(ce, "spi_create: upload model"); }
  rc = e->bad.reserve(sizeof(unsigned long long));
  if (!rc) rc = e->items.reserve(sizeof(SingleTable));
  if (rc) { cudaFree(e->d_model); delete e; return rc; }
  cudaMemset(e->bad.p, 0, sizeof(unsigned long long));
  // default kernel: the lane layout at the 168-register cap (the fastest on the C1 workload)
  if ((rc = spi_set_kernel_layout(e, SPI_LAYOUT_LANE)) || (rc = spi_set_kernel_config(e, 3))) {
    spi_destroy(e);
    return rc;
  }
  *out = e;
  return SPI_OK;
}

int spi_destroy(spi_engine* e) {
  if (!e) return SPI_OK;
  if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
  if (e->capture_stream) cudaStreamDestroy(e->capture_stream);
  if (e->d_model) cudaFree(e->d_model);
  delete e;
  return SPI_OK;
}

int spi_set_stream(spi_engine* e, void* stream) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  e->stream = (cudaStream_t)stream;
  return SPI_OK;
}

int spi_load_windows(spi_engine* e, const float* init, const float* actions, const float* target,
                     const float* weight, int W, int H, float norm) {
  if (!e || !init || !actions || !target) return set_error(SPI_EINVAL, "spi_load_windows: null argument");
  if (W <= 0 || H <= 0) return set_error(SPI_EINVAL, "spi_load_windows: W=%d H=%d must be > 0", W, H);
  if ((long long)W * H * 12 > (1ll << 31)) return set_error(SPI_EINVAL, "spi_load_windows: too many window steps");
  int rc;
  if ((rc = e->init.reserve((size_t)W * SPI_STATE_DIM * 4))) return rc;
  if ((rc = e->tgt.reserve((size_t)W * SPI_STATE_DIM * 4))) return rc;
  if ((rc = e->act.reserve((size_t)W * H * 12 * 4))) return rc;
  if ((rc = e->weight.reserve((size_t)W * 4))) return rc;
  if ((rc = refresh_after_realloc(e))) return rc;
  const long long ns = (long long)W * SPI_STATE_DIM;
  rows_to_soa<<<blocks_for(ns, 256), 256, 0, e->stream>>>(init, e->init.f(), W, SPI_STATE_DIM);
  rows_to_soa<<<blocks_for(ns, 256), 256, 0, e->stream>>>(target, e->tgt.f(), W, SPI_STATE_DIM);
  actions_to_hw<<<blocks_for((long long)W * H * 12, 256), 256, 0, e->stream>>>(actions, e->act.f(), W, H);
  if (weight)
    cudaMemcpyAsync(e->weight.p, weight, (size_t)W * 4, cudaMemcpyDeviceToDevice, e->stream);
  else
    fill_f32<<<blocks_for(W, 256), 256, 0, e->stream>>>(e->weight.f(), 1.0f, W);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_load_windows");
  e->W = W;
  e->H = H;
  e->norm = norm > 0.f ? norm : (float)W;
  e->ran = false;
  // a captured CEM iteration bakes in W, H and norm: capture again on next use
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  return SPI_OK;
}

int spi_set_theta(spi_engine* e, const float* theta, int N) {
  if (!e || !theta) return set_error(SPI_EINVAL, "spi_set_theta: null argument");
  if (N <= 0) return set_error(SPI_EINVAL, "spi_set_theta: N=%d must be > 0", N);
  int rc = e->theta.reserve((size_t)N * SPI_THETA_DIM * 4);
  if (rc) return rc;
  if ((rc = refresh_after_realloc(e))) return rc;
  cudaError_t ce = cudaMemcpyAsync(e->theta.p, theta, (size_t)N * SPI_THETA_DIM * 4,
                                   cudaMemcpyDeviceToDevice, e->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_set_theta");
  e->N = N;
  e->ran = false;
  return SPI_OK;
}

int spi_set_kernel_config(spi_engine* e, int min_blocks) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  const int lo = e->layout == SPI_LAYOUT_LANE ? 2 : 3;
  if (min_blocks < lo || min_blocks > 5)
    return set_error(SPI_EINVAL, "spi_set_kernel_config: min_blocks %d outside [%d, 5]", min_blocks, lo);
  e->min_blocks = min_blocks;
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  return SPI_OK;
}

int spi_set_kernel_layout(spi_engine* e, int layout) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  if (layout != SPI_LAYOUT_QUAD && layout != SPI_LAYOUT_LANE && layout != SPI_LAYOUT_BLOCK)
    return set_error(SPI_EINVAL, "spi_set_kernel_layout: layout %d not 0/1/2", layout);
  if (layout == SPI_LAYOUT_LANE) {
    // the parking area is above the 48 KB default for dynamic shared memory
    const cudaError_t ce = items_prepare_lane();
    if (ce != cudaSuccess) return cuda_error(ce, "spi_set_kernel_layout: shared-memory attribute");
  } else if (e->min_blocks < 3) {
    e->min_blocks = 3;
  }
  e->layout = layout;
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  return SPI_OK;
}

int spi_set_cost(spi_engine* e, int mode, const float* sq_weights) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  if (mode != 0 && mode != 1) return set_error(SPI_EINVAL, "spi_set_cost: mode %d not 0/1", mode);
  e->cost_mode = mode;
  if (sq_weights) memcpy(e->sq_w, sq_weights, sizeof(e->sq_w));
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  return SPI_OK;
}

int spi_run(spi_engine* e) { return run_impl(e, nullptr); }

int spi_run_trace(spi_engine* e, float* trace) {
  if (!trace) return set_error(SPI_EINVAL, "spi_run_trace: null trace");
  return run_impl(e, trace);
}

int spi_read_costs(spi_engine* e, float* comp, float* cost) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  if (!e->ran) return set_error(SPI_ESTATE, "spi_read_costs before spi_run");
  cudaError_t ce = cudaSuccess;
  if (comp) ce = cudaMemcpyAsync(comp, e->comp.p, (size_t)e->N * SPI_N_COMP * 4, cudaMemcpyDefault, e->stream);
  if (ce == cudaSuccess && cost) ce = cudaMemcpyAsync(cost, e->cost.p, (size_t)e->N * 4, cudaMemcpyDefault, e->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_read_costs");
  return SPI_OK;
}

int spi_read_theta(spi_engine* e, float* theta) {
  if (!e || !theta) return set_error(SPI_EINVAL, "spi_read_theta: null argument");
  if (e->N <= 0) return set_error(SPI_ESTATE, "spi_read_theta: no theta batch");
  cudaError_t ce = cudaMemcpyAsync(theta, e->theta.p, (size_t)e->N * SPI_THETA_DIM * 4, cudaMemcpyDefault, e->stream);
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_read_theta");
}

int spi_sync(spi_engine* e, int64_t* n_nonfinite) {
  if (!e) return set_error(SPI_EINVAL, "null engine");
  cudaError_t ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_sync");
  if (n_nonfinite) {
    unsigned long long v = 0;
    ce = cudaMemcpy(&v, e->bad.p, sizeof(v), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return cuda_error(ce, "spi_sync: read counter");
    *n_nonfinite = (int64_t)v;
  }
  return SPI_OK;
}

}  // extern "C"
