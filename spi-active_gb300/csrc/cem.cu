// cem.cu -- C ABI of the device CEM (spi_cem_* in spi_engine.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "cem.cuh"
#include "engine_impl.h"

using namespace spi;

namespace {

int cem_sample_impl(spi_engine* e) {
  int rc = refresh_after_realloc(e);
  if (rc) return rc;
  e->N = e->cem_n;
  CemState* st = (CemState*)e->cem.p;
  cem_sample_kernel<<<dim3(blocks_for(e->N, 128), 1), 128, 0, e->stream>>>(st);
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "cem_sample_kernel");
}

int cem_refit_impl(spi_engine* e) {
  cem_refit_kernel<<<1, 1024, cem_refit_smem(e->N), e->stream>>>((CemState*)e->cem.p);
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "cem_refit_kernel");
}

int cem_step_impl(spi_engine* e) {
  int rc = cem_sample_impl(e);
  if (!rc) rc = run_impl(e, nullptr);
  if (!rc) rc = cem_refit_impl(e);
  return rc;
}

}  // namespace

int spi::refresh_after_realloc(spi_engine* e) {
  const unsigned gen = e->theta.generation + e->cost.generation + e->partial.generation + e->comp.generation +
                       e->init.generation + e->act.generation + e->tgt.generation + e->weight.generation;
  if (gen == e->seen_generation) return SPI_OK;
  e->seen_generation = gen;
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  if (!e->cem_ready) return SPI_OK;
  float* ptrs[2] = {e->theta.f(), e->cost.f()};
  CemState* st = (CemState*)e->cem.p;
  cudaError_t ce = cudaMemcpyAsync(&st->theta, &ptrs[0], sizeof(float*), cudaMemcpyHostToDevice, e->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync((void*)&st->cost, &ptrs[1], sizeof(float*), cudaMemcpyHostToDevice, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);   // the host array is on the stack
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "refresh CEM buffer pointers");
}

extern "C" {

int spi_cem_init(spi_engine* e, const spi_cem_config* c) {
  if (!e || !c) return set_error(SPI_EINVAL, "spi_cem_init: null argument");
  if (c->n_samples < 2 || c->n_samples > CEM_MAX_SAMPLES)
    return set_error(SPI_EINVAL, "spi_cem_init: n_samples=%d outside [2, %d]", c->n_samples, CEM_MAX_SAMPLES);
  if (c->dim < 1 || c->dim > CEM_MAX_DIM) return set_error(SPI_EINVAL, "spi_cem_init: dim=%d outside [1, 13]", c->dim);
  if (!(c->elite_frac > 0.0 && c->elite_frac <= 1.0)) return set_error(SPI_EINVAL, "spi_cem_init: elite_frac");
  if (!(c->alpha > 0.0 && c->alpha <= 1.0)) return set_error(SPI_EINVAL, "spi_cem_init: alpha in (0, 1]");
  if (e->W <= 0) return set_error(SPI_ESTATE, "spi_cem_init before spi_load_windows");
  CemState h;
  memset(&h, 0, sizeof(h));
  unsigned used = 0;
  for (int d = 0; d < c->dim; ++d) {
    const int s = c->param_ids[d];
    if (s < 0 || s >= SPI_THETA_DIM || (used >> s) & 1u)
      return set_error(SPI_EINVAL, "spi_cem_init: param_ids[%d]=%d invalid or repeated", d, s);
    used |= 1u << s;
    if (!(c->hi[d] > c->lo[d])) return set_error(SPI_EINVAL, "spi_cem_init: empty prior for dim %d", d);
    h.param_ids[d] = s;
    h.lo[d] = c->lo[d];
    h.hi[d] = c->hi[d];
    h.min_std[d] = c->min_std_frac * (c->hi[d] - c->lo[d]);
    h.mu[d] = 0.5 * (c->lo[d] + c->hi[d]);
    const double w = c->hi[d] - c->lo[d];
    h.cov[d * CEM_MAX_DIM + d] = w * w / 12.0;
    h.L[d * CEM_MAX_DIM + d] = w / std::sqrt(12.0);
  }
  memcpy(h.nominal, c->nominal, sizeof(h.nominal));
  memcpy(h.best_theta, c->nominal, sizeof(h.best_theta));
  h.best_cost = INFINITY;
  h.alpha = c->alpha;
  h.dim = c->dim;
  h.n_samples = c->n_samples;
  h.n_elite = (int)std::floor(c->elite_frac * c->n_samples + 0.5);
  if (h.n_elite < 2) h.n_elite = 2;
  h.seed = c->seed;
  h.job = c->job_id;
  h.active = 1;
  cudaError_t ce = cudaFuncSetAttribute(cem_refit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kCemRefitMaxSmem);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_init: refit shared memory");
  int rc = e->cem.reserve(sizeof(CemState));
  if (rc) return rc;
  if ((rc = e->theta.reserve((size_t)c->n_samples * SPI_THETA_DIM * 4))) return rc;
  const int G = (e->W + 7) / 8;
  if ((rc = e->partial.reserve((size_t)c->n_samples * G * SPI_N_COMP * 4))) return rc;
  if ((rc = e->comp.reserve((size_t)c->n_samples * SPI_N_COMP * 4))) return rc;
  if ((rc = e->cost.reserve((size_t)c->n_samples * 4))) return rc;
  h.theta = e->theta.f();
  h.cost = e->cost.f();
  ce = cudaMemcpyAsync(e->cem.p, &h, sizeof(h), cudaMemcpyHostToDevice, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_init: upload");
  e->N = c->n_samples;
  e->cem_n = c->n_samples;
  e->cem_ready = true;
  if (e->graph_exec) { cudaGraphExecDestroy(e->graph_exec); e->graph_exec = nullptr; }
  e->seen_generation = e->theta.generation + e->cost.generation + e->partial.generation + e->comp.generation +
                       e->init.generation + e->act.generation + e->tgt.generation + e->weight.generation;
  return SPI_OK;
}

int spi_cem_sample(spi_engine* e) {
  if (!e || !e->cem_ready) return set_error(SPI_ESTATE, "spi_cem_sample before spi_cem_init");
  return cem_sample_impl(e);
}

int spi_cem_refit(spi_engine* e) {
  if (!e || !e->cem_ready) return set_error(SPI_ESTATE, "spi_cem_refit before spi_cem_init");
  if (!e->ran) return set_error(SPI_ESTATE, "spi_cem_refit before spi_run");
  return cem_refit_impl(e);
}

int spi_cem_step(spi_engine* e) {
  if (!e || !e->cem_ready) return set_error(SPI_ESTATE, "spi_cem_step before spi_cem_init");
  return cem_step_impl(e);
}

int spi_cem_run(spi_engine* e, int iterations, int use_graph) {
  if (!e || !e->cem_ready) return set_error(SPI_ESTATE, "spi_cem_run before spi_cem_init");
  if (iterations < 0) return set_error(SPI_EINVAL, "spi_cem_run: iterations < 0");
  if (!use_graph) {
    for (int i = 0; i < iterations; ++i) {
      int rc = cem_step_impl(e);
      if (rc) return rc;
    }
    return SPI_OK;
  }
  if (!e->graph_exec) {
    // capture one iteration on a private stream (the engine stream may be the legacy
    // default stream, which cannot be captured), replay it on the engine stream
    if (!e->capture_stream) {
      cudaError_t ce = cudaStreamCreateWithFlags(&e->capture_stream, cudaStreamNonBlocking);
      if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_run: capture stream");
    }
    cudaGraph_t g = nullptr;
    cudaStream_t user = e->stream;
    e->stream = e->capture_stream;
    cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) { e->stream = user; return cuda_error(ce, "spi_cem_run: begin capture"); }
    int rc = cem_step_impl(e);
    ce = cudaStreamEndCapture(e->stream, &g);
    e->stream = user;
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_run: end capture");
    ce = cudaGraphInstantiate(&e->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) { e->graph_exec = nullptr; return cuda_error(ce, "spi_cem_run: instantiate"); }
  }
  for (int i = 0; i < iterations; ++i) {
    cudaError_t ce = cudaGraphLaunch(e->graph_exec, e->stream);
    if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_run: graph launch");
  }
  e->ran = true;
  return SPI_OK;
}

int spi_cem_read(spi_engine* e, double* mu, double* cov, float* best_theta, float* best_cost, int32_t* iteration) {
  if (!e || !e->cem_ready) return set_error(SPI_ESTATE, "spi_cem_read before spi_cem_init");
  CemState h;
  cudaError_t ce = cudaStreamSynchronize(e->stream);
  if (ce == cudaSuccess) ce = cudaMemcpy(&h, e->cem.p, sizeof(h), cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_cem_read");
  const int P = h.dim;
  if (mu) for (int i = 0; i < P; ++i) mu[i] = h.mu[i];
  if (cov) for (int i = 0; i < P; ++i) for (int j = 0; j < P; ++j) cov[i * P + j] = h.cov[i * CEM_MAX_DIM + j];
  if (best_theta) memcpy(best_theta, h.best_theta, sizeof(h.best_theta));
  if (best_cost) *best_cost = h.best_cost;
  if (iteration) *iteration = h.iter;
  return SPI_OK;
}

}  // extern "C"
