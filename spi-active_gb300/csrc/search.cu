// search.cu -- spi_search_*: the device CEM over a caller-scored population.
//
// The engine's CEM (cem.cu) scores its population with spi_run. Some searches score
// candidates with something else: the active-exploration search ranks excitation parameters by
// a Fisher objective (spi_fd_fisher or the sensitivities). spi_search keeps one CEM state on
// the device, draws populations into its own [n][13] buffer with the same sampling kernel and
// refits from costs the caller computed on the device, with the same refit kernel (sort,
// elite mean and covariance in FP64, smoothing, std floor, FP64 Cholesky). It replaces the
// host-side Optuna ask / tell of the reference's excitation search
// (spigym/agents/sysid/active_sysid.py:165-257, CmaEsSampler in
// spigym/config/algo/active_sysid.yaml:20).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "cem.cuh"
#include "common.h"

using namespace spi;

struct spi_search {
  cudaStream_t stream = nullptr;
  DeviceBuf state;    // one CemState
  DeviceBuf pop;      // [n][13]
  DeviceBuf cost;     // [n]
  int n = 0;
  bool sampled = false;
};

extern "C" {

int spi_search_create(const spi_cem_config* c, void* stream, spi_search** out) {
  if (!c || !out) return set_error(SPI_EINVAL, "spi_search_create: null argument");
  *out = nullptr;
  if (c->n_samples < 2 || c->n_samples > CEM_MAX_SAMPLES)
    return set_error(SPI_EINVAL, "spi_search_create: n_samples=%d outside [2, %d]", c->n_samples, CEM_MAX_SAMPLES);
  if (c->dim < 1 || c->dim > CEM_MAX_DIM)
    return set_error(SPI_EINVAL, "spi_search_create: dim=%d outside [1, 13]", c->dim);
  if (!(c->elite_frac > 0.0 && c->elite_frac <= 1.0)) return set_error(SPI_EINVAL, "spi_search_create: elite_frac");
  if (!(c->alpha > 0.0 && c->alpha <= 1.0)) return set_error(SPI_EINVAL, "spi_search_create: alpha in (0, 1]");
  CemState h;
  memset(&h, 0, sizeof(h));
  unsigned used = 0;
  for (int d = 0; d < c->dim; ++d) {
    const int s = c->param_ids[d];
    if (s < 0 || s >= SPI_THETA_DIM || ((used >> s) & 1u))
      return set_error(SPI_EINVAL, "spi_search_create: param_ids[%d]=%d invalid or repeated", d, s);
    used |= 1u << s;
    if (!(c->hi[d] > c->lo[d])) return set_error(SPI_EINVAL, "spi_search_create: empty range for dim %d", d);
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
  spi_search* s = new spi_search();
  s->stream = static_cast<cudaStream_t>(stream);
  s->n = c->n_samples;
  int rc = s->state.reserve(sizeof(CemState));
  if (!rc) rc = s->pop.reserve((size_t)c->n_samples * SPI_THETA_DIM * 4);
  if (!rc) rc = s->cost.reserve((size_t)c->n_samples * 4);
  if (rc) { delete s; return rc; }
  h.theta = s->pop.f();
  h.cost = s->cost.f();
  cudaError_t ce = cudaFuncSetAttribute(cem_refit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kCemRefitMaxSmem);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(s->state.p, &h, sizeof(h), cudaMemcpyHostToDevice, s->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s->stream);   // h lives on this stack
  if (ce != cudaSuccess) { delete s; return cuda_error(ce, "spi_search_create: upload"); }
  *out = s;
  return SPI_OK;
}

int spi_search_destroy(spi_search* s) {
  if (s) {
    if (s->stream) cudaStreamSynchronize(s->stream);
    delete s;
  }
  return SPI_OK;
}

/* Draw the next population into the search's buffer; *population receives its device address
 * ([n][13]: the identified slots sampled, the others at their nominal values). */
int spi_search_sample(spi_search* s, float** population) {
  if (!s) return set_error(SPI_EINVAL, "spi_search_sample: null search");
  const unsigned blocks = (unsigned)((s->n + 127) / 128);
  cem_sample_kernel<<<dim3(blocks, 1), 128, 0, s->stream>>>((const CemState*)s->state.p);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_search_sample");
  s->sampled = true;
  if (population) *population = s->pop.f();
  return SPI_OK;
}

/* Refit from cost device [n] (lower is better) of the last population; iteration += 1. */
int spi_search_refit(spi_search* s, const float* cost) {
  if (!s || !cost) return set_error(SPI_EINVAL, "spi_search_refit: null argument");
  if (!s->sampled) return set_error(SPI_ESTATE, "spi_search_refit before spi_search_sample");
  cudaError_t ce = cudaMemcpyAsync(s->cost.p, cost, (size_t)s->n * 4, cudaMemcpyDeviceToDevice, s->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_search_refit: cost copy");
  cem_refit_kernel<<<1, 1024, cem_refit_smem(s->n), s->stream>>>((CemState*)s->state.p);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_search_refit");
  s->sampled = false;
  return SPI_OK;
}

int spi_search_read(spi_search* s, double* mu, double* cov, float* best, float* best_cost, int32_t* iteration) {
  if (!s) return set_error(SPI_EINVAL, "spi_search_read: null search");
  CemState h;
  cudaError_t ce = cudaStreamSynchronize(s->stream);
  if (ce == cudaSuccess) ce = cudaMemcpy(&h, s->state.p, sizeof(h), cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_search_read");
  const int P = h.dim;
  if (mu) for (int i = 0; i < P; ++i) mu[i] = h.mu[i];
  if (cov) for (int i = 0; i < P; ++i) for (int j = 0; j < P; ++j) cov[i * P + j] = h.cov[i * CEM_MAX_DIM + j];
  if (best) memcpy(best, h.best_theta, sizeof(h.best_theta));
  if (best_cost) *best_cost = h.best_cost;
  if (iteration) *iteration = h.iter;
  return SPI_OK;
}

}  // extern "C"
