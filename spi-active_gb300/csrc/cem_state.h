// cem_state.h -- per-job CEM state kept in device memory.
#pragma once

#include "spi_engine.h"

namespace spi {

constexpr int CEM_MAX_DIM = SPI_THETA_DIM;
constexpr int CEM_MAX_SAMPLES = 16384;

struct CemState {
  double mu[CEM_MAX_DIM];
  double cov[CEM_MAX_DIM * CEM_MAX_DIM];
  double L[CEM_MAX_DIM * CEM_MAX_DIM];
  double lo[CEM_MAX_DIM], hi[CEM_MAX_DIM], min_std[CEM_MAX_DIM];
  double alpha;
  float nominal[SPI_THETA_DIM];
  float best_theta[SPI_THETA_DIM];
  float best_cost;
  int param_ids[CEM_MAX_DIM];
  int dim, n_samples, n_elite, iter, job, status;
  int active;              // 0: slot unused (kernels skip it)
  unsigned long long seed;
  float* theta;            // population [n_samples][13] this state samples into
  const float* cost;       // costs [n_samples] its refit reads
};

}  // namespace spi
