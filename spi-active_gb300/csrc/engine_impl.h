// engine_impl.h -- the engine object behind the opaque spi_engine handle.
#pragma once

#include <cuda_runtime.h>

#include "cem_state.h"
#include "common.h"
#include "dynamics.cuh"

struct spi_engine {
  spi::DevModel host_model;
  spi::DevModel* d_model = nullptr;
  cudaStream_t stream = nullptr;
  spi::DeviceBuf init, act, tgt, weight;   // windows, structure-of-arrays
  int W = 0, H = 0;
  float norm = 1.f;
  spi::DeviceBuf theta;                    // [N][13]
  int N = 0;
  spi::DeviceBuf partial, comp, cost;      // [N][G][9], [N][9], [N]
  spi::DeviceBuf bad;                      // one unsigned long long
  int cost_mode = 1;
  float sq_w[6] = {10.f, 5.f, 0.1f, 0.1f, 1.f, 0.01f};
  bool ran = false;
  // CEM
  spi::DeviceBuf cem;                      // one CemState
  bool cem_ready = false;
  cudaGraphExec_t graph_exec = nullptr;
  cudaStream_t capture_stream = nullptr;   // graphs are captured here, replayed on `stream`
};

namespace spi {
int run_impl(spi_engine* e, float* trace);
inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }
}  // namespace spi
