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
  int min_blocks = 3;                      // rollout kernel occupancy variant
  int layout = 0;                          // SPI_LAYOUT_QUAD / SPI_LAYOUT_LANE
  spi::DeviceBuf items;                    // one-slot work table of the rollout kernel (items.h)
  // CEM
  spi::DeviceBuf cem;                      // one CemState
  bool cem_ready = false;
  int cem_n = 0;                           // CEM population size
  cudaGraphExec_t graph_exec = nullptr;
  cudaStream_t capture_stream = nullptr;   // graphs are captured here, replayed on `stream`
  unsigned seen_generation = 0;            // buffer generations the graph / CEM pointers refer to
  spi::DeviceBuf sens_ids;                 // sensitivity directions (theta slots)
  spi::DeviceBuf adj_ckpt, adj_seg, adj_part;   // adjoint checkpoints, segment states, partials
  int h_sens_ids[SPI_THETA_DIM] = {0};
};

namespace spi {
int run_impl(spi_engine* e, float* trace);
// Call after any DeviceBuf::reserve of theta / cost / partial / comp / windows: if one of
// them moved, drops the captured CEM graph and points the device CEM state at the new
// theta / cost buffers.
int refresh_after_realloc(spi_engine* e);
inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }
}  // namespace spi
