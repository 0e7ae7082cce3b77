// items.h -- the rollout kernels of the single-job engine and of the server, one compiled copy each.
//
// Both the engine (spi_run, the engine CEM) and the continuous-batching server (spi_server_tick)
// evaluate their (theta, window) pairs with the same kernels, defined once in items.cu: every
// warp takes a work item and looks up, in a slot table, which job the item belongs to. The
// engine is a table of one slot. Because both callers launch
// the same compiled kernel, a job's costs are bitwise identical whether it runs alone on the
// engine or inside the server's mix; two separately compiled copies of the rollout may contract
// different multiply-add pairs into FMAs and differ in the last bit.
#pragma once

#include <cuda_runtime.h>

#include "dynamics.cuh"
#include "rollout.cuh"

namespace spi {

// Work items of one round: slot order[k]'s items are begin[order[k]] .. + items_of(slot).
struct TickInfo {
  long long total;   // work items this round
  int n_order;       // slots in `order`
  int items_per_claim;
};

// Device tables of a launch. Round r reads order[r * max_slots ..], begin[r * max_slots ..]
// and info[r].
struct ItemTables {
  const SlotDesc* slots;
  const int* order;
  const long long* begin;
  const TickInfo* info;
  int max_slots;
};

// A table of one slot in device memory (the single-job engine's).
struct SingleTable {
  SlotDesc slot;
  TickInfo info;
  long long begin;
  int order;
};

// Work items of a job: (theta, eight-window group) pairs in the quad layout, four of them (one
// warp's worth) in the lane layout.
inline long long items_of(int layout, long long N, int G) {
  const long long groups = N * (long long)G;
  return layout == SPI_LAYOUT_LANE ? (groups + 3) / 4 : groups;
}

// Raise the dynamic shared-memory limit of every lane-layout instantiation (once per process).
cudaError_t items_prepare_lane();
// Resident CTAs of 128 threads per SM for (layout, min_blocks).
cudaError_t items_occupancy(int layout, int min_blocks, int* ctas_per_sm);
// CTAs that give every claim of `items` work items (items_per_claim each) its own warp.
inline long long items_grid(long long items, int items_per_claim) {
  const long long claims = (items + items_per_claim - 1) / items_per_claim;
  return (claims + 3) / 4;
}
// Whether `func` is one of the rollout kernels items_launch launches (kernel argument 2 is the
// round).
bool items_is_rollout_kernel(const void* func);
// Launch round `round` of the tables on `grid` CTAs of 128 threads. layout SPI_LAYOUT_QUAD
// (min_blocks 3..5) or SPI_LAYOUT_LANE (min_blocks 2..4); the lane kernel takes the model by
// value, the quad kernel from d_model.
cudaError_t items_launch(int layout, int min_blocks, const DevModel& host_model, const DevModel* d_model,
                         const ItemTables& t, int round, int grid, unsigned long long* n_bad, cudaStream_t stream);
// Write a one-slot table (desc, its item count, per-claim count) on the stream.
cudaError_t items_fill_single(SingleTable* d, const SlotDesc& desc, long long items, int items_per_claim,
                              cudaStream_t stream);
inline ItemTables single_tables(SingleTable* d) {
  return ItemTables{&d->slot, &d->order, &d->begin, &d->info, 1};
}

}  // namespace spi
