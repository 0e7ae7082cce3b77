// items.cu -- the rollout kernels shared by the single-job engine and the server.
//
// A launch evaluates the work items of one round of a slot table. Warp k of the grid takes
// items k * per .. k * per + per - 1 (per = the round's items_per_claim), so a launch needs
// items_grid(items, per) CTAs of four warps. A warp finds the slot of an item by binary search
// over the round's slots (laid out in `order`) and evaluates it:
//   quad layout  one (theta, eight-window group) item, four lanes per window (rollout_group);
//   lane layout  four consecutive (theta, eight-window group) items of one slot, one lane per
//                window (rollout_lane_item).
// Results go to the slot's partial[(n G + g)][SPI_N_COMP]; where an item runs does not change
// them. This is the only translation unit that instantiates the rollout for spi_run, the engine
// CEM and spi_server_tick, so the three produce bitwise-identical partials for the same job.
#include <cuda_runtime.h>

#include "items.h"
#include "rollout.cuh"
#include "rollout_lane.cuh"

namespace spi {
namespace {

// Slot of `item`: the last slot in order[0 .. n_order) whose range starts at or before it.
__device__ __forceinline__ int slot_of(const int* order, const long long* begin, int n_order, long long item) {
  int lo = 0, hi = n_order - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (begin[order[mid]] <= item) lo = mid; else hi = mid - 1;
  }
  return order[lo];
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) rollout_quad_kernel(const DevModel* __restrict__ model, ItemTables t,
                                                                 int round, unsigned long long* __restrict__ n_bad) {
  __shared__ DevModel M;
  load_model_smem(&M, model);
  __syncthreads();
  const TickInfo* info = t.info + round;
  const int* order = t.order + (size_t)round * t.max_slots;
  const long long* begin = t.begin + (size_t)round * t.max_slots;
  const long long total = info->total;
  const int n_order = info->n_order, per = info->items_per_claim;
  const long long first = __shfl_sync(0xffffffffu,
                                      ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * per, 0);
  for (int k = 0; k < per; ++k) {
    const long long item = first + k;
    if (item >= total) break;
    const int slot = slot_of(order, begin, n_order, item);
    const SlotDesc& S = t.slots[slot];
    const long long local = item - begin[slot];
    const int n = (int)(local / S.G), g = (int)(local % S.G);
    rollout_group<false>(M, S.win, S.theta + (size_t)n * SPI_THETA_DIM, g,
                         S.partial + ((size_t)n * S.G + g) * SPI_N_COMP, nullptr, n_bad);
  }
}

// CTAs of 128 threads with kLaneParkBytes of dynamic shared memory; the model by value; MS its
// motor shape (motor_shape_of the model, or kMotorRuntime). The round's table is read again
// for each item (after a compiler memory barrier), so no table value holds a register through
// the rollout.
template <int MINB, int MS = kMotorRuntime>
__global__ void __launch_bounds__(128, MINB) rollout_lane_kernel(const __grid_constant__ DevModel M, ItemTables t,
                                                                 int round, unsigned long long* __restrict__ n_bad) {
  extern __shared__ float4 lane_smem[];              // kLaneParkBytes
  __shared__ BaseParams<float> bp_warp[4][4];
  __shared__ float4 gains_warp[4][4][8];
  // the warp's first item, broadcast from lane 0 so that the compiler treats it (and the slot
  // lookups that follow) as warp-uniform
  const long long first = __shfl_sync(0xffffffffu,
                                      ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) *
                                          t.info[round].items_per_claim, 0);
  for (int k = 0;; ++k) {
    const TickInfo* info = t.info + round;
    const long long item = first + k;
    if (k >= info->items_per_claim || item >= info->total) break;
    const int* order = t.order + (size_t)round * t.max_slots;
    const long long* begin = t.begin + (size_t)round * t.max_slots;
    const int slot = slot_of(order, begin, info->n_order, item);
    rollout_lane_item<MS>(M, t.slots + slot, (item - begin[slot]) * 4, n_bad, lane_smem, bp_warp, gains_warp);
    asm volatile("" ::: "memory");
  }
}

__global__ void fill_single_kernel(SingleTable* d, SlotDesc desc, long long items, int per) {
  d->slot = desc;
  d->info.total = items;
  d->info.n_order = 1;
  d->info.items_per_claim = per;
  d->begin = 0;
  d->order = 0;
}

}  // namespace

bool items_is_rollout_kernel(const void* func) {
  const void* k[] = {(const void*)rollout_quad_kernel<3>, (const void*)rollout_quad_kernel<4>,
                     (const void*)rollout_quad_kernel<5>, (const void*)rollout_lane_kernel<2>,
                     (const void*)rollout_lane_kernel<3>, (const void*)rollout_lane_kernel<3, kMotorSpeedLimit>,
                     (const void*)rollout_lane_kernel<4>, (const void*)rollout_lane_kernel<4, kMotorSpeedLimit>};
  for (const void* p : k)
    if (p == func) return true;
  return false;
}

cudaError_t items_prepare_lane() {
  const int b = kLaneParkBytes;
  cudaError_t ce = cudaFuncSetAttribute(rollout_lane_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(rollout_lane_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(rollout_lane_kernel<3, kMotorSpeedLimit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              b);
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(rollout_lane_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(rollout_lane_kernel<4, kMotorSpeedLimit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              b);
  return ce;
}

cudaError_t items_occupancy(int layout, int min_blocks, int* occ) {
  *occ = 0;
  if (layout == SPI_LAYOUT_LANE) {
    if (min_blocks <= 2)
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_lane_kernel<2>, 128, kLaneParkBytes);
    if (min_blocks == 3)
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_lane_kernel<3>, 128, kLaneParkBytes);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_lane_kernel<4>, 128, kLaneParkBytes);
  }
  if (min_blocks <= 3) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_quad_kernel<3>, 128, 0);
  if (min_blocks == 4) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_quad_kernel<4>, 128, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rollout_quad_kernel<5>, 128, 0);
}

cudaError_t items_launch(int layout, int min_blocks, const DevModel& host_model, const DevModel* d_model,
                         const ItemTables& t, int round, int grid, unsigned long long* n_bad, cudaStream_t stream) {
  if (layout == SPI_LAYOUT_LANE) {
    const bool sl = motor_shape_of(host_model) == kMotorSpeedLimit;
    if (min_blocks <= 2)
      rollout_lane_kernel<2><<<grid, 128, kLaneParkBytes, stream>>>(host_model, t, round, n_bad);
    else if (min_blocks == 3 && sl)
      rollout_lane_kernel<3, kMotorSpeedLimit><<<grid, 128, kLaneParkBytes, stream>>>(host_model, t, round, n_bad);
    else if (min_blocks == 3)
      rollout_lane_kernel<3><<<grid, 128, kLaneParkBytes, stream>>>(host_model, t, round, n_bad);
    else if (sl)
      rollout_lane_kernel<4, kMotorSpeedLimit><<<grid, 128, kLaneParkBytes, stream>>>(host_model, t, round, n_bad);
    else
      rollout_lane_kernel<4><<<grid, 128, kLaneParkBytes, stream>>>(host_model, t, round, n_bad);
  } else if (min_blocks <= 3) {
    rollout_quad_kernel<3><<<grid, 128, 0, stream>>>(d_model, t, round, n_bad);
  } else if (min_blocks == 4) {
    rollout_quad_kernel<4><<<grid, 128, 0, stream>>>(d_model, t, round, n_bad);
  } else {
    rollout_quad_kernel<5><<<grid, 128, 0, stream>>>(d_model, t, round, n_bad);
  }
  return cudaGetLastError();
}

cudaError_t items_fill_single(SingleTable* d, const SlotDesc& desc, long long items, int items_per_claim,
                              cudaStream_t stream) {
  fill_single_kernel<<<1, 1, 0, stream>>>(d, desc, items, items_per_claim);
  return cudaGetLastError();
}

}  // namespace spi
