// step.cu -- spi_step_states: advance caller-owned states in place by n control steps.
//
// The BaseSimulator-style path of the reference (spigym/simulator/base_simulator/
// base_simulator.py:121-150: apply torques, simulate, refresh the root / dof state tensors),
// driven by actions at the control rate (spigym/envs/legged_base_task/legged_robot_base.py:
// 169-209): each row of `state` [B][37] (pos, quat xyzw, lin vel, ang vel, q, qd; world
// frame) is rolled `steps` control steps under its own theta [B][13] and actions
// [B][steps][12] and written back.
#include <cuda_runtime.h>

#include "engine_impl.h"
#include "rollout.cuh"

using namespace spi;

namespace {

// One lane quad per row.
__global__ void __launch_bounds__(128) step_kernel(const DevModel* __restrict__ model, float* __restrict__ state,
                                                   const float* __restrict__ actions, const float* __restrict__ theta,
                                                   int B, int steps) {
  __shared__ DevModel M;
  load_model_smem(&M, model);
  __syncthreads();
  const int lane = threadIdx.x & 31, leg = lane & 3;
  long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const bool active = row < B;
  if (!active) row = B - 1;
  float* x = state + (size_t)row * SPI_STATE_DIM;
  float th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = theta[(size_t)row * SPI_THETA_DIM + i];
  const BaseParams<float> bp = base_params<float>(M, th);
  const LegParams<float> lp = leg_params<float>(th, leg);
  BaseState<float> Bs;
  LegState<float> L;
  {
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = x[i];
    base_from_world(Bs, s13);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      L.q[k] = x[13 + 3 * leg + k];
      L.qd[k] = x[25 + 3 * leg + k];
    }
  }
  __syncwarp();   // every lane of the quad has read the row before lane 0 overwrites it below
  for (int h = 0; h < steps; ++h) {
    const float* ap = actions + ((size_t)row * steps + h) * 12 + 3 * leg;
    float act[3] = {ap[0], ap[1], ap[2]};
    for (int s = 0; s < M.decimation; ++s) substep(M, leg, Bs, L, bp, lp, act);
  }
  if (!active) return;
  if (leg == 0) {
    float s13[13];
    base_to_world(Bs, s13);
#pragma unroll
    for (int i = 0; i < 13; ++i) x[i] = s13[i];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    x[13 + 3 * leg + k] = L.q[k];
    x[25 + 3 * leg + k] = L.qd[k];
  }
}

}  // namespace

extern "C" int spi_step_states(spi_engine* e, float* state, const float* actions, const float* theta, int B,
                               int steps) {
  if (!e || !state || !actions || !theta) return set_error(SPI_EINVAL, "spi_step_states: null argument");
  if (B <= 0 || steps <= 0) return set_error(SPI_EINVAL, "spi_step_states: B=%d steps=%d", B, steps);
  step_kernel<<<(unsigned)(((long long)B + 31) / 32), 128, 0, e->stream>>>(e->d_model, state, actions, theta, B,
                                                                            steps);
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_step_states");
}
