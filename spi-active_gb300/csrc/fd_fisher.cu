// fd_fisher.cu -- spi_fd_fisher: the reference's finite-difference Fisher objective, fused.
//
// The reference scores a candidate excitation by running it on groups of 1 main + P auxiliary
// envs (spigym/envs/sysid/active_sysid_openloop.py:29-80): aux k carries the main's parameters
// with +delta on exploration parameter k. After every control step it adds the reward
// trace(J^T J), J = (s_main - s_aux) / delta over the 13 root-state entries (origin-compensated
// position, xyzw quaternion, world linear and angular velocity) and the 12 joint positions
// (:402-426), and every ksync steps it copies the main's state onto its aux envs (:246-252,
// :316-330). The objective is the reward summed over the episode (active_sysid.py:527-600).
//
// Here one CTA of 128 threads holds 32 rollouts (four lanes each, the quad layout of
// rollout.cuh) and packs whole groups of P + 1 rollouts into them: floor(32 / (P + 1)) groups
// per CTA. Each rollout keeps its state in registers for the whole episode; after each
// control step the rollouts publish their 25 observed values to shared memory, the aux
// rollouts form their squared differences against their main, and the main adds the group's
// reward to its running sum. At a resync step the main publishes its full internal state
// (base pose, velocity and rotation matrix, joint state) and the aux rollouts take it over, so
// the copy is exact. Slots that hold no rollout of a group run a copy of a valid one (every
// lane of a warp must take part in the quad shuffles) and write nothing.
#include <cuda_runtime.h>

#include "engine_impl.h"
#include "rollout.cuh"

using namespace spi;

namespace {

constexpr int kSlots = 32;        // rollouts per CTA of 128 threads
constexpr int kObs = 25;          // root state 13 + joint positions 12
constexpr int kBaseFloats = 22;   // BaseState<float>: p 3, quaternion 4, nu 6, R 9

__device__ __forceinline__ void base_pack(const BaseState<float>& B, float* d) {
  d[0] = B.p.x; d[1] = B.p.y; d[2] = B.p.z;
  d[3] = B.qx; d[4] = B.qy; d[5] = B.qz; d[6] = B.qw;
  d[7] = B.nu.w.x; d[8] = B.nu.w.y; d[9] = B.nu.w.z;
  d[10] = B.nu.v.x; d[11] = B.nu.v.y; d[12] = B.nu.v.z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) d[13 + 3 * i + j] = B.R.m[i][j];
}
__device__ __forceinline__ void base_unpack(BaseState<float>& B, const float* s) {
  B.p = v3(s[0], s[1], s[2]);
  B.qx = s[3]; B.qy = s[4]; B.qz = s[5]; B.qw = s[6];
  B.nu.w = v3(s[7], s[8], s[9]);
  B.nu.v = v3(s[10], s[11], s[12]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B.R.m[i][j] = s[13 + 3 * i + j];
}

struct FdArgs {
  const float* x0;        // [C][37]
  const float* actions;   // [C][T][12]
  const float* theta;     // [C][13] main theta per candidate
  int C, T, P, ksync, skip;
  int ids[SPI_THETA_DIM];
  float delta;
  float* reward_sum;      // [C]
  float* reward_trace;    // [C][T] or null
};

__global__ void __launch_bounds__(128) fd_fisher_kernel(const DevModel* __restrict__ model, const FdArgs a) {
  __shared__ DevModel M;
  __shared__ float obs[kSlots][kObs + 1];
  __shared__ float rew[kSlots];
  __shared__ float xs[kSlots / 2][kBaseFloats + 4 * 6];   // one main state per group (<= 16 groups)
  load_model_smem(&M, model);
  __syncthreads();

  const int G = a.P + 1;                     // rollouts per group
  const int gpc = kSlots / G;                // groups per CTA
  const int lane = threadIdx.x & 31, leg = lane & 3;
  const int slot = threadIdx.x >> 2;         // 0..31
  int grp = slot / G, member = slot % G;
  long long cand = (long long)blockIdx.x * gpc + grp;
  const bool valid = grp < gpc && cand < a.C;
  if (!valid) {                              // a stand-in: the CTA's first group's main
    grp = 0;
    member = 0;
    cand = (long long)blockIdx.x * gpc;
    if (cand >= a.C) cand = a.C - 1;
  }
  const int main_slot = grp * G;

  float th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = a.theta[(size_t)cand * SPI_THETA_DIM + i];
  if (member > 0) th[a.ids[member - 1]] += a.delta;
  const BaseParams<float> bp = base_params<float>(M, th);
  const LegParams<float> lp = leg_params<float>(th, leg);

  BaseState<float> B;
  LegState<float> L;
  {
    const float* x = a.x0 + (size_t)cand * SPI_STATE_DIM;
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = x[i];
    base_from_world(B, s13);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      L.q[k] = x[13 + 3 * leg + k];
      L.qd[k] = x[25 + 3 * leg + k];
    }
  }
  const float inv_delta = 1.0f / a.delta;
  float total = 0.f;
  for (int t = 0; t < a.T; ++t) {
    const float* ap = a.actions + ((size_t)cand * a.T + t) * 12 + 3 * leg;
    const float act[3] = {ap[0], ap[1], ap[2]};
    for (int s = 0; s < M.decimation; ++s) substep(M, leg, B, L, bp, lp, act);
    // publish the observation: root state (world) and joint positions
    if (leg == 0) {
      float s13[13];
      base_to_world(B, s13);
#pragma unroll
      for (int i = 0; i < 13; ++i) obs[slot][i] = s13[i];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) obs[slot][13 + 3 * leg + k] = L.q[k];
    __syncthreads();
    float r = 0.f;
    if (member > 0) {
      if (leg == 0) {
#pragma unroll
        for (int i = 0; i < 13; ++i) {
          const float d = (obs[main_slot][i] - obs[slot][i]) * inv_delta;
          r = fmaf(d, d, r);
        }
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int i = 13 + 3 * leg + k;
        const float d = (obs[main_slot][i] - obs[slot][i]) * inv_delta;
        r = fmaf(d, d, r);
      }
    }
    r = qsum(r);
    if (leg == 0) rew[slot] = (valid && member > 0) ? r : 0.f;
    __syncthreads();
    if (valid && member == 0 && leg == 0) {
      float R = 0.f;
      for (int k = 1; k < G; ++k) R += rew[slot + k];
      if (t >= a.skip) total += R;
      if (a.reward_trace) a.reward_trace[(size_t)cand * a.T + t] = R;
    }
    // resync: aux <- main after 1-based step t + 1 when (t + 1) % ksync == 1 (every step if
    // 0 <= ksync <= 1, never if ksync < 0)
    const int step = t + 1;
    if (a.ksync >= 0 && (a.ksync <= 1 || step % a.ksync == 1)) {
      if (valid && member == 0) {
        float* d = xs[grp];
        if (leg == 0) base_pack(B, d);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          d[kBaseFloats + 6 * leg + k] = L.q[k];
          d[kBaseFloats + 6 * leg + 3 + k] = L.qd[k];
        }
      }
      __syncthreads();
      if (valid && member > 0) {
        const float* s = xs[grp];
        base_unpack(B, s);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          L.q[k] = s[kBaseFloats + 6 * leg + k];
          L.qd[k] = s[kBaseFloats + 6 * leg + 3 + k];
        }
      }
    }
    __syncthreads();   // obs / rew / xs are rewritten next step
  }
  if (valid && member == 0 && leg == 0) a.reward_sum[cand] = total;
}

}  // namespace

extern "C" int spi_fd_fisher(spi_engine* e, const float* x0, const float* actions, const float* theta, int C,
                             int T, const int32_t* param_ids, int P, float delta, int ksync, int skip,
                             float* reward_sum, float* reward_trace) {
  if (!e || !x0 || !actions || !theta || !param_ids || !reward_sum)
    return set_error(SPI_EINVAL, "spi_fd_fisher: null argument");
  if (C <= 0 || T <= 0) return set_error(SPI_EINVAL, "spi_fd_fisher: C=%d T=%d must be > 0", C, T);
  if (P < 1 || P > SPI_THETA_DIM) return set_error(SPI_EINVAL, "spi_fd_fisher: P=%d outside [1, 13]", P);
  if (!(delta != 0.f) || !(delta == delta)) return set_error(SPI_EINVAL, "spi_fd_fisher: delta must be nonzero");
  if (skip < 0 || skip > T) return set_error(SPI_EINVAL, "spi_fd_fisher: skip=%d outside [0, T]", skip);
  FdArgs a;
  a.x0 = x0; a.actions = actions; a.theta = theta;
  a.C = C; a.T = T; a.P = P; a.ksync = ksync; a.skip = skip; a.delta = delta;
  a.reward_sum = reward_sum; a.reward_trace = reward_trace;
  unsigned used = 0;
  for (int k = 0; k < SPI_THETA_DIM; ++k) a.ids[k] = 0;
  for (int k = 0; k < P; ++k) {
    const int s = param_ids[k];
    if (s < 0 || s >= SPI_THETA_DIM || ((used >> s) & 1u))
      return set_error(SPI_EINVAL, "spi_fd_fisher: param_ids[%d]=%d invalid or repeated", k, s);
    used |= 1u << s;
    a.ids[k] = s;
  }
  const int gpc = kSlots / (P + 1);
  const unsigned ctas = (unsigned)(((long long)C + gpc - 1) / gpc);
  fd_fisher_kernel<<<ctas, 128, 0, e->stream>>>(e->d_model, a);
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_fd_fisher");
}
