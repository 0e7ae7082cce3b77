// rollout_lane.cuh -- lane-per-rollout layout of the rollout: one lane carries one (theta,
// window) pair through all four legs.
//
// A warp evaluates one theta sample against 32 consecutive windows (four window groups of
// eight). Per physics substep each lane runs phase A for legs FL, FR, RL, RR in turn, adding
// their base contributions, solves the base once (phase B) and runs phase C for the four
// legs. Compared with the quad layout (rollout.cuh) the base solve is not repeated on four
// lanes, no shuffles combine the legs, and every model constant is read at a compile-time
// offset of the kernel's parameter block (the model is passed by value), so the constants
// are operands of the arithmetic instead of shared-memory loads.
//
// The LegWork of legs FL, FR and RL is parked in shared memory ([leg][field][thread]) while
// the later legs and the base solve run; RR's stays in registers.
//
// The error components of each window are formed at the final step, summed over each group
// of eight lanes with xor-shuffles (the same tree as the quad layout's slot sum) and written
// as one partial per (theta, window group): the partial layout, and so finalize_costs, is
// the quad layout's.
#pragma once

#include <cuda_runtime.h>

#include "rollout.cuh"

namespace spi {

__device__ __forceinline__ void add_legout(LegOut<float>& a, const LegOut<float>& b) {
  a.I.A.xx += b.I.A.xx; a.I.A.yy += b.I.A.yy; a.I.A.zz += b.I.A.zz;
  a.I.A.xy += b.I.A.xy; a.I.A.xz += b.I.A.xz; a.I.A.yz += b.I.A.yz;
  a.I.C.xx += b.I.C.xx; a.I.C.yy += b.I.C.yy; a.I.C.zz += b.I.C.zz;
  a.I.C.xy += b.I.C.xy; a.I.C.xz += b.I.C.xz; a.I.C.yz += b.I.C.yz;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) a.I.B.m[i][j] += b.I.B.m[i][j];
  a.p.w = a.p.w + b.p.w;
  a.p.v = a.p.v + b.p.v;
}

// Sum over the eight lanes of a window group (lanes with equal lane >> 3).
__device__ __forceinline__ float group8_sum(float x) {
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  x += __shfl_xor_sync(0xffffffffu, x, 4);
  return x;
}

// Register budget: one lane holds four legs' joint states, the base state and the leg-sum
// accumulators, so everything else lives in shared memory -- each leg's work record (written
// by phase A as it is produced), the control step's actions, and the theta-derived base and
// leg parameters (one copy per warp, all lanes share theta). The __syncwarp() between legs
// keeps the compiler from interleaving the legs' arithmetic, which would need more registers
// than the 168 that three CTAs per SM leave.

// Shared-memory layout per CTA: parking [3 legs][kParkFloats][128 threads], then actions
// [12][128 threads].
constexpr int kLaneParkBytes = (3 * kParkFloats + 12) * 128 * (int)sizeof(float);

// One physics substep of one rollout on one lane. park: this thread's first parking slot
// (stride 128 floats between fields, kParkFloats * 128 between legs); act: this thread's first
// action slot (stride 128); bp / lp: the warp's base and (front, rear) leg parameters.
__device__ __forceinline__ void substep_lane(const DevModel& M, BaseState<float>& B, LegState<float> (&L)[4],
                                             const float* act, float* park, const BaseParams<float>* bp,
                                             const LegParams<float>* lp) {
  LegOut<float> sum;
  LegWork<float> w3;
#pragma unroll
  for (int leg = 0; leg < 4; ++leg) {
    const LegParams<float> P = lp[leg >= 2 ? 1 : 0];
    const float a3[3] = {act[(3 * leg) * 128], act[(3 * leg + 1) * 128], act[(3 * leg + 2) * 128]};
    if (leg < 3) {
      ParkedWork pw{park + leg * kParkFloats * 128, 128};
      LegOut<float> o = phase_a(M, leg, B, L[leg], P, a3, pw);
      if (leg == 0) sum = o; else add_legout(sum, o);
    } else {
      LegOut<float> o = phase_a(M, leg, B, L[leg], P, a3, w3);
      add_legout(sum, o);
    }
    __syncwarp();
  }
  const SV<float> a0 = phase_b(M, *bp, sum, B);
  __syncwarp();
  phase_c(M, 3, a0, w3, L[3]);
#pragma unroll
  for (int leg = 0; leg < 3; ++leg) {
    __syncwarp();
    LegWork<float> lw;
    unpark_legwork(lw, park + leg * kParkFloats * 128, 128);
    phase_c(M, leg, a0, lw, L[leg]);
  }
}

// One warp per (theta n, block of 32 windows); grid covers N * ceil(W / 32) warps; G is the
// number of eight-window groups (ceil(W / 8)) of the partial layout. CTAs of 128 threads with
// kLaneParkBytes of dynamic shared memory.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) rollout_lane_kernel(const __grid_constant__ DevModel M, WinView win,
                                                                 const float* __restrict__ theta, int N, int G,
                                                                 float* __restrict__ partial,
                                                                 unsigned long long* __restrict__ n_bad) {
  extern __shared__ float lane_smem[];               // kLaneParkBytes
  __shared__ BaseParams<float> bp_warp[4];
  __shared__ LegParams<float> lp_warp[4][2];
  const int WB = (win.W + 31) >> 5;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (warp >= (long long)N * WB) return;   // uniform per warp
  const int n = (int)(warp / WB), wb = (int)(warp % WB);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int W = win.W, H = win.H;
  int w = wb * 32 + lane;
  const bool active = w < W;
  if (!active) w = W - 1;

  {
    float th[SPI_THETA_DIM];
    const float* th13 = theta + (size_t)n * SPI_THETA_DIM;
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(th13 + i);
    if (lane == 0) {
      bp_warp[wib] = base_params<float>(M, th);
      lp_warp[wib][0] = leg_params<float>(th, 0);
      lp_warp[wib][1] = leg_params<float>(th, 2);
    }
    __syncwarp();
  }

  BaseState<float> B;
  LegState<float> L[4];
  {
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = __ldg(win.init + i * W + w);
    base_from_world(B, s13);
#pragma unroll
    for (int leg = 0; leg < 4; ++leg)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        L[leg].q[k] = __ldg(win.init + (13 + 3 * leg + k) * W + w);
        L[leg].qd[k] = __ldg(win.init + (25 + 3 * leg + k) * W + w);
      }
  }
  float* park = lane_smem + threadIdx.x;
  float* act = lane_smem + 3 * kParkFloats * 128 + threadIdx.x;
  const int dec = M.decimation;
  for (int h = 0; h < H; ++h) {
    const float4* ap = reinterpret_cast<const float4*>(win.act + ((size_t)h * W + w) * 12);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float4 a = __ldg(ap + i);
      act[(4 * i) * 128] = a.x; act[(4 * i + 1) * 128] = a.y;
      act[(4 * i + 2) * 128] = a.z; act[(4 * i + 3) * 128] = a.w;
    }
    for (int s = 0; s < dec; ++s) substep_lane(M, B, L, act, park, &bp_warp[wib], lp_warp[wib]);
  }
  // final-step error components of this lane's window
  float s13[13];
  base_to_world(B, s13);
  float sp = 0.f, sq = 0.f, sv = 0.f, sw = 0.f, sj = 0.f, sjd = 0.f;
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 13; ++i) {
    const float d = s13[i] - __ldg(win.tgt + i * W + w);
    finite = finite && isfinite(s13[i]);
    if (i < 3) sp += d * d; else if (i < 7) sq += d * d; else if (i < 10) sv += d * d; else sw += d * d;
  }
#pragma unroll
  for (int leg = 0; leg < 4; ++leg)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float dq = L[leg].q[k] - __ldg(win.tgt + (13 + 3 * leg + k) * W + w);
      const float dqd = L[leg].qd[k] - __ldg(win.tgt + (25 + 3 * leg + k) * W + w);
      finite = finite && isfinite(L[leg].q[k]) && isfinite(L[leg].qd[k]);
      sj += dq * dq;
      sjd += dqd * dqd;
    }
  if (active && !finite) atomicAdd(n_bad, 1ull);
  const float wt = active ? __ldg(win.weight + w) : 0.f;
  const float comp[SPI_N_COMP] = {sqrtf(sp), sqrtf(sq), sqrtf(sj), sp, sq, sv, sw, sj, sjd};
  const int g = wb * 4 + (lane >> 3);
  float* out = partial + ((size_t)n * G + g) * SPI_N_COMP;
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) {
    const float v = group8_sum(active ? comp[k] * wt : 0.f);
    if ((lane & 7) == 0 && g < G) out[k] = v;
  }
}

}  // namespace spi
