// rollout_lane.cuh -- lane-per-rollout layout of the rollout: one lane carries one (theta,
// window) pair through all four legs.
//
// A warp evaluates four (theta, eight-window group) items, one lane per window. Per physics
// substep each lane runs phase A for legs FL, FR, RL, RR in turn, adding
// their base contributions, solves the base once (phase B) and runs phase C for the four
// legs. Compared with the quad layout (rollout.cuh) the base solve is not repeated on four
// lanes and no shuffles combine the legs; the model is passed by value in the kernel's
// parameter block.
//
// The error components of each window are formed at the final step, summed over each group
// of eight lanes with xor-shuffles (the same tree as the quad layout's slot sum) and written
// as one partial per (theta, window group): the partial layout, and so finalize_costs, is
// the quad layout's.
#pragma once

#include <cuda_runtime.h>

#include "rollout.cuh"

namespace spi {

// Sum over the eight lanes of a window group (lanes with equal lane >> 3).
__device__ __forceinline__ float group8_sum(float x) {
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  x += __shfl_xor_sync(0xffffffffu, x, 4);
  return x;
}

// Code size and register budget: the four legs run in a loop that is not unrolled (four
// unrolled copies of phase A overflow the instruction cache), so per-leg data is indexed at run
// time: each leg's joint state, work record and joint targets live in shared memory, and the
// model's per-leg constants are 16-byte loads from the kernel's parameter block (DevModel::legc).
// The theta-derived base parameters and leg gains are one copy per warp (all lanes share
// theta).

// Shared-memory layout per CTA: 16-byte fields, [field][128 threads] throughout, so that each
// warp access is one conflict-free 128-bit load or store per field:
//   parking      4 legs x kParkVec fields;
//   leg state a  4 legs x 1 field: (q0, q1, q2, qd0);
//   targets      4 legs x 1 field: the joint targets of the control step's actions (t0, t1, t2, 0);
//   leg state b  4 legs x one 8-byte field: (qd1, qd2).
// Offsets below are in 16-byte fields of 128 threads. 136 floats per thread, 68 KB per CTA:
// three CTAs (12 warps) per SM.
constexpr int kLaneStateA = 4 * kParkVec;
constexpr int kLaneTargets = kLaneStateA + 4;
constexpr int kLaneStateB = kLaneTargets + 4;
constexpr int kLaneParkBytes = (kLaneStateB + 2) * 128 * (int)sizeof(float4);

// One thread's slots: sm = this thread's first 16-byte field; sb = its first (qd1, qd2) field.
struct LaneSlots {
  float4* sm;
  float2* sb;
  __device__ __forceinline__ static LaneSlots of(float4* lane_smem) {
    return LaneSlots{lane_smem + threadIdx.x, reinterpret_cast<float2*>(lane_smem + kLaneStateB * 128) + threadIdx.x};
  }
  __device__ __forceinline__ LegState<float> leg_state(int leg) const {
    const float4 u = sm[(kLaneStateA + leg) * 128];
    const float2 v = sb[leg * 128];
    LegState<float> L;
    L.q[0] = u.x; L.q[1] = u.y; L.q[2] = u.z;
    L.qd[0] = u.w; L.qd[1] = v.x; L.qd[2] = v.y;
    return L;
  }
  __device__ __forceinline__ void put_leg_state(int leg, const LegState<float>& L) const {
    sm[(kLaneStateA + leg) * 128] = make_float4(L.q[0], L.q[1], L.q[2], L.qd[0]);
    sb[leg * 128] = make_float2(L.qd[1], L.qd[2]);
  }
  __device__ __forceinline__ float4* park(int leg) const { return sm + leg * kParkVec * 128; }
  // the joint targets of the twelve actions of one control step (legs in order)
  __device__ __forceinline__ void put_targets(const DevModel& M, const float4 a0, const float4 a1,
                                              const float4 a2) const {
    const float a[12] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w, a2.x, a2.y, a2.z, a2.w};
    float t[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) t[j] = joint_target(M, j % 3, j / 3, a[j]);
    float4* p = sm + kLaneTargets * 128;
    p[0] = make_float4(t[0], t[1], t[2], 0.f);
    p[128] = make_float4(t[3], t[4], t[5], 0.f);
    p[256] = make_float4(t[6], t[7], t[8], 0.f);
    p[384] = make_float4(t[9], t[10], t[11], 0.f);
  }
};

// A leg's LegGains as two 16-byte fields (kpk 3, lim 3, fc, arm).
__device__ __forceinline__ LegGains<float> load_gains(const float4* g) {
  const float4 a = g[0], b = g[1];
  LegGains<float> r;
  r.kpk[0] = a.x; r.kpk[1] = a.y; r.kpk[2] = a.z;
  r.lim[0] = a.w; r.lim[1] = b.x; r.lim[2] = b.y;
  r.fc = b.z; r.arm = b.w;
  return r;
}
__device__ __forceinline__ void store_gains(const LegGains<float>& r, float4* g) {
  g[0] = make_float4(r.kpk[0], r.kpk[1], r.kpk[2], r.lim[0]);
  g[1] = make_float4(r.lim[1], r.lim[2], r.fc, r.arm);
}

// One physics substep of one rollout on one lane. s: this thread's slots; bp: the warp's base
// parameters; gains: the warp's four legs' LegGains (two fields each).
template <int MS>
__device__ __forceinline__ void substep_lane(const DevModel& M, BaseState<float>& B, const LaneSlots& s,
                                             const BaseParams<float>* bp, const float4* gains) {
  // articulated inertia and bias force at the base: the base body's own, plus each leg's
  LegOut<float> sum = base_terms(*bp, B);
  const float4* tgt = s.sm + kLaneTargets * 128;
  const bool corners = corners_may_touch(M, B);
#pragma unroll 1
  for (int leg = 0; leg < 4; ++leg) {
    const LegGains<float> P = load_gains(gains + 2 * leg);
    const float4 a = tgt[leg * 128];
    const float a3[3] = {a.x, a.y, a.z};
    ParkedWork pw{s.park(leg), 128};
    phase_a_into<MS>(M, leg, B, s.leg_state(leg), P, a3, pw, sum, corners);
  }
  const SV<float> a0 = base_solve(M, sum.I, sum.p, B);
#pragma unroll 1
  for (int leg = 0; leg < 4; ++leg) {
    LegState<float> L = s.leg_state(leg);
    LegWork<float> lw;
    unpark_legwork(lw, s.park(leg), 128);
    phase_c(M, leg, a0, lw, L);
    s.put_leg_state(leg, L);
  }
}

// One warp: four consecutive items of the flattened list of (theta n, eight-window group g)
// pairs of the job S, n * G + g for g < G = ceil(W / 8), starting at item g0; eight lanes per
// item, one window each. Items may belong to different theta samples, so a window set with few
// windows still fills the warp. Writes each item's weighted error components to
// S->partial[(n G + g)][SPI_N_COMP]. lane_smem: the CTA's kLaneParkBytes of dynamic shared
// memory; bp_warp / gains_warp: the CTA's per-warp, per-item parameter slots. MS: the motor
// shape (motor_shape_of the model, or kMotorRuntime). Callable repeatedly by one warp.
//
// S lives in global memory (a slot table). Each field is read where it is needed, and the
// fields used after the control-step loop are read again after a compiler memory barrier, so
// that none of them holds a register through the loop: the loop then compiles as it does with
// the fields in the kernel's parameter block (same FP32 instruction stream, no spills at the
// 128-register cap).
template <int MS = kMotorRuntime>
__device__ __forceinline__ void rollout_lane_item(const DevModel& M, const SlotDesc* S, long long g0,
                                                  unsigned long long* n_bad, float4* lane_smem,
                                                  BaseParams<float> (*bp_warp)[4], float4 (*gains_warp)[4][8]) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, grp = lane >> 3, sub = lane & 7;
  int w;                             // this lane's window (clamped into the set)
  __syncwarp();                      // the warp's previous item has finished with its slots
  {
    const int W = S->win.W, G = S->G;
    const long long items = (long long)S->N * G;
    long long q = g0 + grp;
    if (q >= items) q = items - 1;
    const int n = (int)(q / G), g = (int)(q % G);
    w = min(g * 8 + sub, W - 1);
    const float* theta = S->theta + (size_t)n * SPI_THETA_DIM;
    float th[SPI_THETA_DIM];
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(theta + i);
    if (sub == 0) bp_warp[wib][grp] = base_params<float>(M, th);
    if (sub < 4) store_gains(leg_gains(M, leg_params<float>(th, sub), sub), gains_warp[wib][grp] + 2 * sub);
    __syncwarp();
  }

  const LaneSlots sl = LaneSlots::of(lane_smem);
  BaseState<float> B;
  {
    const float* init = S->win.init;
    const int W = S->win.W;
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = __ldg(init + i * W + w);
    base_from_world(B, s13);
#pragma unroll
    for (int leg = 0; leg < 4; ++leg) {
      LegState<float> L;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        L.q[k] = __ldg(init + (13 + 3 * leg + k) * W + w);
        L.qd[k] = __ldg(init + (25 + 3 * leg + k) * W + w);
      }
      sl.put_leg_state(leg, L);
    }
  }
  {
    const int dec = M.decimation;
    const float* act = S->win.act;
    const int W = S->win.W, H = S->win.H;
    for (int h = 0; h < H; ++h) {
      const float4* ap = reinterpret_cast<const float4*>(act + ((size_t)h * W + w) * 12);
      sl.put_targets(M, __ldg(ap), __ldg(ap + 1), __ldg(ap + 2));
      for (int s = 0; s < dec; ++s) substep_lane<MS>(M, B, sl, &bp_warp[wib][grp], gains_warp[wib][grp]);
    }
  }
  asm volatile("" ::: "memory");     // read the descriptor again below, do not keep it live above
  const int W = S->win.W, G = S->G;
  const long long items = (long long)S->N * G;
  long long q = g0 + grp;
  const bool item_live = q < items;
  if (!item_live) q = items - 1;
  const int n = (int)(q / G), g = (int)(q % G);
  const bool active = item_live && g * 8 + sub < W;
  const float* tgt = S->win.tgt;
  LegState<float> L[4];
#pragma unroll
  for (int leg = 0; leg < 4; ++leg) L[leg] = sl.leg_state(leg);
  // final-step error components of this lane's window
  float s13[13];
  base_to_world(B, s13);
  float sp = 0.f, sq = 0.f, sv = 0.f, sw = 0.f, sj = 0.f, sjd = 0.f;
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 13; ++i) {
    const float d = s13[i] - __ldg(tgt + i * W + w);
    finite = finite && isfinite(s13[i]);
    if (i < 3) sp += d * d; else if (i < 7) sq += d * d; else if (i < 10) sv += d * d; else sw += d * d;
  }
#pragma unroll
  for (int leg = 0; leg < 4; ++leg)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float dq = L[leg].q[k] - __ldg(tgt + (13 + 3 * leg + k) * W + w);
      const float dqd = L[leg].qd[k] - __ldg(tgt + (25 + 3 * leg + k) * W + w);
      finite = finite && isfinite(L[leg].q[k]) && isfinite(L[leg].qd[k]);
      sj += dq * dq;
      sjd += dqd * dqd;
    }
  if (active && !finite) atomicAdd(n_bad, 1ull);
  const float wt = active ? __ldg(S->win.weight + w) : 0.f;
  const float comp[SPI_N_COMP] = {sqrtf(sp), sqrtf(sq), sqrtf(sj), sp, sq, sv, sw, sj, sjd};
  float* out = S->partial + ((size_t)n * G + g) * SPI_N_COMP;
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) {
    const float v = group8_sum(active ? comp[k] * wt : 0.f);
    if (sub == 0 && item_live) out[k] = v;
  }
}

}  // namespace spi
