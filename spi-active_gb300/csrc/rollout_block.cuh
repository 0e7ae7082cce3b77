// rollout_block.cuh -- quad layout with the base solved once per rollout (block layout).
//
// As in the quad layout (rollout.cuh), four lanes carry one rollout, one leg each, eight
// rollouts per warp, one (theta, window group) per warp. The CTA's four warps cooperate on
// the base instead of every lane solving it:
//
//   phase A   every lane: its leg's base contribution (LegOut, 27 floats) -> shared memory
//   barrier
//   phase B   one warp, one lane per rollout of the CTA (32): sums its rollout's four legs
//             in the quad layout's order ((FL + FR) + (RL + RR)), solves and integrates the
//             base, and publishes the base state and acceleration to shared memory; the
//             warp taking the turn rotates with the substep so that every scheduler gets
//             the same share
//   barrier
//   phase C   every lane: its leg's joint accelerations from the published base acceleration
//
// The base state of the CTA's 32 rollouts lives in shared memory; a lane reads the part
// phase A needs (velocity, orientation, height). No shuffles combine the legs, and the 6x6
// base solve runs 32 times per CTA-substep instead of 128 times.
//
// All four warps of a CTA take part in both barriers of every substep, so every warp of
// the grid runs the same number of substeps (one window set, one horizon); warps past the
// last (theta, group) run clamped inputs and write nothing.
#pragma once

#include <cuda_runtime.h>

#include "rollout.cuh"

namespace spi {

constexpr int kLegOutFloats = 27;
constexpr int kLegOutStride = 132;   // 128 threads + 4: the phase-B lanes' reads are conflict-free
constexpr int kBaseFloats = 28;      // p 3, q 4 (xyzw), nu 6 (w, v), R 9, a0 6
constexpr int kBaseParamFloats = 10; // m, h 3, Io 6

struct BlockSmem {
  float4 park[kParkVec * 128];
  float legout[kLegOutFloats * kLegOutStride];
  float base[kBaseFloats * 32];
  float bpar[kBaseParamFloats * 32];
};

__device__ __forceinline__ void store_legout(const LegOut<float>& o, float* p, int stride) {
  const float v[kLegOutFloats] = {o.I.A.xx, o.I.A.yy, o.I.A.zz, o.I.A.xy, o.I.A.xz, o.I.A.yz,
                                  o.I.B.m[0][0], o.I.B.m[0][1], o.I.B.m[0][2],
                                  o.I.B.m[1][0], o.I.B.m[1][1], o.I.B.m[1][2],
                                  o.I.B.m[2][0], o.I.B.m[2][1], o.I.B.m[2][2],
                                  o.I.C.xx, o.I.C.yy, o.I.C.zz, o.I.C.xy, o.I.C.xz, o.I.C.yz,
                                  o.p.w.x, o.p.w.y, o.p.w.z, o.p.v.x, o.p.v.y, o.p.v.z};
#pragma unroll
  for (int f = 0; f < kLegOutFloats; ++f) p[f * stride] = v[f];
}
__device__ __forceinline__ LegOut<float> load_legout(const float* p, int stride) {
  LegOut<float> o;
  o.I.A.xx = p[0]; o.I.A.yy = p[stride]; o.I.A.zz = p[2 * stride];
  o.I.A.xy = p[3 * stride]; o.I.A.xz = p[4 * stride]; o.I.A.yz = p[5 * stride];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.I.B.m[i][j] = p[(6 + 3 * i + j) * stride];
  o.I.C.xx = p[15 * stride]; o.I.C.yy = p[16 * stride]; o.I.C.zz = p[17 * stride];
  o.I.C.xy = p[18 * stride]; o.I.C.xz = p[19 * stride]; o.I.C.yz = p[20 * stride];
  o.p.w = v3(p[21 * stride], p[22 * stride], p[23 * stride]);
  o.p.v = v3(p[24 * stride], p[25 * stride], p[26 * stride]);
  return o;
}
// Sum of two leg contributions, field by field.
__device__ __forceinline__ LegOut<float> legout_sum(const LegOut<float>& a, const LegOut<float>& b) {
  LegOut<float> o = a;
  add_to(o.I, b.I);
  o.p.w = o.p.w + b.p.w;
  o.p.v = o.p.v + b.p.v;
  return o;
}

// Base state of one rollout in the [field][32] table (p, q, nu, R at fields 0..21).
__device__ __forceinline__ void store_base(const BaseState<float>& B, float* p) {
  p[0] = B.p.x; p[32] = B.p.y; p[64] = B.p.z;
  p[96] = B.qx; p[128] = B.qy; p[160] = B.qz; p[192] = B.qw;
  p[224] = B.nu.w.x; p[256] = B.nu.w.y; p[288] = B.nu.w.z;
  p[320] = B.nu.v.x; p[352] = B.nu.v.y; p[384] = B.nu.v.z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) p[(13 + 3 * i + j) * 32] = B.R.m[i][j];
}
__device__ __forceinline__ BaseState<float> load_base(const float* p) {
  BaseState<float> B;
  B.p = v3(p[0], p[32], p[64]);
  B.qx = p[96]; B.qy = p[128]; B.qz = p[160]; B.qw = p[192];
  B.nu.w = v3(p[224], p[256], p[288]);
  B.nu.v = v3(p[320], p[352], p[384]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B.R.m[i][j] = p[(13 + 3 * i + j) * 32];
  return B;
}
// What phase A reads of the base: velocity, orientation and height.
__device__ __forceinline__ BaseState<float> load_base_view(const float* p) {
  BaseState<float> B;
  B.p = v3(0.f, 0.f, p[64]);
  B.qx = 0.f; B.qy = 0.f; B.qz = 0.f; B.qw = 1.f;
  B.nu.w = v3(p[224], p[256], p[288]);
  B.nu.v = v3(p[320], p[352], p[384]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B.R.m[i][j] = p[(13 + 3 * i + j) * 32];
  return B;
}
__device__ __forceinline__ void store_a0(const SV<float>& a, float* p) {
  p[22 * 32] = a.w.x; p[23 * 32] = a.w.y; p[24 * 32] = a.w.z;
  p[25 * 32] = a.v.x; p[26 * 32] = a.v.y; p[27 * 32] = a.v.z;
}
__device__ __forceinline__ SV<float> load_a0(const float* p) {
  SV<float> a;
  a.w = v3(p[22 * 32], p[23 * 32], p[24 * 32]);
  a.v = v3(p[25 * 32], p[26 * 32], p[27 * 32]);
  return a;
}
__device__ __forceinline__ void store_bpar(const BaseParams<float>& b, float* p) {
  p[0] = b.m; p[32] = b.h.x; p[64] = b.h.y; p[96] = b.h.z;
  p[128] = b.Io.xx; p[160] = b.Io.yy; p[192] = b.Io.zz; p[224] = b.Io.xy; p[256] = b.Io.xz; p[288] = b.Io.yz;
}
__device__ __forceinline__ BaseParams<float> load_bpar(const float* p) {
  BaseParams<float> b;
  b.m = p[0]; b.h = v3(p[32], p[64], p[96]);
  b.Io.xx = p[128]; b.Io.yy = p[160]; b.Io.zz = p[192]; b.Io.xy = p[224]; b.Io.xz = p[256]; b.Io.yz = p[288];
  return b;
}

// Global warp index of warp `wi` of this CTA, clamped to the last item; *live = in range.
__device__ __forceinline__ long long block_item(int wi, long long total, bool* live) {
  long long gw = (long long)blockIdx.x * 4 + wi;
  *live = gw < total;
  return *live ? gw : total - 1;
}

// One CTA of 128 threads: four (theta, 8-window group) items, one per warp, as in the quad
// layout, with the base of each rollout solved once (see the file comment).
template <int MINB>
__global__ void __launch_bounds__(128, MINB) rollout_block_kernel(const DevModel* __restrict__ model, WinView win,
                                                                  const float* __restrict__ theta, int N, int G,
                                                                  float* __restrict__ partial,
                                                                  unsigned long long* __restrict__ n_bad) {
  __shared__ DevModel M;
  __shared__ BlockSmem sm;
  load_model_smem(&M, model);
  __syncthreads();
  const int tid = threadIdx.x, wi = tid >> 5, lane = tid & 31, leg = lane & 3, slot = lane >> 2;
  const int W = win.W, H = win.H;
  const long long total = (long long)N * G;

  // Base owner role: lane `lane` of a warp stands for rollout `lane` of the CTA (warp lane >> 3,
  // slot lane & 7). Warp 0 initialises the table.
  if (wi == 0) {
    bool live;
    const long long gw = block_item(lane >> 3, total, &live);
    const int n = (int)(gw / G), g = (int)(gw % G);
    const int w = min(g * 8 + (lane & 7), W - 1);
    float th[SPI_THETA_DIM];
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(theta + (size_t)n * SPI_THETA_DIM + i);
    store_bpar(base_params<float>(M, th), sm.bpar + lane);
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = __ldg(win.init + i * W + w);
    BaseState<float> B;
    base_from_world(B, s13);
    store_base(B, sm.base + lane);
  }

  // Leg role: this lane's leg of rollout rb = wi * 8 + slot.
  bool warp_live;
  const long long gw = block_item(wi, total, &warp_live);
  const int n = (int)(gw / G), g = (int)(gw % G);
  int w = g * 8 + slot;
  const bool active = warp_live && w < W;
  if (w >= W) w = W - 1;
  const int rb = wi * 8 + slot;
  LegParams<float> lp;
  {
    float th[SPI_THETA_DIM];
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(theta + (size_t)n * SPI_THETA_DIM + i);
    lp = leg_params<float>(th, leg);
  }
  LegState<float> L;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    L.q[k] = __ldg(win.init + (13 + 3 * leg + k) * W + w);
    L.qd[k] = __ldg(win.init + (25 + 3 * leg + k) * W + w);
  }
  float* my_legout = sm.legout + tid + (tid >> 5);          // row stride kLegOutStride
  const float* my_base = sm.base + rb;
  ParkedWork pw{sm.park + tid, 128};
  __syncthreads();

  const int dec = M.decimation;
  int sub = blockIdx.x;                                      // rotation offset
  for (int h = 0; h < H; ++h) {
    float act[3];
    const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
    act[0] = __ldg(ap); act[1] = __ldg(ap + 1); act[2] = __ldg(ap + 2);
    for (int s = 0; s < dec; ++s, ++sub) {
      {
        const BaseState<float> Bv = load_base_view(my_base);
        const LegOut<float> o = phase_a(M, leg, Bv, L, lp, act, pw);
        store_legout(o, my_legout, kLegOutStride);
      }
      __syncthreads();
      if (wi == (sub & 3)) {
        // rollout `lane` of the CTA: its four legs are threads (lane >> 3) * 32 + (lane & 7) * 4 + l
        const int t0 = (lane >> 3) * 32 + (lane & 7) * 4;
        const float* lo = sm.legout + t0 + (t0 >> 5);
        const LegOut<float> sum = legout_sum(legout_sum(load_legout(lo, kLegOutStride),
                                                        load_legout(lo + 1, kLegOutStride)),
                                             legout_sum(load_legout(lo + 2, kLegOutStride),
                                                        load_legout(lo + 3, kLegOutStride)));
        BaseState<float> B = load_base(sm.base + lane);
        const SV<float> a0 = phase_b(M, load_bpar(sm.bpar + lane), sum, B);
        store_base(B, sm.base + lane);
        store_a0(a0, sm.base + lane);
      }
      __syncthreads();
      LegWork<float> lw;
      unpark_legwork(lw, sm.park + tid, 128);
      phase_c(M, leg, load_a0(my_base), lw, L);
    }
  }
  // final-step error components (as rollout_group)
  float s13[13];
  base_to_world(load_base(my_base), s13);
  float sp = 0.f, sq = 0.f, sv = 0.f, sw = 0.f, sj = 0.f, sjd = 0.f;
  bool finite = true;
  if (leg == 0) {
#pragma unroll
    for (int i = 0; i < 13; ++i) {
      float d = s13[i] - __ldg(win.tgt + i * W + w);
      finite = finite && isfinite(s13[i]);
      if (i < 3) sp += d * d; else if (i < 7) sq += d * d; else if (i < 10) sv += d * d; else sw += d * d;
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float dq = L.q[k] - __ldg(win.tgt + (13 + 3 * leg + k) * W + w);
    float dqd = L.qd[k] - __ldg(win.tgt + (25 + 3 * leg + k) * W + w);
    finite = finite && isfinite(L.q[k]) && isfinite(L.qd[k]);
    sj += dq * dq;
    sjd += dqd * dqd;
  }
  sp = qsum(sp); sq = qsum(sq); sv = qsum(sv); sw = qsum(sw); sj = qsum(sj); sjd = qsum(sjd);
  const float bad = qsum(finite ? 0.f : 1.f);
  if (active && leg == 0 && bad > 0.f) atomicAdd(n_bad, 1ull);
  const float wt = active ? __ldg(win.weight + w) : 0.f;
  float comp[SPI_N_COMP] = {sqrtf(sp), sqrtf(sq), sqrtf(sj), sp, sq, sv, sw, sj, sjd};
  float* out = partial + ((size_t)n * G + g) * SPI_N_COMP;
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) {
    float v = active ? comp[k] * wt : 0.f;
    v = slot_sum(v);
    if (lane == 0 && warp_live) out[k] = v;
  }
}

}  // namespace spi
