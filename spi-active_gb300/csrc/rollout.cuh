// rollout.cuh -- warp-level rollout of (theta, window) pairs and the fixed-order cost reduction.
//
// Lane layout (CTAs of 128 threads): four lanes per rollout (lane & 3 = leg FL, FR, RL, RR), eight rollouts per
// warp (lane >> 2 = slot). A warp evaluates one theta sample against eight consecutive
// windows ("window group"). Per physics substep each lane runs phase A for its leg, the
// quad sums the four leg contributions with two xor-shuffles (bitwise identical on all four
// lanes), every lane solves the base (phase B) redundantly, then runs phase C for its leg.
//
// Per window the error components (SPI_N_COMP) are formed at the final step, weighted,
// summed over the warp's eight windows with xor-shuffles and written by lane 0 as one
// partial per (theta, window group). finalize_costs sums the partials of a theta in group
// order, so results do not depend on scheduling.
#pragma once

#include <cuda_runtime.h>

#include "dynamics.cuh"

namespace spi {

// Windows in engine (structure-of-arrays) layout.
struct WinView {
  const float* init;    // [37][W]
  const float* act;     // [H][W][12]
  const float* tgt;     // [37][W]
  const float* weight;  // [W]
  int W, H;
};

// One job's buffers as the rollout kernels (and the server's finalize kernel) see them.
struct SlotDesc {
  WinView win;
  float* theta;     // [N][SPI_THETA_DIM]
  float* partial;   // [N][G][SPI_N_COMP]
  float* comp;      // [N][SPI_N_COMP]
  float* cost;      // [N]
  int N, G;         // theta samples; eight-window groups, ceil(W / 8)
  float norm;
  int active;
};

__device__ __forceinline__ float qsum(float x) {
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  return x;
}
__device__ __forceinline__ void qsum3(V3<float>& v) { v.x = qsum(v.x); v.y = qsum(v.y); v.z = qsum(v.z); }
__device__ __forceinline__ void qsum_s3(S3<float>& s) {
  s.xx = qsum(s.xx); s.yy = qsum(s.yy); s.zz = qsum(s.zz);
  s.xy = qsum(s.xy); s.xz = qsum(s.xz); s.yz = qsum(s.yz);
}
__device__ __forceinline__ void qsum_out(LegOut<float>& o) {
  qsum_s3(o.I.A);
  qsum_s3(o.I.C);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.I.B.m[i][j] = qsum(o.I.B.m[i][j]);
  qsum3(o.p.w);
  qsum3(o.p.v);
}
// Sum over the eight rollouts of a warp (lanes with equal lane & 3).
__device__ __forceinline__ float slot_sum(float x) {
  x += __shfl_xor_sync(0xffffffffu, x, 4);
  x += __shfl_xor_sync(0xffffffffu, x, 8);
  x += __shfl_xor_sync(0xffffffffu, x, 16);
  return x;
}

__device__ __forceinline__ void load_model_smem(DevModel* dst, const DevModel* __restrict__ src) {
  const unsigned* s = reinterpret_cast<const unsigned*>(src);
  unsigned* d = reinterpret_cast<unsigned*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(DevModel) / 4); i += blockDim.x) d[i] = s[i];
}

// Roll one warp's eight windows for theta th13 (13 floats, same for the warp) and write the
// window group's weighted error components to partial9 (lane 0). trace, when non-null, is
// the [W][H][37] block of this theta.
// The LegWork that phase C reads (24 floats: K'[3] 18, y 3, l10 / l20 / l21 3), parked in
// shared memory between phase A and phase C so that its registers are free during the
// reduction and the base solve. It is six float4 fields, two per joint column k:
// (K'_k.w, K'_k.v.x) and (K'_k.v.y, K'_k.v.z, y_k, l_k) with l = (l10, l20, l21); field f of a
// thread lives at p[f * stride], so a warp's 128-bit accesses are conflict-free for stride 128.
constexpr int kParkFloats = 24;
constexpr int kParkVec = kParkFloats / 4;

// Phase A's work record written straight to the parking area as each column is produced, so
// that none of it occupies registers for the rest of phase A.
struct ParkedWork {
  float4* p;
  int stride;
  __device__ __forceinline__ void put_col(int k, const SV<float>& v, float yk, float lk) {
    p[2 * k * stride] = make_float4(v.w.x, v.w.y, v.w.z, v.v.x);
    p[(2 * k + 1) * stride] = make_float4(v.v.y, v.v.z, yk, lk);
  }
};

__device__ __forceinline__ void unpark_legwork(LegWork<float>& W, const float4* src, int stride) {
  float l[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 a = src[2 * k * stride], b = src[(2 * k + 1) * stride];
    W.Kp[k].w = v3(a.x, a.y, a.z);
    W.Kp[k].v = v3(a.w, b.x, b.y);
    W.y[k] = b.z;
    l[k] = b.w;
  }
  W.l10 = l[0]; W.l20 = l[1]; W.l21 = l[2];
}

// One physics substep of a lane quad: phase A (leg), quad reduction, phase B (base solve),
// phase C (leg), with the lane's LegWork parked in shared memory ([field][thread], conflict-
// free) from phase A to phase C. Blocks must be 128 threads. Every kernel of
// the quad layout that steps the dynamics calls this one function.
__device__ __forceinline__ void substep(const DevModel& M, int leg, BaseState<float>& B, LegState<float>& L,
                                        const BaseParams<float>& bp, const LegParams<float>& lp,
                                        const float act[3]) {
  __shared__ float4 lw_smem[kParkVec * 128];
  ParkedWork pw{lw_smem + threadIdx.x, 128};
  LegOut<float> o = phase_a(M, leg, B, L, lp, act, pw);
  qsum_out(o);
  SV<float> a0 = phase_b(M, bp, o, B);
  LegWork<float> lw2;
  unpark_legwork(lw2, lw_smem + threadIdx.x, 128);
  phase_c(M, leg, a0, lw2, L);
}

template <bool TRACE>
__device__ __forceinline__ void rollout_group(const DevModel& M, const WinView& win, const float* th13,
                                              int group, float* partial9, float* trace,
                                              unsigned long long* n_bad) {
  const int lane = threadIdx.x & 31;
  const int leg = lane & 3;
  int w = group * 8 + (lane >> 2);
  const bool active = w < win.W;
  if (!active) w = win.W - 1;
  const int W = win.W, H = win.H;

  float th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(th13 + i);
  const BaseParams<float> bp = base_params<float>(M, th);
  const LegParams<float> lp = leg_params<float>(th, leg);

  BaseState<float> B;
  LegState<float> L;
  {
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = __ldg(win.init + i * W + w);
    base_from_world(B, s13);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      L.q[k] = __ldg(win.init + (13 + 3 * leg + k) * W + w);
      L.qd[k] = __ldg(win.init + (25 + 3 * leg + k) * W + w);
    }
  }
  const int dec = M.decimation;
  for (int h = 0; h < H; ++h) {
    float act[3];
    const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
    act[0] = __ldg(ap); act[1] = __ldg(ap + 1); act[2] = __ldg(ap + 2);
    for (int s = 0; s < dec; ++s) substep(M, leg, B, L, bp, lp, act);
    if (TRACE && active) {
      float* tp = trace + ((size_t)w * H + h) * SPI_STATE_DIM;
      if (leg == 0) {
        float s13[13];
        base_to_world(B, s13);
#pragma unroll
        for (int i = 0; i < 13; ++i) tp[i] = s13[i];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        tp[13 + 3 * leg + k] = L.q[k];
        tp[25 + 3 * leg + k] = L.qd[k];
      }
    }
  }
  // final-step error components
  float s13[13];
  base_to_world(B, s13);
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
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) {
    float v = active ? comp[k] * wt : 0.f;
    v = slot_sum(v);
    if (lane == 0) partial9[k] = v;
  }
}

// One warp per (theta n, window group g); grid covers N * G warps. MINB is the occupancy
// target handed to the register allocator (CTAs of 128 threads per SM): 3 keeps every value in
// registers (168), 4 caps at 128 registers with a few spills; the engine picks one at run time.
template <bool TRACE, int MINB>
__global__ void __launch_bounds__(128, MINB) rollout_kernel(const DevModel* __restrict__ model, WinView win,
                                                      const float* __restrict__ theta, int N, int G,
                                                      float* __restrict__ partial, float* __restrict__ trace,
                                                      unsigned long long* __restrict__ n_bad) {
  __shared__ DevModel M;
  load_model_smem(&M, model);
  __syncthreads();
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (warp >= (long long)N * G) return;   // uniform per warp
  const int n = (int)(warp / G), g = (int)(warp % G);
  float* tr = TRACE ? trace + (size_t)n * win.W * win.H * SPI_STATE_DIM : nullptr;
  rollout_group<TRACE>(M, win, theta + (size_t)n * SPI_THETA_DIM, g,
                       partial + ((size_t)n * G + g) * SPI_N_COMP, tr, n_bad);
}

// comp[n][k] = sum_g partial[n][g][k] / norm; cost from the cost mode. Shared by every
// finalize kernel, with the weighted sum written as explicit fmaf so that the single-job
// engine and the server produce bitwise-identical costs.
__device__ __forceinline__ void finalize_one(const float* __restrict__ partial, int n, int G, float norm, int mode,
                                             const float* w, float* __restrict__ comp, float* __restrict__ cost) {
  float c[SPI_N_COMP];
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) c[k] = 0.f;
  for (int g = 0; g < G; ++g) {
    const float* p = partial + ((size_t)n * G + g) * SPI_N_COMP;
#pragma unroll
    for (int k = 0; k < SPI_N_COMP; ++k) c[k] = __fadd_rn(c[k], p[k]);
  }
  const float inv = __frcp_rn(norm);
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) c[k] = __fmul_rn(c[k], inv);
  if (comp) {
#pragma unroll
    for (int k = 0; k < SPI_N_COMP; ++k) comp[(size_t)n * SPI_N_COMP + k] = c[k];
  }
  if (cost) {
    float v;
    if (mode == 0) {
      v = __fmul_rn(10.f, c[0]);
      v = __fmaf_rn(5.f, c[1], v);
      v = __fadd_rn(v, c[2]);
    } else {
      v = __fmul_rn(w[0], c[3]);
#pragma unroll
      for (int k = 1; k < 6; ++k) v = __fmaf_rn(w[k], c[3 + k], v);
    }
    cost[n] = v;
  }
}

static __global__ void finalize_costs(const float* __restrict__ partial, int N, int G, float norm, int mode,
                                      float w0, float w1, float w2, float w3, float w4, float w5,
                                      float* __restrict__ comp, float* __restrict__ cost) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const float w[6] = {w0, w1, w2, w3, w4, w5};
  finalize_one(partial, n, G, norm, mode, w, comp, cost);
}

}  // namespace spi
