// adjoint.cu -- spi_adjoint: cost and d cost / d theta of every theta sample by the hand-written
// reverse sweep of the rollout (adjoint.cuh), with checkpoints every 5 control steps.
//
// Layout: the quad layout of rollout.cuh (CTAs of 128 threads; four lanes per rollout, one leg
// each; one warp = one theta sample x 8 consecutive windows). Per rollout:
//   1. forward H control steps from the window's start, storing the state (base pose and
//      velocity, joint state: 37 values) before control steps 0, 5, 10, ... in `ckpt`;
//   2. the final state's cost and its adjoint (the engine's cost mode and weights);
//   3. for each 5-step segment, last first: recompute the segment forward from its checkpoint,
//      storing the state before each physics substep in `seg`, then run the substep adjoints
//      backwards over it; the theta adjoint accumulates on the way;
//   4. the window-weighted costs and theta adjoints of the warp's 8 windows are summed (fixed
//      order) into one partial per (theta, window group); adjoint_finalize sums a theta's partials
//      in group order and divides by the window normaliser, as the cost of spi_run does.
// Scratch (engine-owned, component-major [slot][component][rollout] so a warp's accesses are
// contiguous): ckpt ceil(H / 5) x 37 and seg 5 decimation x 37 floats per rollout.
#include <cuda_runtime.h>

#include "adjoint.cuh"
#include "engine_impl.h"
#include "rollout.cuh"

using namespace spi;

namespace {

constexpr int kSegSteps = 5;   // control steps between checkpoints

__device__ __forceinline__ void store_state(float* buf, long long R, long long rid, int leg, const BaseState<float>& B,
                                            const LegState<float>& L) {
  if (leg == 0) {
    const float v[13] = {B.p.x, B.p.y, B.p.z, B.qx, B.qy, B.qz, B.qw,
                         B.nu.w.x, B.nu.w.y, B.nu.w.z, B.nu.v.x, B.nu.v.y, B.nu.v.z};
#pragma unroll
    for (int i = 0; i < 13; ++i) buf[i * R + rid] = v[i];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    buf[(13 + 3 * leg + k) * R + rid] = L.q[k];
    buf[(25 + 3 * leg + k) * R + rid] = L.qd[k];
  }
}
__device__ __forceinline__ void load_state(const float* buf, long long R, long long rid, int leg, BaseState<float>& B,
                                           LegState<float>& L) {
  float v[13];
#pragma unroll
  for (int i = 0; i < 13; ++i) v[i] = buf[i * R + rid];
  B.p = v3(v[0], v[1], v[2]);
  B.qx = v[3]; B.qy = v[4]; B.qz = v[5]; B.qw = v[6];
  B.nu.w = v3(v[7], v[8], v[9]);
  B.nu.v = v3(v[10], v[11], v[12]);
  B.R = quat_to_R(B.qx, B.qy, B.qz, B.qw);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    L.q[k] = buf[(13 + 3 * leg + k) * R + rid];
    L.qd[k] = buf[(25 + 3 * leg + k) * R + rid];
  }
}

__device__ __forceinline__ void qsum_sv(SV<float>& s) { qsum3(s.w); qsum3(s.v); }

// One substep's adjoint on a lane quad (lane = leg): lam / lq / lqd hold the adjoint of the
// state after the substep on entry and of B0 / L0 on exit; gth accumulates the theta adjoint
// (the lane's leg-group slots; lane 0 also the base slots).
__device__ __forceinline__ void substep_adjoint(const DevModel& M, int leg, const BaseState<float>& B0,
                                                const LegState<float>& L0, const BaseParams<float>& bp,
                                                const LegParams<float>& lp, const float* th, const float act[3],
                                                adj::BaseAdj<float>& lam, float lq[3], float lqd[3], float gth[13]) {
  // forward recompute: the leg factorisation, the base articulated inertia, the accelerations
  adj::SolveWork<float> W;
  LegOut<float> o = phase_a(M, leg, B0, L0, lp, act, W);
  qsum_out(o);
  Art<float> IA = rigid(bp.m, bp.h, bp.Io);
  add_to(IA, o.I);
  const SV<float> pA = crf_acc(B0.nu, rigid_mul(bp.m, bp.h, bp.Io, B0.nu), o.p);
  BaseState<float> B1 = B0;
  const SV<float> a0 = base_solve(M, IA, pA, B1);
  float qdd[3];
  adj::leg_qdd(W, a0, qdd);
  // integrator backwards (the base part is the same on the four lanes)
  adj::BaseAdj<float> lam0;
  SV<float> a0b;
  M3<float> R0b = adj::zm3<float>();
  adj::base_integrate_bar(M, B0, B1, lam, lam0, a0b, R0b);
  float qb0[3], qdb0[3], qddb[3];
  adj::leg_integrate_bar(M, lq, lqd, qb0, qdb0, qddb);
  // mu = M'^-1 (a0b; qddb)
  float z[3];
  SV<float> kz = adj::leg_solve_down(W, qddb, z);
  qsum_sv(kz);
  const SV<float> mub = adj::art_solve(IA, adj::sub_sv(a0b, kz));
  float mu[3];
  adj::leg_solve_up(W, z, mub, mu);
  // the residual backwards with the seed mu
  float tgt[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) tgt[k] = joint_target(M, k, leg, act[k]);
  adj::LegTape<float> t;
  float r[3];
  SV<float> fb;
  adj::leg_residual<kMotorRuntime>(M, leg, B0, L0, lp, tgt, a0, qdd, t, r, fb);
  adj::BaseBar<float> bb = adj::zero_base_bar<float>();
  float qb[3] = {0.f, 0.f, 0.f}, qdb[3] = {0.f, 0.f, 0.f};
  adj::LegParamBar<float> pb = {0.f, 0.f, 0.f, 0.f};
  adj::leg_residual_bar<kMotorRuntime>(M, leg, B0, L0, lp, tgt, a0, qdd, t, mu, mub, bb, qb, qdb, pb);
  if (corners_may_touch(M, B0)) {
#pragma unroll
    for (int j = 0; j < 2; ++j) adj::corner_residual_bar(M, B0, lc_corner<float>(M.legc[leg], j), a0, mub, bb);
  }
  if (leg == 0) {
    float mb = 0.f;
    V3<float> hb = adj::z3<float>();
    S3<float> Iob;
    Iob.xx = Iob.yy = Iob.zz = Iob.xy = Iob.xz = Iob.yz = 0.f;
    adj::base_residual_bar(bp, B0, a0, mub, bb, mb, hb, Iob);
    float gb[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    adj::base_params_bar(M, th, mb, hb, Iob, gb);
#pragma unroll
    for (int i = 0; i < 5; ++i) gth[i] -= gb[i];
  }
  // the base adjoints of the four legs (and the base's own terms) summed
  bb.pz = qsum(bb.pz);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) bb.R.m[i][j] = qsum(bb.R.m[i][j]);
  qsum_sv(bb.nu);
  lam0.p.z -= bb.pz;
  lam0.nu = adj::sub_sv(lam0.nu, bb.nu);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) R0b.m[i][j] -= bb.R.m[i][j];
  adj::quat_to_R_bar(B0.qx, B0.qy, B0.qz, B0.qw, R0b, lam0.qx, lam0.qy, lam0.qz, lam0.qw);
  lam = lam0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lq[k] = qb0[k] - qb[k];
    lqd[k] = qdb0[k] - qdb[k];
  }
  const int g = leg >= 2 ? 9 : 5;
  gth[g] -= pb.kps; gth[g + 1] -= pb.fc; gth[g + 2] -= pb.arm; gth[g + 3] -= pb.ts;
}

struct AdjArgs {
  WinView win;
  const float* theta;
  int N, G, mode;
  float w[6];          // squared-error block weights (mode 1)
  float* ckpt;         // [ceil(H / 5)][37][R]
  float* seg;          // [5 decimation][37][R]
  long long R;         // rollouts: N G 8
  float* part_cost;    // [N][G]
  float* part_grad;    // [N][G][13]
  unsigned long long* n_bad;
};

__global__ void __launch_bounds__(128) adjoint_kernel(const DevModel* __restrict__ model, const AdjArgs a) {
  __shared__ DevModel M;
  load_model_smem(&M, model);
  __syncthreads();
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (warp >= (long long)a.N * a.G) return;   // uniform per warp
  const int n = (int)(warp / a.G), g = (int)(warp % a.G);
  const int lane = threadIdx.x & 31, leg = lane & 3;
  const WinView& win = a.win;
  int w = g * 8 + (lane >> 2);
  const bool active = w < win.W;
  if (!active) w = win.W - 1;
  const int W = win.W, H = win.H, dec = M.decimation;
  const long long rid = warp * 8 + (lane >> 2);

  float th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(a.theta + (size_t)n * SPI_THETA_DIM + i);
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
  // 1. forward with checkpoints
  const long long ck_stride = 37 * a.R;
  for (int h = 0; h < H; ++h) {
    if (h % kSegSteps == 0) store_state(a.ckpt + (h / kSegSteps) * ck_stride, a.R, rid, leg, B, L);
    float act[3];
    const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
    act[0] = __ldg(ap); act[1] = __ldg(ap + 1); act[2] = __ldg(ap + 2);
    for (int s = 0; s < dec; ++s) substep(M, leg, B, L, bp, lp, act);
  }
  // 2. final cost and its adjoint
  float s13[13], tg13[13];
  base_to_world(B, s13);
#pragma unroll
  for (int i = 0; i < 13; ++i) tg13[i] = __ldg(win.tgt + i * W + w);
  float d13[13], sb13[13];
#pragma unroll
  for (int i = 0; i < 13; ++i) { d13[i] = s13[i] - tg13[i]; sb13[i] = 0.f; }
  float dq[3], dqd[3], lq[3], lqd[3];
  bool finite = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dq[k] = L.q[k] - __ldg(win.tgt + (13 + 3 * leg + k) * W + w);
    dqd[k] = L.qd[k] - __ldg(win.tgt + (25 + 3 * leg + k) * W + w);
    finite = finite && isfinite(L.q[k]) && isfinite(L.qd[k]);
    lq[k] = 0.f;
    lqd[k] = 0.f;
  }
#pragma unroll
  for (int i = 0; i < 13; ++i) finite = finite && isfinite(s13[i]);
  float cost;
  if (a.mode == 1) {
    const float wq[6] = {a.w[0], a.w[1], a.w[2], a.w[3], a.w[4], a.w[5]};
    float base = 0.f;
#pragma unroll
    for (int i = 0; i < 13; ++i) {
      const float wi = i < 3 ? wq[0] : (i < 7 ? wq[1] : (i < 10 ? wq[2] : wq[3]));
      base += wi * d13[i] * d13[i];
      sb13[i] = 2.f * wi * d13[i];
    }
    float legs = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      legs += wq[4] * dq[k] * dq[k] + wq[5] * dqd[k] * dqd[k];
      lq[k] = 2.f * wq[4] * dq[k];
      lqd[k] = 2.f * wq[5] * dqd[k];
    }
    cost = base + qsum(legs);
  } else {
    float np = 0.f, nq = 0.f, nj = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) np += d13[i] * d13[i];
#pragma unroll
    for (int i = 3; i < 7; ++i) nq += d13[i] * d13[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) nj += dq[k] * dq[k];
    np = sqrtf(np); nq = sqrtf(nq); nj = sqrtf(qsum(nj));
    cost = 10.f * np + 5.f * nq + nj;
#pragma unroll
    for (int i = 0; i < 3; ++i) sb13[i] = np > 0.f ? 10.f * d13[i] / np : 0.f;
#pragma unroll
    for (int i = 3; i < 7; ++i) sb13[i] = nq > 0.f ? 5.f * d13[i] / nq : 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) lq[k] = nj > 0.f ? dq[k] / nj : 0.f;
  }
  const float bad = qsum(finite ? 0.f : 1.f);
  if (active && leg == 0 && bad > 0.f) atomicAdd(a.n_bad, 1ull);
  adj::BaseAdj<float> lam = adj::base_to_world_bar(B, sb13);
  float gth[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) gth[i] = 0.f;
  __syncwarp();   // checkpoints written by lane 0 of each quad are read by all four
  // 3. segments backwards
  const int nseg = (H + kSegSteps - 1) / kSegSteps;
  for (int c = nseg - 1; c >= 0; --c) {
    const int h0 = c * kSegSteps, h1 = min(H, h0 + kSegSteps);
    load_state(a.ckpt + c * ck_stride, a.R, rid, leg, B, L);
    for (int h = h0; h < h1; ++h) {
      float act[3];
      const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
      act[0] = __ldg(ap); act[1] = __ldg(ap + 1); act[2] = __ldg(ap + 2);
      for (int s = 0; s < dec; ++s) {
        store_state(a.seg + ((h - h0) * dec + s) * ck_stride, a.R, rid, leg, B, L);
        substep(M, leg, B, L, bp, lp, act);
      }
    }
    __syncwarp();
    for (int h = h1 - 1; h >= h0; --h) {
      float act[3];
      const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
      act[0] = __ldg(ap); act[1] = __ldg(ap + 1); act[2] = __ldg(ap + 2);
      for (int s = dec - 1; s >= 0; --s) {
        BaseState<float> B0;
        LegState<float> L0;
        load_state(a.seg + ((h - h0) * dec + s) * ck_stride, a.R, rid, leg, B0, L0);
        substep_adjoint(M, leg, B0, L0, bp, lp, th, act, lam, lq, lqd, gth);
      }
    }
    __syncwarp();   // the segment buffer is rewritten by the next segment
  }
  // 4. window-weighted sums over the warp's 8 windows
  const float wt = active ? __ldg(win.weight + w) : 0.f;
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) gth[i] = slot_sum(qsum(gth[i]) * wt);
  cost = slot_sum(leg == 0 ? cost * wt : 0.f);
  if (lane == 0) {
    a.part_cost[(size_t)n * a.G + g] = cost;
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) a.part_grad[((size_t)n * a.G + g) * SPI_THETA_DIM + i] = gth[i];
  }
}

__global__ void adjoint_finalize(const float* __restrict__ part_cost, const float* __restrict__ part_grad, int N,
                                 int G, float norm, float* __restrict__ cost, float* __restrict__ grad) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float c = 0.f, gr[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) gr[i] = 0.f;
  for (int g = 0; g < G; ++g) {
    c += part_cost[(size_t)n * G + g];
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) gr[i] += part_grad[((size_t)n * G + g) * SPI_THETA_DIM + i];
  }
  const float inv = 1.0f / norm;
  if (cost) cost[n] = c * inv;
  if (grad) {
#pragma unroll
    for (int i = 0; i < SPI_THETA_DIM; ++i) grad[(size_t)n * SPI_THETA_DIM + i] = gr[i] * inv;
  }
}

}  // namespace

extern "C" int spi_adjoint(spi_engine* e, const float* theta, int N, float* cost, float* grad) {
  if (!e || !theta) return set_error(SPI_EINVAL, "spi_adjoint: null argument");
  if (N <= 0) return set_error(SPI_EINVAL, "spi_adjoint: N=%d must be > 0", N);
  if (e->W <= 0 || e->H <= 0) return set_error(SPI_ESTATE, "spi_adjoint before spi_load_windows");
  const int G = (e->W + 7) / 8;
  const long long R = (long long)N * G * 8;
  const int nseg = (e->H + kSegSteps - 1) / kSegSteps;
  int rc = e->adj_ckpt.reserve((size_t)nseg * 37 * R * sizeof(float));
  if (!rc) rc = e->adj_seg.reserve((size_t)kSegSteps * e->host_model.decimation * 37 * R * sizeof(float));
  if (!rc) rc = e->adj_part.reserve((size_t)N * G * (SPI_THETA_DIM + 1) * sizeof(float));
  if (rc) return rc;
  AdjArgs a;
  a.win = WinView{e->init.f(), e->act.f(), e->tgt.f(), e->weight.f(), e->W, e->H};
  a.theta = theta;
  a.N = N;
  a.G = G;
  a.mode = e->cost_mode;
  for (int i = 0; i < 6; ++i) a.w[i] = e->sq_w[i];
  a.ckpt = e->adj_ckpt.f();
  a.seg = e->adj_seg.f();
  a.R = R;
  a.part_cost = e->adj_part.f();
  a.part_grad = e->adj_part.f() + (size_t)N * G;
  a.n_bad = (unsigned long long*)e->bad.p;
  adjoint_kernel<<<blocks_for((long long)N * G, 4), 128, 0, e->stream>>>(e->d_model, a);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_adjoint: adjoint_kernel launch");
  adjoint_finalize<<<blocks_for(N, 128), 128, 0, e->stream>>>(a.part_cost, a.part_grad, N, G, e->norm, cost, grad);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_adjoint: finalize launch");
  return SPI_OK;
}
