// sensitivity.cu -- per-window state sensitivities d s_H / d theta and Fisher information.
//
// spi_sensitivity: forward-mode (tangent-linear) derivatives of every window's final state
// with respect to K theta slots, for N theta samples: one lane quad per (sample, window,
// direction), running the templated dynamics with the dual scalar Df (value + one tangent).
// With K <= 13 parameters and a 37-dimensional state, K forward tangents give the whole
// Jacobian J_w (37 x K) of each window -- cheaper than 37 reverse (adjoint) sweeps -- and the
// cost gradient follows as dc/dtheta = (dc/ds_H) J_w without checkpointing.
//
// spi_fisher: F_n = sum_w J_w^T diag(q) J_w (FP32 accumulation), log det(F_n + eps I) and
// trace(F_n) in FP64 -- the active-exploration scores (trace is the reference's objective,
// spigym/envs/sysid/active_sysid_openloop.py:402-426; log det the D-optimal one).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>

#include "dual.cuh"
#include "engine_impl.h"
#include "rollout.cuh"

using namespace spi;

namespace {

__device__ __forceinline__ Df dq_sum(Df x) {
  x.v += __shfl_xor_sync(0xffffffffu, x.v, 1);
  x.d += __shfl_xor_sync(0xffffffffu, x.d, 1);
  x.v += __shfl_xor_sync(0xffffffffu, x.v, 2);
  x.d += __shfl_xor_sync(0xffffffffu, x.d, 2);
  return x;
}
__device__ __forceinline__ void dq_sum_out(LegOut<Df>& o) {
  o.I.A.xx = dq_sum(o.I.A.xx); o.I.A.yy = dq_sum(o.I.A.yy); o.I.A.zz = dq_sum(o.I.A.zz);
  o.I.A.xy = dq_sum(o.I.A.xy); o.I.A.xz = dq_sum(o.I.A.xz); o.I.A.yz = dq_sum(o.I.A.yz);
  o.I.C.xx = dq_sum(o.I.C.xx); o.I.C.yy = dq_sum(o.I.C.yy); o.I.C.zz = dq_sum(o.I.C.zz);
  o.I.C.xy = dq_sum(o.I.C.xy); o.I.C.xz = dq_sum(o.I.C.xz); o.I.C.yz = dq_sum(o.I.C.yz);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.I.B.m[i][j] = dq_sum(o.I.B.m[i][j]);
  o.p.w.x = dq_sum(o.p.w.x); o.p.w.y = dq_sum(o.p.w.y); o.p.w.z = dq_sum(o.p.w.z);
  o.p.v.x = dq_sum(o.p.v.x); o.p.v.y = dq_sum(o.p.v.y); o.p.v.z = dq_sum(o.p.v.z);
}

struct SensArgs {
  const int* param_ids;  // [K] device
  int K;
  int N;
  float* J;              // [N][W][37][K]
  float* xH;             // [N][W][37] or null
};

// One lane quad per (sample n, window w, direction k); 8 quads per warp.
__global__ void __launch_bounds__(128) sensitivity_kernel(const DevModel* __restrict__ model, WinView win,
                                                          const float* __restrict__ theta, SensArgs a) {
  __shared__ DevModel M;
  load_model_smem(&M, model);
  __syncthreads();
  const int lane = threadIdx.x & 31, leg = lane & 3;
  const long long total = (long long)a.N * win.W * a.K;
  long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const bool active = q < total;
  if (!active) q = total - 1;
  const int k = (int)(q % a.K);
  const long long nw = q / a.K;
  const int w = (int)(nw % win.W), n = (int)(nw / win.W);
  const int W = win.W, H = win.H;
  const int slot = a.param_ids[k];

  Df th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i)
    th[i] = Df(__ldg(theta + (size_t)n * SPI_THETA_DIM + i), i == slot ? 1.f : 0.f);
  const BaseParams<Df> bp = base_params<Df>(M, th);
  const LegParams<Df> lp = leg_params<Df>(th, leg);
  BaseState<Df> B;
  LegState<Df> L;
  {
    Df s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = Df(__ldg(win.init + i * W + w));
    base_from_world(B, s13);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      L.q[j] = Df(__ldg(win.init + (13 + 3 * leg + j) * W + w));
      L.qd[j] = Df(__ldg(win.init + (25 + 3 * leg + j) * W + w));
    }
  }
  for (int h = 0; h < H; ++h) {
    const float* ap = win.act + ((size_t)h * W + w) * 12 + 3 * leg;
    Df act[3] = {Df(__ldg(ap)), Df(__ldg(ap + 1)), Df(__ldg(ap + 2))};
    for (int s = 0; s < M.decimation; ++s) {
      LegWork<Df> lw;
      LegOut<Df> o = phase_a(M, leg, B, L, lp, act, lw);
      dq_sum_out(o);
      SV<Df> a0 = phase_b(M, bp, o, B);
      phase_c(M, leg, a0, lw, L);
    }
  }
  if (!active) return;
  Df s13[13];
  base_to_world(B, s13);
  float* Jp = a.J + (((size_t)n * W + w) * SPI_STATE_DIM) * a.K + k;
  float* xp = a.xH ? a.xH + ((size_t)n * W + w) * SPI_STATE_DIM : nullptr;
  if (leg == 0) {
#pragma unroll
    for (int i = 0; i < 13; ++i) {
      Jp[(size_t)i * a.K] = s13[i].d;
      if (xp && k == 0) xp[i] = s13[i].v;
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Jp[(size_t)(13 + 3 * leg + j) * a.K] = L.q[j].d;
    Jp[(size_t)(25 + 3 * leg + j) * a.K] = L.qd[j].d;
    if (xp && k == 0) {
      xp[13 + 3 * leg + j] = L.q[j].v;
      xp[25 + 3 * leg + j] = L.qd[j].v;
    }
  }
}

// F[n] = sum_w J^T diag(q) J (K x K, FP32 accumulation); one CTA per sample.
__global__ void fisher_kernel(const float* __restrict__ J, int N, int W, int K, const float* __restrict__ q,
                              float* __restrict__ F) {
  const int n = blockIdx.x;
  const int nent = K * K;
  for (int e = threadIdx.x; e < nent; e += blockDim.x) {
    const int p = e / K, r = e % K;
    if (r < p) continue;
    float acc = 0.f;
    for (int w = 0; w < W; ++w) {
      const float* Jw = J + (((size_t)n * W + w) * SPI_STATE_DIM) * K;
#pragma unroll 1
      for (int i = 0; i < SPI_STATE_DIM; ++i) acc += (q ? q[i] : 1.f) * Jw[i * K + p] * Jw[i * K + r];
    }
    F[(size_t)n * nent + p * K + r] = acc;
    F[(size_t)n * nent + r * K + p] = acc;
  }
}

// F[n] = sum_w J^T diag(q) J on tensor cores: one warp per sample, BF16 operands, FP32
// accumulation, mma.sync m16n8k16 (A = (Q^1/2 J)^T as a 16 x 16 row-major tile, B = Q^1/2 J as a
// 16 x 8 column-major tile, two n-tiles cover the 16 padded parameters). Rows of J are consumed
// 16 at a time; rows past W * 37 and parameters past K are zero.
__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}
__device__ __forceinline__ float jq(const float* __restrict__ Jn, const float* __restrict__ q, int rows, int K,
                                    int r, int p) {
  if (r >= rows || p >= K) return 0.f;
  const float w = q ? sqrtf(q[r % SPI_STATE_DIM]) : 1.f;
  return w * Jn[(size_t)r * K + p];
}
__global__ void fisher_mma_kernel(const float* __restrict__ J, int N, int W, int K, const float* __restrict__ q,
                                  float* __restrict__ F) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= N) return;                        // uniform per warp
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const float* Jn = J + (size_t)warp * W * SPI_STATE_DIM * K;
  const int rows = W * SPI_STATE_DIM;
  float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = 0; k0 < rows; k0 += 16) {
    // A[m][k] = Jq[k0 + k][m]: rows m = g, g + 8; cols k = 2t, 2t + 1, 2t + 8, 2t + 9
    const unsigned a0 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t, g), jq(Jn, q, rows, K, k0 + 2 * t + 1, g));
    const unsigned a1 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t, g + 8), jq(Jn, q, rows, K, k0 + 2 * t + 1, g + 8));
    const unsigned a2 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t + 8, g), jq(Jn, q, rows, K, k0 + 2 * t + 9, g));
    const unsigned a3 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t + 8, g + 8),
                                  jq(Jn, q, rows, K, k0 + 2 * t + 9, g + 8));
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      // B[k][n] = Jq[k0 + k][8 nt + n]: k = 2t, 2t + 1 (b0) and 2t + 8, 2t + 9 (b1); n = g
      const int n = 8 * nt + g;
      const unsigned b0 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t, n), jq(Jn, q, rows, K, k0 + 2 * t + 1, n));
      const unsigned b1 = pack_bf16(jq(Jn, q, rows, K, k0 + 2 * t + 8, n), jq(Jn, q, rows, K, k0 + 2 * t + 9, n));
      float* c = nt ? c1 : c0;
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};\n"
          : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
  }
  // D fragment: rows g and g + 8, cols 2t and 2t + 1 of each n-tile
  float* Fn = F + (size_t)warp * K * K;
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) {
    const float* c = nt ? c1 : c0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int m = g + (e >= 2 ? 8 : 0), n = 8 * nt + 2 * t + (e & 1);
      if (m < K && n < K) Fn[m * K + n] = c[e];
    }
  }
}

// log det(F + eps I) by FP64 Cholesky, and trace(F); one thread per sample.
__global__ void logdet_kernel(const float* __restrict__ F, int N, int K, double eps, double* __restrict__ logdet,
                              double* __restrict__ trace) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double L[SPI_THETA_DIM * SPI_THETA_DIM];
  const float* f = F + (size_t)n * K * K;
  double ld = 0.0, tr = 0.0;
  bool ok = true;
  for (int j = 0; j < K; ++j) {
    double d = (double)f[j * K + j] + eps;
    tr += (double)f[j * K + j];
    for (int k = 0; k < j; ++k) d -= L[j * K + k] * L[j * K + k];
    if (!(d > 0.0)) { ok = false; break; }
    const double ljj = sqrt(d);
    L[j * K + j] = ljj;
    ld += 2.0 * log(ljj);
    for (int i = j + 1; i < K; ++i) {
      double s = (double)f[i * K + j];
      for (int k = 0; k < j; ++k) s -= L[i * K + k] * L[j * K + k];
      L[i * K + j] = s / ljj;
    }
  }
  if (logdet) logdet[n] = ok ? ld : -INFINITY;
  if (trace) trace[n] = tr;
}

}  // namespace

extern "C" {

int spi_sensitivity(spi_engine* e, const float* theta, int N, const int32_t* param_ids, int K, float* J, float* xH) {
  if (!e || !theta || !param_ids || !J) return set_error(SPI_EINVAL, "spi_sensitivity: null argument");
  if (e->W <= 0) return set_error(SPI_ESTATE, "spi_sensitivity before spi_load_windows");
  if (N <= 0 || K < 1 || K > SPI_THETA_DIM) return set_error(SPI_EINVAL, "spi_sensitivity: N=%d K=%d", N, K);
  for (int k = 0; k < K; ++k)
    if (param_ids[k] < 0 || param_ids[k] >= SPI_THETA_DIM)
      return set_error(SPI_EINVAL, "spi_sensitivity: param_ids[%d]=%d", k, param_ids[k]);
  int rc = e->sens_ids.reserve(SPI_THETA_DIM * sizeof(int));
  if (rc) return rc;
  memcpy(e->h_sens_ids, param_ids, K * sizeof(int));
  cudaError_t ce = cudaMemcpyAsync(e->sens_ids.p, e->h_sens_ids, K * sizeof(int), cudaMemcpyHostToDevice, e->stream);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_sensitivity: ids");
  WinView win{e->init.f(), e->act.f(), e->tgt.f(), e->weight.f(), e->W, e->H};
  SensArgs a{(const int*)e->sens_ids.p, K, N, J, xH};
  const long long quads = (long long)N * e->W * K;
  sensitivity_kernel<<<(unsigned)((quads + 31) / 32), 128, 0, e->stream>>>(e->d_model, win, theta, a);
  ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_sensitivity: launch");
}

int spi_fisher(const float* J, int N, int W, int K, const float* state_weight, double eps, float* F, double* logdet,
               double* trace, void* stream) {
  return spi_fisher_ex(J, N, W, K, state_weight, eps, 0, F, logdet, trace, stream);
}

int spi_fisher_ex(const float* J, int N, int W, int K, const float* state_weight, double eps, int tensor_cores,
                  float* F, double* logdet, double* trace, void* stream) {
  if (!J || !F || N <= 0 || W <= 0 || K < 1 || K > SPI_THETA_DIM)
    return set_error(SPI_EINVAL, "spi_fisher: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (tensor_cores)
    fisher_mma_kernel<<<(N + 3) / 4, 128, 0, s>>>(J, N, W, K, state_weight, F);
  else
    fisher_kernel<<<N, 128, 0, s>>>(J, N, W, K, state_weight, F);
  if (logdet || trace) logdet_kernel<<<(N + 127) / 128, 128, 0, s>>>(F, N, K, eps, logdet, trace);
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? SPI_OK : cuda_error(ce, "spi_fisher");
}

}  // extern "C"
