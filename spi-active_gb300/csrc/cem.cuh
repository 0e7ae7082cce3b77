// cem.cuh -- cross-entropy-method refit and sampling on the device.
//
// Per job: the population theta [N][13] (float), its costs [N]; the distribution
// (mean, covariance, Cholesky factor) in FP64. One refit = sort (cost, index) keys
// (NaN last; ties by index), mean and covariance of the n_elite best, smoothing
// alpha, per-dimension std floor, FP64 Cholesky. Sampling: Philox4x32-10 words
// (counter = sample, iteration, block, job; key = seed) -> Box-Muller normals ->
// theta = clip(mu + L z, lo, hi); iteration 0 samples the prior box uniformly.
// All iteration state lives on the device, so an iteration can be graph-captured.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cem_state.h"
#include "spi_engine.h"

namespace spi {

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}

__device__ __forceinline__ double u01(uint32_t w) { return ((double)w + 0.5) * 2.3283064365386963e-10; }
// -ln(u) for u = (w + 0.5) 2^-32 in FP32. Near u = 1 the logarithm is taken of the exact
// complement, 1 - u = (2^32 - 1 - w + 0.5) 2^-32, so draws close to 1 keep their small radius.
__device__ __forceinline__ float neg_log_u01f(uint32_t w) {
  if (w < 0x80000000u) return -logf(((float)w + 0.5f) * 2.3283064e-10f);
  return -log1pf(-((float)(0xFFFFFFFFu - w) + 0.5f) * 2.3283064e-10f);
}

// Orderable key: cost ascending (NaN last), then index ascending.
__device__ __forceinline__ unsigned long long cost_key(float c, unsigned idx) {
  uint32_t b = __float_as_uint(c);
  uint32_t o;
  if (isnan(c)) o = 0xFFFFFFFFu;
  else o = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
  return ((unsigned long long)o << 32) | idx;
}

// Draw the population of the current iteration into st->theta; one grid row per state.
// rounds (optional, one per state): a state takes part only while round < rounds[state].
static __global__ void cem_sample_kernel(const CemState* __restrict__ st_all, const int* __restrict__ rounds = nullptr,
                                         int round = 0) {
  const CemState* st = st_all + blockIdx.y;
  // exits uniform per CTA, before the barrier
  if (!st->active || (int)(blockIdx.x * blockDim.x) >= st->n_samples) return;
  if (rounds && round >= rounds[blockIdx.y]) return;
  const int P = st->dim, it = st->iter;
  // the distribution, staged once per CTA (as FP32 for the Gaussian draws), so that the
  // per-dimension loops below read shared memory instead of waiting on global loads
  __shared__ float s_L[CEM_MAX_DIM * CEM_MAX_DIM];
  __shared__ float s_mu[CEM_MAX_DIM], s_lo[CEM_MAX_DIM], s_hi[CEM_MAX_DIM];
  __shared__ float s_nom[SPI_THETA_DIM];
  __shared__ int s_ids[CEM_MAX_DIM];
  for (int i = threadIdx.x; i < P * CEM_MAX_DIM; i += blockDim.x) s_L[i] = (float)st->L[i];
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    s_mu[i] = (float)st->mu[i];
    s_lo[i] = (float)st->lo[i];
    s_hi[i] = (float)st->hi[i];
    s_ids[i] = st->param_ids[i];
  }
  for (int i = threadIdx.x; i < SPI_THETA_DIM; i += blockDim.x) s_nom[i] = st->nominal[i];
  __syncthreads();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= st->n_samples) return;
  float* theta = st->theta + (size_t)n * SPI_THETA_DIM;
  const uint32_t k0 = (uint32_t)(st->seed & 0xFFFFFFFFull), k1 = (uint32_t)(st->seed >> 32);
  // Iteration 0 draws the uniform prior box in FP64 (no transcendental work). Later iterations
  // draw Gaussians in FP32: Box-Muller and the Cholesky product are a few hundred operations
  // per sample, which GB300's FP64 units would take tens of microseconds to finish, while the
  // sample is stored as FP32 anyway (rounding to float commutes with the clamp to [lo, hi]).
  float out[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) out[i] = s_nom[i];
  if (it == 0) {
    double z[CEM_MAX_DIM + 3];
#pragma unroll
    for (int b = 0; b < (CEM_MAX_DIM + 3) / 4; ++b) {
      if (4 * b >= P) break;
      uint32_t c[4] = {(uint32_t)n, (uint32_t)it, (uint32_t)b, (uint32_t)st->job};
      philox4x32_10(c, k0, k1);
#pragma unroll
      for (int q = 0; q < 4; ++q) z[4 * b + q] = u01(c[q]);
    }
    for (int d = 0; d < P; ++d) {
      const double v = st->lo[d] + (st->hi[d] - st->lo[d]) * z[d];
      const int slot = s_ids[d];
#pragma unroll
      for (int i = 0; i < SPI_THETA_DIM; ++i)
        if (i == slot) out[i] = (float)v;
    }
  } else {
    float z[CEM_MAX_DIM + 3];
#pragma unroll
    for (int b = 0; b < (CEM_MAX_DIM + 3) / 4; ++b) {
      if (4 * b >= P) break;
      uint32_t c[4] = {(uint32_t)n, (uint32_t)it, (uint32_t)b, (uint32_t)st->job};
      philox4x32_10(c, k0, k1);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float r = sqrtf(2.0f * neg_log_u01f(c[2 * q]));
        float sn, co;
        sincospif(2.0f * (((float)c[2 * q + 1] + 0.5f) * 2.3283064e-10f), &sn, &co);
        z[4 * b + 2 * q] = r * co;
        z[4 * b + 2 * q + 1] = r * sn;
      }
    }
    for (int d = 0; d < P; ++d) {
      float v = s_mu[d];
      for (int e = 0; e <= d; ++e) v = fmaf(s_L[d * CEM_MAX_DIM + e], z[e], v);
      v = fminf(fmaxf(v, s_lo[d]), s_hi[d]);
      const int slot = s_ids[d];
#pragma unroll
      for (int i = 0; i < SPI_THETA_DIM; ++i)
        if (i == slot) out[i] = v;
    }
  }
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) theta[i] = out[i];
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Dynamic shared memory of cem_refit_kernel for a population of n: the selection keys
// (8 bytes each) and the elite index list (4 bytes each).
inline size_t cem_refit_smem(int n) { return (size_t)n * (sizeof(unsigned long long) + sizeof(int)); }
constexpr int kCemRefitMaxSmem = CEM_MAX_SAMPLES * (int)(sizeof(unsigned long long) + sizeof(int));

// One CTA (1024 threads) per state: elite select + mean / covariance + Cholesky. rounds as
// in cem_sample_kernel. Dynamic shared memory: cem_refit_smem(n_samples) bytes.
//
// The elites are the n_elite smallest keys (cost ascending, NaN last, then index; keys are
// unique). They are selected by radix select, 8 bits a pass from the top of the key: a pass
// histograms the keys that share the bits decided so far, and the bin holding the target rank
// fixes the next 8 bits. It stops when every key of that bin is an elite (at the latest when the
// bin holds one key), typically after two to four passes over the cost bits, so the CTA meets
// three barriers a pass instead of the ~36 of a full sort. The elites are then listed in index
// order (a block-wide prefix sum), which fixes the order of the FP64 sums below.
static __global__ void __launch_bounds__(1024) cem_refit_kernel(CemState* __restrict__ st_all,
                                                               const int* __restrict__ rounds = nullptr,
                                                               int round = 0) {
  if (rounds && round >= rounds[blockIdx.x]) return;   // uniform per CTA, before any barrier
  extern __shared__ unsigned long long keys[];
  __shared__ double s_mu[CEM_MAX_DIM];
  __shared__ double s_cov[CEM_MAX_DIM * CEM_MAX_DIM];
  __shared__ unsigned s_hist[256];
  __shared__ unsigned long long s_prefix, s_mask, s_best;
  __shared__ int s_rank, s_done;
  __shared__ int s_scan[32];
  CemState* st = st_all + blockIdx.x;
  if (!st->active) return;   // uniform per CTA
  const float* theta = st->theta;
  const float* cost = st->cost;
  const int N = st->n_samples, P = st->dim, ne = st->n_elite;
  int* eidx = reinterpret_cast<int*>(keys + N);   // the elite index list, after the keys
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  // keys in index order, one contiguous run per thread
  const int run = (N + blockDim.x - 1) / blockDim.x;
  const int i0 = min(N, (int)threadIdx.x * run), i1 = min(N, i0 + run);
  unsigned long long kmin = ~0ull;
  for (int i = i0; i < i1; ++i) {
    const unsigned long long k = cost_key(cost[i], (unsigned)i);
    keys[i] = k;
    kmin = k < kmin ? k : kmin;
  }
  // the best key (block minimum), for the best-so-far record
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, kmin, o);
    kmin = v < kmin ? v : kmin;
  }
  if (threadIdx.x == 0) { s_prefix = 0; s_mask = 0; s_rank = ne - 1; s_done = 0; s_best = ~0ull; }
  __syncthreads();
  if (lane == 0) atomicMin(&s_best, kmin);
  // radix select of the key of rank ne - 1
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) s_hist[b] = 0;
    __syncthreads();
    const unsigned long long prefix = s_prefix, mask = s_mask;
    for (int i = i0; i < i1; ++i) {
      const unsigned long long k = keys[i];
      if ((k & mask) == prefix) atomicAdd(&s_hist[(unsigned)(k >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    if (warp == 0) {
      const unsigned rank = (unsigned)s_rank;
      unsigned c[8], sum = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) { c[q] = s_hist[8 * lane + q]; sum += c[q]; }
      unsigned incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const unsigned excl = incl - sum;
      __syncwarp();
      if (rank >= excl && rank < incl) {            // exactly one lane: its bins hold the rank
        unsigned before = excl;
        int q = 0;
        while (rank >= before + c[q]) before += c[q++];
        const unsigned r = rank - before;
        s_prefix = prefix | ((unsigned long long)(8 * lane + q) << shift);
        s_mask = mask | (0xFFull << shift);
        s_rank = (int)r;
        if (c[q] == r + 1) s_done = 1;              // every key of the bin is an elite
      }
    }
    __syncthreads();
    if (s_done) break;                              // uniform: read after the barrier
  }
  // elites: keys whose decided bits are below the final prefix, or equal to it
  const unsigned long long fprefix = s_prefix, fmask = s_mask;
  int cnt = 0;
  for (int i = i0; i < i1; ++i) cnt += (keys[i] & fmask) <= fprefix ? 1 : 0;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_scan[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = lane < nwarps ? s_scan[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    s_scan[lane] = v;                                // inclusive warp totals
  }
  __syncthreads();
  int pos = incl - cnt + (warp > 0 ? s_scan[warp - 1] : 0);
  for (int i = i0; i < i1; ++i)
    if ((keys[i] & fmask) <= fprefix) eidx[pos++] = i;
  __syncthreads();
  // elite mean, one warp per dimension
  for (int d = warp; d < P; d += nwarps) {
    const int slot = st->param_ids[d];
    double s = 0.0;
    for (int e = lane; e < ne; e += 32) s += (double)theta[(size_t)eidx[e] * SPI_THETA_DIM + slot];
    s = warp_sum_d(s);
    if (lane == 0) s_mu[d] = s / ne;
  }
  __syncthreads();
  // elite covariance, one warp per upper-triangle entry (three entries a warp at most: P <= 13
  // gives at most 91 entries for 32 warps). The elite rows are centred once, kEliteChunk at a
  // time, in shared memory (FP64 work is scarce); each lane still sums its elites e = lane,
  // lane + 32, ... in order, so the result equals a pass over the unstaged rows.
  constexpr int kEliteChunk = 256;   // a multiple of 32
  __shared__ double s_c[kEliteChunk * CEM_MAX_DIM];
  const int nent = P * (P + 1) / 2;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int e0 = 0; e0 < ne; e0 += kEliteChunk) {
    const int m = min(kEliteChunk, ne - e0);
    __syncthreads();                  // the previous chunk has been read
    for (int t = threadIdx.x; t < m * P; t += blockDim.x) {
      const int e = t / P, d = t % P;
      s_c[e * CEM_MAX_DIM + d] =
          (double)theta[(size_t)eidx[e0 + e] * SPI_THETA_DIM + st->param_ids[d]] - s_mu[d];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = warp + k * nwarps;
      if (q < nent) {
        int i = 0, r = q;
        while (r >= P - i) { r -= P - i; ++i; }
        const int j = i + r;
        double s = acc[k];
        for (int e = lane; e < m; e += 32) s += s_c[e * CEM_MAX_DIM + i] * s_c[e * CEM_MAX_DIM + j];
        acc[k] = s;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int q = warp + k * nwarps;
    if (q < nent) {
      int i = 0, r = q;
      while (r >= P - i) { r -= P - i; ++i; }
      const int j = i + r;
      const double s = warp_sum_d(acc[k]);
      if (lane == 0) { s_cov[i * CEM_MAX_DIM + j] = s / ne; s_cov[j * CEM_MAX_DIM + i] = s / ne; }
    }
  }
  __syncthreads();
  // smoothed mean and covariance (+ the std floor on the diagonal), element-parallel, kept in
  // shared memory for the factorisation and written out once
  __shared__ double s_L[CEM_MAX_DIM * CEM_MAX_DIM];
  __shared__ int s_ok;
  const double a = st->alpha;
  if (threadIdx.x == 0) s_ok = 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) st->mu[i] = a * s_mu[i] + (1.0 - a) * st->mu[i];
  for (int q = threadIdx.x; q < P * P; q += blockDim.x) {
    const int i = q / P, j = q % P;
    double v = a * s_cov[i * CEM_MAX_DIM + j] + (1.0 - a) * st->cov[i * CEM_MAX_DIM + j];
    if (i == j) v += st->min_std[i] * st->min_std[i];
    s_cov[i * CEM_MAX_DIM + j] = v;
    st->cov[i * CEM_MAX_DIM + j] = v;
  }
  __syncthreads();
  // Cholesky, lower, by one warp: column j's diagonal on lane 0, then its rows i > j on lanes
  // (each entry's sum in the serial order k = 0 .. j - 1)
  if (warp == 0) {
    for (int j = 0; j < P; ++j) {
      if (lane == 0) {
        double d = s_cov[j * CEM_MAX_DIM + j];
        for (int k = 0; k < j; ++k) d -= s_L[j * CEM_MAX_DIM + k] * s_L[j * CEM_MAX_DIM + k];
        if (!(d > 0.0)) { s_ok = 0; d = st->min_std[j] * st->min_std[j]; }
        s_L[j * CEM_MAX_DIM + j] = sqrt(d);
      }
      __syncwarp();
      const double ljj = s_L[j * CEM_MAX_DIM + j];
      for (int i = j + 1 + lane; i < P; i += 32) {
        double v = s_cov[i * CEM_MAX_DIM + j];
        for (int k = 0; k < j; ++k) v -= s_L[i * CEM_MAX_DIM + k] * s_L[j * CEM_MAX_DIM + k];
        s_L[i * CEM_MAX_DIM + j] = v / ljj;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < P * P; q += blockDim.x) {
    const int i = q / P, j = q % P;
    st->L[i * CEM_MAX_DIM + j] = j <= i ? s_L[i * CEM_MAX_DIM + j] : 0.0;
  }
  if (threadIdx.x == 0) {
    if (!s_ok) st->status = 1;
    const unsigned b = (unsigned)(s_best & 0xFFFFFFFFull);
    const float bc = cost[b];
    if (bc < st->best_cost || (isnan(st->best_cost) && !isnan(bc))) {
      st->best_cost = bc;
      for (int i = 0; i < SPI_THETA_DIM; ++i) st->best_theta[i] = theta[(size_t)b * SPI_THETA_DIM + i];
    }
    st->iter += 1;
  }
}

}  // namespace spi
