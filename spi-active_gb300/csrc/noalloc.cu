// noalloc.cu -- spi_eval_windows_noalloc: windowed rollout + cost that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc. Examples: a serving process that
// reserves its whole HBM budget up front, a host framework that owns every device
// allocation, and a control loop where cudaMalloc's implicit device synchronisation would
// stall other streams. This entry point evaluates theta samples against windows with the same
// dynamics as spi_run, but:
//   * it reads the caller's windows in the reference's row layout ([W][37], [W][H][12])
//     instead of copying them into engine storage;
//   * the robot model travels by value as a kernel parameter;
//   * the per-(theta, window group) cost partials live in g_partials below, a file-scope
//     device array of fixed size that every GPU loading this library keeps until exit.
// The caller passes all inputs and outputs as device pointers.
//
// Limits and sharing: N * ceil(W / 8) <= SPI_NOALLOC_MAX_GROUPS (larger requests are
// rejected with SPI_EINVAL). Every call uses the same g_partials array, so calls whose
// kernels overlap on the GPU (different streams, or different host threads) race on it;
// serialise them. Each call writes every partial it later reads, so stale contents of an
// earlier call are never summed. The first call on a device resolves the array's device
// address with cudaGetSymbolAddress (with that device current); make that first call
// before any stream capture.
//
// Non-finite rollouts: spi_run counts rollouts whose final state is not finite (read with
// spi_sync); this entry point keeps no such count, since a counter would be one more piece of
// device memory. A non-finite final state reaches the outputs instead: every error component
// of that window is summed (with weight 0 too, as 0 * NaN is NaN), so the theta's row of comp
// turns non-finite. Callers check comp (or the cost) themselves.
#include <cuda_runtime.h>

#include <mutex>

#include "common.h"
#include "model.h"
#include "rollout.cuh"

using namespace spi;

namespace {

constexpr int kMaxGroups = SPI_NOALLOC_MAX_GROUPS;
constexpr int kMaxDevices = 64;

// cost partials [theta][window group][SPI_N_COMP]
static __device__ __align__(256) float g_partials[(size_t)kMaxGroups * SPI_N_COMP];

std::mutex g_mu;
float* g_partials_addr[kMaxDevices] = {nullptr};

// One warp per (theta n, window group g): 8 windows, 4 lanes (legs) per window.
__global__ void __launch_bounds__(128) rollout_rows_kernel(const DevModel model, const float* __restrict__ init,
                                                           const float* __restrict__ actions,
                                                           const float* __restrict__ target,
                                                           const float* __restrict__ weight, int W, int H,
                                                           const float* __restrict__ theta, int N, int G,
                                                           float* __restrict__ partials) {
  __shared__ DevModel M;
  {
    const unsigned* s = reinterpret_cast<const unsigned*>(&model);
    unsigned* d = reinterpret_cast<unsigned*>(&M);
    for (int i = threadIdx.x; i < (int)(sizeof(DevModel) / 4); i += blockDim.x) d[i] = s[i];
  }
  __syncthreads();
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (warp >= (long long)N * G) return;
  const int n = (int)(warp / G), g = (int)(warp % G);
  const int lane = threadIdx.x & 31, leg = lane & 3;
  int w = g * 8 + (lane >> 2);
  const bool active = w < W;
  if (!active) w = W - 1;

  float th[SPI_THETA_DIM];
#pragma unroll
  for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = __ldg(theta + (size_t)n * SPI_THETA_DIM + i);
  const BaseParams<float> bp = base_params<float>(M, th);
  const LegParams<float> lp = leg_params<float>(th, leg);
  const float* x0 = init + (size_t)w * SPI_STATE_DIM;
  BaseState<float> B;
  LegState<float> L;
  {
    float s13[13];
#pragma unroll
    for (int i = 0; i < 13; ++i) s13[i] = __ldg(x0 + i);
    base_from_world(B, s13);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      L.q[k] = __ldg(x0 + 13 + 3 * leg + k);
      L.qd[k] = __ldg(x0 + 25 + 3 * leg + k);
    }
  }
  for (int h = 0; h < H; ++h) {
    const float* ap = actions + ((size_t)w * H + h) * 12 + 3 * leg;
    float act[3] = {__ldg(ap), __ldg(ap + 1), __ldg(ap + 2)};
    for (int s = 0; s < M.decimation; ++s) substep(M, leg, B, L, bp, lp, act);
  }
  const float* tg = target + (size_t)w * SPI_STATE_DIM;
  float s13[13];
  base_to_world(B, s13);
  float sp = 0.f, sq = 0.f, sv = 0.f, sw = 0.f, sj = 0.f, sjd = 0.f;
  if (leg == 0) {
#pragma unroll
    for (int i = 0; i < 13; ++i) {
      const float d = s13[i] - __ldg(tg + i);
      if (i < 3) sp += d * d; else if (i < 7) sq += d * d; else if (i < 10) sv += d * d; else sw += d * d;
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dq = L.q[k] - __ldg(tg + 13 + 3 * leg + k);
    const float dqd = L.qd[k] - __ldg(tg + 25 + 3 * leg + k);
    sj += dq * dq;
    sjd += dqd * dqd;
  }
  sp = qsum(sp); sq = qsum(sq); sv = qsum(sv); sw = qsum(sw); sj = qsum(sj); sjd = qsum(sjd);
  const float wt = active ? (weight ? __ldg(weight + w) : 1.0f) : 0.f;
  const float comp[SPI_N_COMP] = {sqrtf(sp), sqrtf(sq), sqrtf(sj), sp, sq, sv, sw, sj, sjd};
  float* out = partials + ((size_t)n * G + g) * SPI_N_COMP;
#pragma unroll
  for (int k = 0; k < SPI_N_COMP; ++k) {
    const float v = slot_sum(active ? comp[k] * wt : 0.f);
    if (lane == 0) out[k] = v;
  }
}

// The engine's finalize (rollout.cuh finalize_one): partials summed in group order, the
// weighted cost formed with the same pinned roundings, so both paths give the same costs
// from the same partials.
__global__ void finalize_rows_kernel(const float* __restrict__ partials, int N, int G, float norm, int mode,
                                     float w0, float w1, float w2, float w3, float w4, float w5,
                                     float* __restrict__ comp, float* __restrict__ cost) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const float w[6] = {w0, w1, w2, w3, w4, w5};
  finalize_one(partials, n, G, norm, mode, w, comp, cost);
}

// Device address of g_partials on the current device, resolved once per device.
int partials_on_current_device(float** out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return cuda_error(ce, "spi_eval_windows_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return set_error(SPI_EINVAL, "spi_eval_windows_noalloc: device %d", dev);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_partials);
    if (ce != cudaSuccess) return cuda_error(ce, "spi_eval_windows_noalloc: cudaGetSymbolAddress");
    g_partials_addr[dev] = static_cast<float*>(p);
  }
  *out = g_partials_addr[dev];
  return SPI_OK;
}

}  // namespace

extern "C" int spi_eval_windows_noalloc(const spi_robot* robot, const float* init, const float* actions,
                                        const float* target, const float* weight, int W, int H, float norm,
                                        const float* theta, int N, int cost_mode, const float* sq_weights,
                                        float* comp, float* cost, void* stream) {
  if (!robot || !init || !actions || !target || !theta)
    return set_error(SPI_EINVAL, "spi_eval_windows_noalloc: null argument");
  if (W <= 0 || H <= 0 || N <= 0)
    return set_error(SPI_EINVAL, "spi_eval_windows_noalloc: W=%d H=%d N=%d must be > 0", W, H, N);
  if (cost_mode != 0 && cost_mode != 1)
    return set_error(SPI_EINVAL, "spi_eval_windows_noalloc: cost_mode %d not 0/1", cost_mode);
  const int G = (W + 7) / 8;
  if ((long long)N * G > kMaxGroups)
    return set_error(SPI_EINVAL,
                     "spi_eval_windows_noalloc: N * ceil(W/8) = %lld exceeds the fixed scratch of %d "
                     "(theta, 8-window group) slots; split the theta batch",
                     (long long)N * G, kMaxGroups);
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return set_error(rc, "spi_eval_windows_noalloc: %s", why);
  float* partials = nullptr;
  if ((rc = partials_on_current_device(&partials))) return rc;
  const float dw[6] = {10.f, 5.f, 0.1f, 0.1f, 1.f, 0.01f};
  const float* w = sq_weights ? sq_weights : dw;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long warps = (long long)N * G;
  rollout_rows_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(M, init, actions, target, weight, W, H,
                                                                   theta, N, G, partials);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_eval_windows_noalloc: rollout launch");
  finalize_rows_kernel<<<(unsigned)((N + 127) / 128), 128, 0, s>>>(
      partials, N, G, norm > 0.f ? norm : (float)W, cost_mode, w[0], w[1], w[2], w[3], w[4], w[5], comp, cost);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_error(ce, "spi_eval_windows_noalloc: finalize launch");
  return SPI_OK;
}
