// Deterministic reductions: per-thread FP32 partial sums over short runs,
// FP64 across threads and blocks, block partials summed in a fixed order.
#include "common.cuh"

namespace mlpcg {

constexpr int kDotThreads = 256;
constexpr int kDotBlocksMax = 1216;  // 8 x 152 SMs

__device__ __forceinline__ double ldd(const float *p) { return (double)__ldg(p); }
__device__ __forceinline__ double ldd(const double *p) { return __ldg(p); }
__device__ __forceinline__ double ldd(const __nv_bfloat16 *p) { return (double)__bfloat162float(*p); }

// Block-wide FP64 sum; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads)
k_dot_partial(const T *__restrict__ x, const T *__restrict__ y, int64_t n, double *__restrict__ partial) {
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    acc = fma(ldd(x + q), ldd(y + q), acc);
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void k_sum_partials(const double *__restrict__ partial, int nblk, double *__restrict__ out) {
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += partial[b];
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[0] = acc;
}

static int dot_blocks(int64_t n) {
  int64_t b = (n + kDotThreads * 4 - 1) / (kDotThreads * 4);
  if (b > kDotBlocksMax) b = kDotBlocksMax;
  if (b < 1) b = 1;
  return (int)b;
}

size_t dot_workspace(int64_t n) { return (size_t)dot_blocks(n) * sizeof(double); }

int launch_dot(const void *x, const void *y, int dt, int64_t n, double *out, void *ws, size_t ws_bytes,
               cudaStream_t st) {
  const int nb = dot_blocks(n);
  MLPCG_REQUIRE(ws_bytes >= (size_t)nb * sizeof(double), MLPCG_ERR_WORKSPACE, "dot workspace too small");
  double *part = (double *)ws;
  if (dt == MLPCG_F32)
    k_dot_partial<float><<<nb, kDotThreads, 0, st>>>((const float *)x, (const float *)y, n, part);
  else if (dt == MLPCG_F64)
    k_dot_partial<double><<<nb, kDotThreads, 0, st>>>((const double *)x, (const double *)y, n, part);
  else
    k_dot_partial<__nv_bfloat16><<<nb, kDotThreads, 0, st>>>((const __nv_bfloat16 *)x, (const __nv_bfloat16 *)y,
                                                            n, part);
  MLPCG_LAUNCH_CHECK();
  k_sum_partials<<<1, 256, 0, st>>>(part, nb, out);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

}  // namespace mlpcg
