// Deterministic reductions: per-thread FP32 partial sums over short runs,
// FP64 across threads and blocks, block partials summed in a fixed order.
#include <mutex>
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
  dependent_launch_enter();
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    acc = fma(ldd(x + q), ldd(y + q), acc);
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void k_sum_partials(const double *__restrict__ partial, int nblk, double *__restrict__ out) {
  dependent_launch_enter();
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

// ---------------------------------------------------------------------------
// mlpcg_dot_noalloc: the same reduction with its block partials in a
// file-scope device array instead of a caller workspace, for callers that
// cannot allocate device memory: real-time loops that must never enter the
// allocator (its latency is unbounded), and host runtimes or plug-in hosts
// that own all device memory through their own arena and give a library
// only the buffers of its inputs and outputs.  One partial per 2048 elements, at most 8192
// partials (64 KiB), so n <= 16,777,216 (a 256^3 grid).  Every GPU that
// loads this library holds the 64 KiB until the process exits.
// ---------------------------------------------------------------------------
constexpr int kNoAllocPartials = 8192;
constexpr int kNoAllocPerBlock = 2048;
constexpr int64_t kNoAllocMaxN = (int64_t)kNoAllocPartials * kNoAllocPerBlock;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

// Device address of g_noalloc_partials, looked up once per device.  In host
// code the array's name is only a host-side stand-in, so the address must
// come from cudaGetSymbolAddress with that device current.
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[kNoAllocMaxDevices];

static int noalloc_scratch(double **out) {
  int dev = 0;
  MLPCG_CUDA_CHECK(cudaGetDevice(&dev));
  MLPCG_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, MLPCG_ERR_UNSUPPORTED,
                "dot_noalloc: device ordinal %d beyond %d", dev, kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    MLPCG_CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return MLPCG_OK;
}

int launch_dot_noalloc(const void *x, const void *y, int dt, int64_t n, double *out, cudaStream_t st) {
  MLPCG_REQUIRE(n <= kNoAllocMaxN, MLPCG_ERR_SHAPE,
                "dot_noalloc: n = %lld exceeds the maximum of %lld elements (%d partial sums in the "
                "library's static scratch); use mlpcg_dot with a workspace",
                (long long)n, (long long)kNoAllocMaxN, kNoAllocPartials);
  double *part = nullptr;
  const int rc = noalloc_scratch(&part);
  if (rc != MLPCG_OK) return rc;
  // every one of the nb partials is written before it is read: nothing to clear
  const int nb = (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
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

extern "C" int mlpcg_dot_noalloc(const void *x, const void *y, int dtype, int64_t n, double *out, void *stream) {
  mlpcg::clear_error();
  MLPCG_REQUIRE(x && y && out, MLPCG_ERR_ARG, "dot_noalloc: NULL argument");
  MLPCG_REQUIRE(mlpcg::valid_dtype(dtype), MLPCG_ERR_UNSUPPORTED, "dot_noalloc: bad dtype %d", dtype);
  MLPCG_REQUIRE(n >= 1, MLPCG_ERR_ARG, "dot_noalloc: n must be >= 1");
  return mlpcg::launch_dot_noalloc(x, y, dtype, n, out, mlpcg::as_stream(stream));
}
