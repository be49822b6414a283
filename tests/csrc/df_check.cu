// Test helper: the integer-only double-float conversions of the solver (df_to_double_bits,
// df_from_double_bits) against the FP64 routines they replace (df_to_double, df_from_double),
// bit for bit, on hashed inputs.  Built and loaded by tests/test_gpu_doublefloat.py.
#include "common.cuh"

using namespace mlpcg;

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Sample i: a normalised pair (hi, lo) -- hi with a random sign and significand and an exponent
// in [-60, 60], |lo| <= ulp(hi) / 2 scaled by 2^-k (k in [0, 15]), every 8th sample an exact tie
// lo = +-ulp(hi) / 2 -- and a double with an exponent in [-70, 70].
__global__ void k_df_check(uint64_t n, uint64_t seed, unsigned long long *bad) {
  unsigned long long bad_to = 0, bad_from = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r0 = mix64(seed ^ (3 * i)), r1 = mix64(seed ^ (3 * i + 1)), r2 = mix64(seed ^ (3 * i + 2));
    const int eh = 127 - 60 + (int)((r0 >> 32) % 121);
    const float hi = __uint_as_float((uint32_t)(r0 & 0x807fffffu) | ((uint32_t)eh << 23));
    const float half_ulp = __uint_as_float((uint32_t)(eh - 24) << 23);
    float lo;
    if ((i & 7) == 7) {
      lo = (r1 & 1) ? half_ulp : -half_ulp;
    } else {
      const int k = (int)((r1 >> 40) % 16);
      const float u = (float)((int32_t)(r1 & 0xffffffu) - (1 << 23)) * (1.f / (float)(1 << 23));  // [-1, 1)
      lo = u * half_ulp * __uint_as_float((uint32_t)(127 - k) << 23);
    }
    const float2 p = make_float2(hi, lo);
    if (__double_as_longlong(df_to_double_bits(p)) != __double_as_longlong(df_to_double(p))) ++bad_to;

    const uint64_t E = (uint64_t)(1023 - 70 + (int)((r2 >> 52) % 141));
    const double v = __longlong_as_double((long long)((r2 & 0x800fffffffffffffull) | (E << 52)));
    const float2 a = df_from_double_bits(v), b = df_from_double(v);
    if (__float_as_uint(a.x) != __float_as_uint(b.x) || __float_as_uint(a.y) != __float_as_uint(b.y)) ++bad_from;
  }
  if (bad_to) atomicAdd(bad, bad_to);
  if (bad_from) atomicAdd(bad + 1, bad_from);
}

}  // namespace

// Mismatch counts of n samples into bad_host[0] (to double) and bad_host[1] (from double);
// returns a cudaError_t value.
extern "C" int df_check(unsigned long long n, unsigned long long seed, unsigned long long *bad_host) {
  unsigned long long *bad = nullptr;
  cudaError_t e = cudaMalloc(&bad, 2 * sizeof(unsigned long long));
  if (e != cudaSuccess) return (int)e;
  e = cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_df_check<<<1216, 256>>>(n, seed, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(bad_host, bad, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  return (int)e;
}
