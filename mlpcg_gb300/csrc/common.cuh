// Shared helpers of the sm_103a kernels: element loads/stores, tap offsets,
// error reporting, launch checks.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

#include "../../include/mlpcg_gb300.h"

namespace mlpcg {

// ---------------------------------------------------------------------------
// error reporting (thread-local last-error string, see mlpcg_last_error)
// ---------------------------------------------------------------------------
void set_error(const char *fmt, ...);
void clear_error();

#define MLPCG_REQUIRE(cond, code, ...)        \
  do {                                        \
    if (!(cond)) {                            \
      ::mlpcg::set_error(__VA_ARGS__);        \
      return (code);                          \
    }                                         \
  } while (0)

#define MLPCG_CUDA_CHECK(expr)                                                  \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) {                                                    \
      ::mlpcg::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                         __FILE__, __LINE__);                                   \
      return MLPCG_ERR_CUDA;                                                    \
    }                                                                           \
  } while (0)

// Checks the launch that was just issued (configuration errors only; the
// kernel itself runs asynchronously).
#define MLPCG_LAUNCH_CHECK() MLPCG_CUDA_CHECK(cudaGetLastError())

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool valid_dtype(int dt) { return dt == MLPCG_F32 || dt == MLPCG_BF16 || dt == MLPCG_F64; }
inline size_t dtype_size(int dt) { return dt == MLPCG_F64 ? 8 : (dt == MLPCG_BF16 ? 2 : 4); }

__host__ __device__ inline int64_t cells(int n1, int n2, int n3) { return (int64_t)n1 * n2 * n3; }
inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Optional epilogue of the finest post-block for the solvers: the products of
// the new preconditioned residual z with the A-images of the two most recent
// search directions, z . ring[head] and z . ring[(head + 2) % 3] (npsd; ring:
// three slots of n floats; none at iteration 0, the first alone at iteration
// 1), or with one fixed vector, z . ring (single != 0: npcg's r . z, every
// iteration), summed per tile of the finest level in FP64 into
// partial[2 * tile + k].  head and it are words of the solver's device state,
// read by the kernel.
struct ZDots {
  const float *ring;
  const int *head, *it;
  double *partial;
  int64_t n;
  int single;
};

// First statement of every kernel of this library.  A kernel reached through a
// programmatic graph edge (the solver's captured iteration) may be scheduled
// while its predecessor still runs: it waits here until the predecessor grid
// has completed and its writes are visible, touching no memory before.
// Launched any other way, the wait does nothing.  By default a kernel's
// successor is released as its blocks exit (the implicit trigger), so the
// successor's blocks are scheduled onto the SMs that free up.
__device__ __forceinline__ void dependent_launch_enter() { cudaGridDependencySynchronize(); }

// Second statement of the kernels with small grids (the small-level block
// kernels, a few blocks per SM at most, and the CG kernels, sized to the
// resident CTAs): their successor's blocks may be scheduled as soon as all of
// this grid's blocks have started, and wait at their entry.  The many-wave
// level-0 and level-1 block kernels do not trigger: their successor's blocks
// would be placed early, unevenly, on the first SMs to free up (triggering in
// every kernel was measured 6 % slower at 256^3).
__device__ __forceinline__ void dependent_launch_trigger() { cudaTriggerProgrammaticLaunchCompletion(); }

// ---------------------------------------------------------------------------
// Double-float arithmetic: a value as the unevaluated sum hi + lo of two
// floats, kept exact by error-free transformations (Knuth's two-sum, Dekker's
// fast two-sum, FMA two-product); the rounded-to-nearest intrinsics keep the
// compiler from contracting or reordering them.  GB300 runs FP64 arithmetic
// at a small fraction of its FP32 rate; these stay on the FP32 pipes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float2 s = two_sum(a.x, b.x);
  return fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_mul_f(float2 a, float b) {
  const float p = __fmul_rn(a.x, b);
  const float e = fmaf(a.y, b, fmaf(a.x, b, -p));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ float2 df_from_double(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}
__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// The same two conversions for bulk use with integer operations only (the
// FP64 pipe is the bottleneck of a pass that converts every cell).  Results
// equal df_from_double / df_to_double bit for bit; values outside the range
// handled here (exponents far from 1, zeros, subnormals, Inf, NaN, or a low
// part tiny against the high part) take the FP64 routine above.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }  // k in [-126, 127]

// the FP64 routines as real calls, so that the rare values that need them do not make the
// compiler evaluate them for every cell
static __device__ __noinline__ float2 df_from_double_call(double v) { return df_from_double(v); }
static __device__ __noinline__ double df_to_double_call(float2 a) { return df_to_double(a); }

__device__ __forceinline__ float2 df_from_double_bits(double v) {
  const uint64_t u = (uint64_t)__double_as_longlong(v);
  const int E = (int)((u >> 52) & 0x7ff) - 1023;
  if (E < -74 || E > 120) return df_from_double_call(v);
  const uint64_t full = (1ull << 52) | (u & ((1ull << 52) - 1));  // 53-bit significand
  const uint64_t hm = (full + (1ull << 28) - 1 + ((full >> 29) & 1)) >> 29;  // rounded to 24 bits (nearest even)
  int rem = (int)((int64_t)full - (int64_t)(hm << 29));  // |rem| <= 2^28: |v| - |hi| in units of 2^(E-52)
  float hi = __uint2float_rn((uint32_t)hm) * pow2f(E - 23);
  if (u >> 63) { hi = -hi; rem = -rem; }  // the sign on the integer keeps a zero low part +0, as v - hi gives
  return make_float2(hi, __int2float_rn(rem) * pow2f(E - 52));
}

__device__ __forceinline__ double df_to_double_bits(float2 a) {
  const uint32_t hb = __float_as_uint(a.x), lb = __float_as_uint(a.y);
  const int eh = (int)((hb >> 23) & 0xff), el = (int)((lb >> 23) & 0xff);
  if (eh == 0 || eh == 255) return df_to_double_call(a);
  // hi as a 53-bit significand in units of 2^(Eh - 52)
  const int64_t H = (int64_t)((1ull << 23) | (hb & 0x7fffffu)) << 29;
  int64_t S = (hb >> 31) ? -H : H;
  if ((lb << 1) != 0) {
    const int sh = el - eh + 29;  // lo's significand shift into those units (<= 5 for a normalised pair)
    if (el == 0 || el == 255 || sh < 0 || sh > 5) return df_to_double_call(a);
    const int64_t L = (int64_t)((1ull << 23) | (lb & 0x7fffffu)) << sh;
    S += (lb >> 31) ? -L : L;
  }
  const uint64_t neg = S < 0 ? 1ull : 0ull;
  uint64_t m = neg ? (uint64_t)(-S) : (uint64_t)S;
  int e = eh - 127 + 1023;  // biased double exponent of 2^(Eh)
  if (m >= (1ull << 53)) {  // one bit too many: drop it, ties to even
    const uint64_t half = m >> 1;
    m = half + ((m & 1ull) & (half & 1ull));
    e += 1;
    if (m >= (1ull << 53)) { m >>= 1; e += 1; }
  } else if (m < (1ull << 52)) {  // |lo| <= 2^29 units: one step restores 53 bits, exactly
    m <<= 1;
    e -= 1;
  }
  return __longlong_as_double((long long)((neg << 63) | ((uint64_t)e << 52) | (m & ((1ull << 52) - 1))));
}
__device__ __forceinline__ float2 df_shfl_xor(float2 a, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}

// Compensated per-thread sum (the running error of every addition is kept)
struct CSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float2 t = two_sum(s, v);
    s = t.x;
    c = __fadd_rn(c, t.y);
  }
  __device__ __forceinline__ double get() const { return (double)s + (double)c; }
};

// ---------------------------------------------------------------------------
// element access in float (fp32 compute for fp32 / bf16 storage)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ldf(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
__device__ __forceinline__ float ldf(const double *p) { return (float)__ldg(p); }
__device__ __forceinline__ void stf(float *p, float v) { *p = v; }
__device__ __forceinline__ void stf(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }
__device__ __forceinline__ void stf(double *p, float v) { *p = (double)v; }

// Tap p = 9k + 3l + o  <->  offset (k-1, l-1, o-1): the index order of the
// reference's 27 coefficient channels (sm_block_3d_kernel.cu:45-52).
__host__ __device__ __forceinline__ int tap_dx(int p) { return p / 9 - 1; }
__host__ __device__ __forceinline__ int tap_dy(int p) { return (p / 3) % 3 - 1; }
__host__ __device__ __forceinline__ int tap_dz(int p) { return p % 3 - 1; }

// Geometry of a field, either unpadded (halo reads outside [0,N) give 0) or
// padded (halo is the outer layer of an (N+2)^3 array).
struct FieldGeom {
  int n1, n2, n3;     // interior sizes
  int padded;         // 0 or 1
  int64_t sy, sx;     // strides of j and i in elements
  int64_t origin;     // element offset of interior cell (0,0,0)
  int64_t bstride;    // elements between batch items
  __host__ __device__ static FieldGeom make(int n1, int n2, int n3, int padded) {
    FieldGeom g;
    g.n1 = n1; g.n2 = n2; g.n3 = n3; g.padded = padded;
    int p3 = n3 + 2 * padded, p2 = n2 + 2 * padded, p1 = n1 + 2 * padded;
    g.sy = p3;
    g.sx = (int64_t)p2 * p3;
    g.origin = padded ? (g.sx + g.sy + 1) : 0;
    g.bstride = (int64_t)p1 * p2 * p3;
    return g;
  }
  // value at interior coordinates (i,j,k), each in [-1, n]; 0 outside the
  // interior of an unpadded field.
  template <typename T>
  __device__ __forceinline__ float at(const T *base, int i, int j, int k) const {
    if (!padded) {
      if ((unsigned)i >= (unsigned)n1 || (unsigned)j >= (unsigned)n2 || (unsigned)k >= (unsigned)n3)
        return 0.f;
    }
    return ldf(base + origin + i * sx + j * sy + k);
  }
};

// ---------------------------------------------------------------------------
// The 27 coefficients of one cell: acc[p] = bias[p] + sum_{s,m,n,o} W[p][s][m][n][o] * v(s,m,n,o)
// with v the image patch around the cell (v(s,m,n,o) = img(s, q + (m-1,n-1,o-1))),
// the contraction of sm_block_3d_kernel.cu:53-64.
//
// Two forms, chosen per cell:
// * material form, when each of the 27 positions of the patch holds one of the
//   three one-hot materials of the image channels [air, fluid, non-solid]
//   (lib/read_data.py:35-39): solid or outside the grid (0,0,0), air (1,0,1),
//   fluid (0,1,1).  A position's three products then sum to a table entry,
//   Wm[material][position][p] = W[p][0][pos] + W[p][2][pos] (air) or
//   W[p][1][pos] + W[p][2][pos] (fluid), 0 (solid), and the coefficients are
//   acc[p] = bias[p] + sum over the 27 positions, in position order, of the
//   entry of the position's material: 27 additions instead of 81 products.
//   Every cell of a finest-level image made from flags takes this form.
// * product form otherwise (the coarse levels' averaged images): bias, then
//   the 81 products in the reference's loop order (s, m, n, o).
// Both forms add in FP32 (round to nearest); their sums differ from the
// reference's sequence only by rounding.  Every kernel that produces
// coefficients (dense planes, classed records, the uniform vectors of the
// classed layout) goes through these definitions, so equal patches give
// bit-identical coefficients whichever kernel computed them.
//
// Shared-memory layout: sW[(s*27 + 9m+3n+o)*7 + pp] holds W[4pp..4pp+3][s][m][n][o]
// (p padded to 28), sWm[(mat*27 + pos)*7 + pp] the material table, sb[p] the
// bias.  coeffs_of_patch_n evaluates NB blocks on one patch (each patch value
// read once per form): block b at sW / sWm + b * kSW, its bias at sb + b * 28.
// ---------------------------------------------------------------------------
constexpr int kSW = 81 * 7;  // float4 entries of one block's weights (and of its material table)

// material of one patch position: 0 solid / outside, 1 air, 2 fluid, 3 none of the three
__device__ __forceinline__ int patch_material(float a, float f, float s) {
  if (a == 0.f && f == 0.f && s == 0.f) return 0;
  if (a == 1.f && f == 0.f && s == 1.f) return 1;
  if (a == 0.f && f == 1.f && s == 1.f) return 2;
  return 3;
}

// the material table entry of weights W (27 x 81, row p) for material mat at position pos
__device__ __forceinline__ float material_weight(const float *__restrict__ W, int p, int mat, int pos) {
  if (mat == 0) return 0.f;
  return __fadd_rn(W[p * 81 + (mat == 1 ? 0 : 27) + pos], W[p * 81 + 54 + pos]);
}

// The material code of each patch position, 2 bits per position (position
// m * 9 + nn * 3 + o at bits 2 pos); false when a position is none of the
// three one-hot materials.
template <typename Patch>
__device__ __forceinline__ bool patch_materials(Patch v, uint64_t &mats) {
  mats = 0;
  bool material = true;
#pragma unroll
  for (int pos = 0; pos < 27; ++pos) {
    const int m = pos / 9, nn = (pos / 3) % 3, o = pos % 3;
    const int mt = patch_material(v(0, m, nn, o), v(1, m, nn, o), v(2, m, nn, o));
    material = material && mt != 3;
    mats |= (uint64_t)(mt & 3) << (2 * pos);
  }
  return material;
}

// The material form: the bias plus, position by position, the material's
// table row (27 additions per coefficient).
template <int NB>
__device__ __forceinline__ void coeffs_of_materials_n(const float4 *sWm, const float *sb, uint64_t mats,
                                                      float (*acc)[28]) {
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int p = 0; p < 28; ++p) acc[b][p] = sb[b * 28 + p];
#pragma unroll
  for (int pos = 0; pos < 27; ++pos) {
    const int mt = (int)((mats >> (2 * pos)) & 3u);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const float4 *w = sWm + b * kSW + (mt * 27 + pos) * 7;
#pragma unroll
      for (int pp = 0; pp < 7; ++pp) {
        const float4 wv = w[pp];
        acc[b][4 * pp + 0] = __fadd_rn(acc[b][4 * pp + 0], wv.x);
        acc[b][4 * pp + 1] = __fadd_rn(acc[b][4 * pp + 1], wv.y);
        acc[b][4 * pp + 2] = __fadd_rn(acc[b][4 * pp + 2], wv.z);
        acc[b][4 * pp + 3] = __fadd_rn(acc[b][4 * pp + 3], wv.w);
      }
    }
  }
}

template <int NB, typename Patch>
__device__ __forceinline__ void coeffs_of_patch_n(const float4 *sW, const float4 *sWm, const float *sb, Patch v,
                                                  float (*acc)[28]) {
  uint64_t mats;
  if (patch_materials(v, mats)) {
    coeffs_of_materials_n<NB>(sWm, sb, mats, acc);
    return;
  }
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int p = 0; p < 28; ++p) acc[b][p] = sb[b * 28 + p];
  for (int s = 0; s < 3; ++s) {
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int nn = 0; nn < 3; ++nn)
#pragma unroll
        for (int o = 0; o < 3; ++o) {
          const float x = v(s, m, nn, o);
#pragma unroll
          for (int b = 0; b < NB; ++b) {
            const float4 *w = sW + b * kSW + (s * 27 + m * 9 + nn * 3 + o) * 7;
#pragma unroll
            for (int pp = 0; pp < 7; ++pp) {
              const float4 wv = w[pp];
              acc[b][4 * pp + 0] = fmaf(wv.x, x, acc[b][4 * pp + 0]);
              acc[b][4 * pp + 1] = fmaf(wv.y, x, acc[b][4 * pp + 1]);
              acc[b][4 * pp + 2] = fmaf(wv.z, x, acc[b][4 * pp + 2]);
              acc[b][4 * pp + 3] = fmaf(wv.w, x, acc[b][4 * pp + 3]);
            }
          }
        }
  }
}
template <typename Patch>
__device__ __forceinline__ void coeffs_of_patch(const float4 *sW, const float4 *sWm, const float *sb, Patch v,
                                                float acc[28]) {
  coeffs_of_patch_n<1>(sW, sWm, sb, v, reinterpret_cast<float (*)[28]>(acc));
}

// The coefficients of a patch whose 27 positions all hold material mat (the
// uniform vectors of the classed layout): the material form, from global W.
__device__ __forceinline__ float uniform_coeff(const float *__restrict__ W, const float *__restrict__ bias, int p,
                                               int mat) {
  float acc = bias[p];
  for (int pos = 0; pos < 27; ++pos) acc = __fadd_rn(acc, material_weight(W, p, mat, pos));
  return acc;
}

// Loads W (27 x 81), its material table and the bias (27) into the shared-memory layout of
// coeffs_of_patch.
__device__ __forceinline__ void load_weights_smem(const float *__restrict__ W, const float *__restrict__ bias,
                                                  float4 *sW, float4 *sWm, float *sb) {
  float *sWf = reinterpret_cast<float *>(sW);
  float *sWmf = reinterpret_cast<float *>(sWm);
  for (int t = threadIdx.x; t < 81 * 28; t += blockDim.x) {
    const int so = t / 28, p = t % 28;
    sWf[t] = p < 27 ? W[p * 81 + so] : 0.f;
    sWmf[t] = p < 27 ? material_weight(W, p, so / 27, so % 27) : 0.f;
  }
  if (threadIdx.x < 28) sb[threadIdx.x] = threadIdx.x < 27 ? bias[threadIdx.x] : 0.f;
}

}  // namespace mlpcg
