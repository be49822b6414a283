// Preconditioner plan: every block's coefficients precomputed once per
// (image, weights), applied by fused, tiled, bandwidth-bound kernels.
//
// SmallSMModelDn3D.eval_forward (sm_model_3d.py:180-262) on one rhs becomes
// 2n+2 launches:
//   pre_l   y_l = B_pre_l(x_l)          fused with x_{l+1} = avg_pool(y_l)
//   l       x_n = B_l(x_n)
//   post_l  x_l = c0_l y_l + c1_l B_post_l(up(x_{l+1}))   (prolongation + combine fused)
// (or, with swap_sm_order, x_l = B_post_l(c0_l y_l + c1_l up(x_{l+1}))).
// At the finest level the prolongation is a pass of its own (k_up_fine)
// whose output the post-block stages like any input: interpolating the
// tile's halo cells inside the block kernel cost more than the extra pass.
// Levels whose z size is not a multiple of 8 use the general kernels of
// stencil.cu / gridops.cu instead.
//
// Tile: 2 (x) x 16 (y) x 64 (z) outputs per 128-thread CTA; each thread owns
// a run of 8 consecutive z cells in 2 x-planes.  The input with its one-cell
// halo is staged in shared memory (4 x 18 x 66 floats in rows of 76): the
// staging issues all of a thread's global loads (16-byte vectors) before its
// first shared store, and each run reads its 9 input rows as three 16-byte
// shared loads apiece.  Coefficients stream from HBM as 16-byte vectors
// (8 BF16 or 4 FP32 values) with the cache-streaming hint, since each is
// read exactly once per application.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <type_traits>
#include <vector>
#include "common.cuh"

namespace mlpcg {

constexpr int TZ = 64, TY = 16, TX = 2;
constexpr int ZT = 8;                 // threads along z, 8 cells each
constexpr int PT = ZT * TY;           // 128 threads
constexpr int HZ = TZ + 2, HY = TY + 2, HX = TX + 2;
constexpr int HZP = 76;               // shared row stride: 16-byte aligned, = 12 (mod 32) floats
constexpr int CZ = TZ / 2 + 2, CY = TY / 2 + 2, CX = TX / 2 + 2;
constexpr int CZP = 48;               // coarse-tile row stride: 16-byte aligned, = 16 (mod 32) floats
constexpr int NVR = TZ / 4;           // 4-wide vectors in a row's interior

// Thread t owns the runs (tx, run_ty(t), 8 run_tz(t) .. +7).  Each group of 8
// consecutive lanes covers 4 tz by 2 ty, so with the row stride above the
// group's 16-byte shared loads of one tile row fall in 8 distinct bank quads.
__device__ __forceinline__ int run_tz(int t) { return (t & 3) | ((t >> 1) & 4); }
__device__ __forceinline__ int run_ty(int t) { return ((t >> 2) & 1) | ((t >> 3) & 2) | ((t >> 5) << 2); }
constexpr unsigned kTyPairLane = 4;   // lane distance between the runs of ty and ty ^ 1

// 4 consecutive values as floats (16-byte / 8-byte aligned vector load)
__device__ __forceinline__ float4 ldv4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ float4 ldv4(const __nv_bfloat16 *p) {
  const uint2 u = __ldg(reinterpret_cast<const uint2 *>(p));
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                     __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
}

// Activation loads of the block bodies.  COH = false: the read-only data path (__ldg), for inputs
// written by earlier kernels; COH = true: through L2 only (__ldcg), for inputs that other CTAs of
// the same launch wrote before a cluster barrier (the coarse-level cluster kernel).
template <bool COH> __device__ __forceinline__ float4 ldv4c(const float *p) {
  return COH ? __ldcg(reinterpret_cast<const float4 *>(p)) : __ldg(reinterpret_cast<const float4 *>(p));
}
template <bool COH> __device__ __forceinline__ float4 ldv4c(const __nv_bfloat16 *p) {
  const uint2 u = COH ? __ldcg(reinterpret_cast<const uint2 *>(p)) : __ldg(reinterpret_cast<const uint2 *>(p));
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                     __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
}
template <bool COH> __device__ __forceinline__ float ldfc(const float *p) { return COH ? __ldcg(p) : __ldg(p); }
template <bool COH> __device__ __forceinline__ float ldfc(const __nv_bfloat16 *p) {
  if (COH) {
    const unsigned short u = __ldcg(reinterpret_cast<const unsigned short *>(p));
    return __uint_as_float((uint32_t)u << 16);
  }
  return __bfloat162float(*p);
}

// The tile a CTA works on: tile coordinates (bx: z, by: y, bz: x, in units of TZ, TY, TX) and the
// linear tile index bx + gx (by + gy bz).  A kernel launched over the tile grid takes its own block
// index (grid_tile); the coarse-level cluster kernel walks the tiles of each level itself.
struct Tile {
  int bx, by, bz;
  unsigned id;
};
__device__ __forceinline__ Tile grid_tile() {
  return Tile{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z,
              blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)};
}

// The 16 tile values S[row][z .. z + 15] (z a multiple of 4) by four 16-byte loads
__device__ __forceinline__ void ld_row16(const float *row, float xr[16]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 a = reinterpret_cast<const float4 *>(row)[q];
    xr[4 * q] = a.x; xr[4 * q + 1] = a.y; xr[4 * q + 2] = a.z; xr[4 * q + 3] = a.w;
  }
}

// The 12 tile values S[row][z .. z + 11] (z a multiple of 4) by three 16-byte loads
__device__ __forceinline__ void ld_row12(const float *row, float xr[12]) {
  const float4 a = reinterpret_cast<const float4 *>(row)[0];
  const float4 b = reinterpret_cast<const float4 *>(row)[1];
  const float4 c = reinterpret_cast<const float4 *>(row)[2];
  xr[0] = a.x; xr[1] = a.y; xr[2] = a.z; xr[3] = a.w;
  xr[4] = b.x; xr[5] = b.y; xr[6] = b.z; xr[7] = b.w;
  xr[8] = c.x; xr[9] = c.y; xr[10] = c.z; xr[11] = c.w;
}

// Fine-tile staging in two halves: load() issues every global load of the
// thread (its 9 interior vectors and at most 2 z-halo values), put() writes
// them to the tile.  Row r = hx * HY + hy; interior vector v of a row covers
// k = z0 + 4 v .. + 3 (tile z index 4 v + 1 ..), the halo values k = z0 - 1
// and z0 + TZ (tile z index 0 and HZ - 1).  Outside the grid the value is 0.
constexpr int kStageVec = HX * HY * NVR / PT;  // 9
constexpr int kStageHalo = 2;                  // 2 * HX * HY = 144 halo values over 128 threads
static_assert(HX * HY * NVR % PT == 0 && 2 * HX * HY <= kStageHalo * PT, "staging split");
struct FineStage {
  float4 v[kStageVec];
  float h[kStageHalo];
};
__device__ __forceinline__ int stage_vec_row(int m) { return threadIdx.x / NVR + m * (PT / NVR); }
__device__ __forceinline__ int stage_halo_id(int m) { return threadIdx.x + m * PT; }

template <typename F4, typename F1>
__device__ __forceinline__ void stage_load(FineStage &st, const Tile &t, int n1, int n2, int n3, F4 ld4, F1 ld1) {
  const int z0 = t.bx * TZ, y0 = t.by * TY, x0 = t.bz * TX;
  const int k = z0 + 4 * (threadIdx.x % NVR);
#pragma unroll
  for (int m = 0; m < kStageVec; ++m) {
    const int r = stage_vec_row(m), i = x0 + r / HY - 1, j = y0 + r % HY - 1;
    st.v[m] = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && k < n3)
      st.v[m] = ld4(i, j, k, ((int64_t)i * n2 + j) * n3 + k);
  }
#pragma unroll
  for (int m = 0; m < kStageHalo; ++m) {
    const int e = stage_halo_id(m), r = e >> 1;
    const int i = x0 + r / HY - 1, j = y0 + r % HY - 1, kk = (e & 1) ? z0 + TZ : z0 - 1;
    st.h[m] = 0.f;
    if (e < 2 * HX * HY && (unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && (unsigned)kk < (unsigned)n3)
      st.h[m] = ld1(i, j, kk, ((int64_t)i * n2 + j) * n3 + kk);
  }
}
__device__ __forceinline__ void stage_put(float (*S)[HY][HZP], const FineStage &st) {
  const int v = threadIdx.x % NVR;
#pragma unroll
  for (int m = 0; m < kStageVec; ++m) {
    const int r = stage_vec_row(m);
    float *row = &S[r / HY][r % HY][4 * v + 1];
    row[0] = st.v[m].x;
    *reinterpret_cast<float2 *>(row + 1) = make_float2(st.v[m].y, st.v[m].z);
    row[3] = st.v[m].w;
  }
#pragma unroll
  for (int m = 0; m < kStageHalo; ++m) {
    const int e = stage_halo_id(m), r = e >> 1;
    if (e < 2 * HX * HY) S[r / HY][r % HY][(e & 1) ? HZ - 1 : 0] = st.h[m];
  }
}

// ---- 8-wide vector access --------------------------------------------------
__device__ __forceinline__ void ld8cs(const float *p, float v[8]) {
  const float4 a = __ldcs(reinterpret_cast<const float4 *>(p));
  const float4 b = __ldcs(reinterpret_cast<const float4 *>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void unpack_bf16x2(uint32_t u, float &lo, float &hi) {
  lo = __uint_as_float(u << 16);
  hi = __uint_as_float(u & 0xffff0000u);
}
__device__ __forceinline__ void ld8cs(const __nv_bfloat16 *p, float v[8]) {
  const uint4 u = __ldcs(reinterpret_cast<const uint4 *>(p));
  unpack_bf16x2(u.x, v[0], v[1]); unpack_bf16x2(u.y, v[2], v[3]);
  unpack_bf16x2(u.z, v[4], v[5]); unpack_bf16x2(u.w, v[6], v[7]);
}
__device__ __forceinline__ void ld8(const float *p, float v[8]) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void ld8(const __nv_bfloat16 *p, float v[8]) {
  const uint4 u = __ldg(reinterpret_cast<const uint4 *>(p));
  unpack_bf16x2(u.x, v[0], v[1]); unpack_bf16x2(u.y, v[2], v[3]);
  unpack_bf16x2(u.z, v[4], v[5]); unpack_bf16x2(u.w, v[6], v[7]);
}
// ld8 for activations: through L2 only (COH) or the read-only path
template <bool COH> __device__ __forceinline__ void ld8c(const float *p, float v[8]) {
  if (!COH) return ld8(p, v);
  const float4 a = __ldcg(reinterpret_cast<const float4 *>(p));
  const float4 b = __ldcg(reinterpret_cast<const float4 *>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <bool COH> __device__ __forceinline__ void ld8c(const __nv_bfloat16 *p, float v[8]) {
  if (!COH) return ld8(p, v);
  const uint4 u = __ldcg(reinterpret_cast<const uint4 *>(p));
  unpack_bf16x2(u.x, v[0], v[1]); unpack_bf16x2(u.y, v[2], v[3]);
  unpack_bf16x2(u.z, v[4], v[5]); unpack_bf16x2(u.w, v[6], v[7]);
}
__device__ __forceinline__ void st8(float *p, const float v[8]) {
  reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
  reinterpret_cast<float4 *>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
}
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}
__device__ __forceinline__ void st8(__nv_bfloat16 *p, const float v[8]) {
  uint4 u;
  u.x = pack_bf16x2(v[0], v[1]); u.y = pack_bf16x2(v[2], v[3]);
  u.z = pack_bf16x2(v[4], v[5]); u.w = pack_bf16x2(v[6], v[7]);
  *reinterpret_cast<uint4 *>(p) = u;
}
__device__ __forceinline__ void st4(float *p, const float v[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(__nv_bfloat16 *p, const float v[4]) {
  uint2 u;
  u.x = pack_bf16x2(v[0], v[1]);
  u.y = pack_bf16x2(v[2], v[3]);
  *reinterpret_cast<uint2 *>(p) = u;
}

// ---------------------------------------------------------------------------
// Classed coefficients.  A block's 27 coefficients at a cell depend only on
// the 3 x 27 image values around it.  Where those are all one of the three
// one-hot materials -- solid (or outside the grid) (0,0,0), air (1,0,1),
// fluid (0,1,1) -- the coefficients are the block's constant vector for that
// material ("uniform" cells); the other ("general") cells lie near material
// interfaces.  A classed level describes each 8-cell z-run (the unit a thread
// applies) by one word: a run whose 8 cells are uniform cells of one
// material is that material's run; every other run is "mixed" and has a
// record of its 27 x 8 coefficients.  The R mixed runs of a tile (numbered in
// thread / run order) keep their records together, tap-major across the
// runs -- coefficient p of cell c of the tile's mixed run r at
// (p * R + r) * 8 + c -- so that a warp's loads of one tap are contiguous,
// as they are in the dense planes.
// Results equal those of the dense planes bit for bit: coeffs_of_patch_n
// (material or product form, per patch) produces every value and the 27 taps
// are summed in the same order.
// ---------------------------------------------------------------------------
enum { CLS_SOLID = 0, CLS_AIR = 1, CLS_FLUID = 2, CLS_GENERAL = 3 };
constexpr int KREC = 32;        // uniform vectors: 27 values padded to 32
constexpr int RREC = 27 * 8;    // coefficients of a mixed run's record
constexpr uint32_t kMixed = 3;  // run word: bits 0-1 material or kMixed, bits 2.. mixed-run index in the tile

// the class codes of the materials are patch_material's
static_assert(CLS_SOLID == 0 && CLS_AIR == 1 && CLS_FLUID == 2 && CLS_GENERAL == 3, "material codes");

// ---------------------------------------------------------------------------
// Neighbourhood pattern table (level 0 of a one-hot image; see k_pattern_coeffs).
// ---------------------------------------------------------------------------
constexpr int kPatBits = 19;
constexpr uint32_t kPatSlots = 1u << kPatBits;  // hash slots
constexpr uint32_t kPatMax = 1u << 17;          // distinct patterns with table values
constexpr int kPatProbe = 64;                   // slots tried per insertion
constexpr unsigned long long kPatEmpty = ~0ull; // no 54-bit key has all bits set
constexpr uint32_t kNoPattern = 0xffffffffu;

// The pattern table as the record writers see it: cell_slot[q] is general cell q's hash slot
// (kNoPattern: none), pidx[slot] its table entry (kNoPattern: none), pcoef the entries'
// coefficients (NB blocks x 28 floats each), *fail nonzero when some general cell has no table
// values.  cell_slot == NULL: no table.
struct PatternArgs {
  const uint32_t *cell_slot, *pidx;
  const float *pcoef;
  const uint32_t *fail;
};

// key's slot in the open-addressed table (linear probing from its hash, at most kPatProbe slots;
// an empty slot is claimed with one compare-and-swap), or kNoPattern when the probe runs out
__device__ __forceinline__ uint32_t pattern_insert(unsigned long long *keys, unsigned long long key) {
  const uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - kPatBits));
  for (int p = 0; p < kPatProbe; ++p) {
    const uint32_t sl = (h + (uint32_t)p) & (kPatSlots - 1);
    unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(keys + sl);
    if (cur == kPatEmpty) cur = atomicCAS(keys + sl, kPatEmpty, key);
    if (cur == kPatEmpty || cur == key) return sl;
  }
  return kNoPattern;
}
__device__ __forceinline__ int material_of(float a, float f, float s) { return patch_material(a, f, s); }
__device__ __forceinline__ int class_of(uint2 cw, int c) {
  return (int)(((c < 4 ? cw.x : cw.y) >> (8 * (c & 3))) & 0xffu);
}

// exclusive scan of one int per thread over the PT threads of a CTA
__device__ __forceinline__ int cta_excl_scan(int v, int &total) {
  __shared__ int ws[PT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  int off = 0, tot = 0;
#pragma unroll
  for (int i = 0; i < PT / 32; ++i) {
    if (i < w) off += ws[i];
    tot += ws[i];
  }
  __syncthreads();
  total = tot;
  return off + x - v;
}

__device__ __forceinline__ unsigned tile_id() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// run words of the thread's two runs (uniform solid for a run outside the grid)
__device__ __forceinline__ void load_run_words(const uint32_t *__restrict__ rw, const Tile &t, int n1, int n2,
                                               int n3, uint32_t w[TX]) {
  const int k0 = t.bx * TZ + run_tz(threadIdx.x) * 8, j = t.by * TY + run_ty(threadIdx.x);
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = t.bz * TX + tx;
    w[tx] = CLS_SOLID;
    if (k0 < n3 && j < n2 && i < n1) w[tx] = __ldg(rw + ((((int64_t)i * n2 + j) * n3 + k0) >> 3));
  }
}

// material code of component c of three channel vectors
__device__ __forceinline__ uint8_t material_at(float4 a, float4 f, float4 s, int c) {
  const float av = c == 0 ? a.x : c == 1 ? a.y : c == 2 ? a.z : a.w;
  const float fv = c == 0 ? f.x : c == 1 ? f.y : c == 2 ? f.z : f.w;
  const float sv = c == 0 ? s.x : c == 1 ? s.y : c == 2 ? s.z : s.w;
  return (uint8_t)material_of(av, fv, sv);
}

// Class byte of every cell, the word of every run, and per tile the numbers
// of mixed runs (rcount) and of general cells (gcount).  The tile's codes
// (with a one-cell halo; outside the grid = solid) are staged in shared
// memory; a cell is uniform when all 27 codes around it agree.
// FROM_CLS = false: the codes are the cells' materials, loaded as 4-wide
// vectors of the three image channels (the classes of a forward block).
// FROM_CLS = true: the codes are the forward block's class bytes (src_cls),
// which gives the classes of the transposed block: its coefficients at q are
// the forward ones of q's 27 neighbours, uniform when those all are alike.
template <bool FROM_CLS>
__global__ void __launch_bounds__(PT)
k_classify(const float *__restrict__ img, const uint8_t *__restrict__ src_cls, int n1, int n2, int n3,
           uint8_t *__restrict__ cls, uint32_t *__restrict__ rw, uint32_t *__restrict__ rcount,
           uint32_t *__restrict__ gcount, unsigned long long *__restrict__ pkeys, uint32_t *__restrict__ cell_slot,
           uint32_t *__restrict__ pfail) {
  dependent_launch_enter();
  __shared__ __align__(16) uint8_t M[HX][HY][HZP];
  const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TY, x0 = blockIdx.z * TX;
  const int64_t n = cells(n1, n2, n3);
  if (FROM_CLS) {
    const int v = threadIdx.x % NVR, k = z0 + 4 * v;
    uint32_t w[kStageVec];
#pragma unroll
    for (int m = 0; m < kStageVec; ++m) {
      const int r = stage_vec_row(m), i = x0 + r / HY - 1, j = y0 + r % HY - 1;
      const bool in = (unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && k < n3;
      // 4 class bytes (k a multiple of 4, n3 of 8: 4-byte aligned); 0 = CLS_SOLID outside
      w[m] = in ? __ldg(reinterpret_cast<const uint32_t *>(src_cls + ((int64_t)i * n2 + j) * n3 + k)) : 0u;
    }
#pragma unroll
    for (int m = 0; m < kStageVec; ++m) {
      const int r = stage_vec_row(m);
#pragma unroll
      for (int c = 0; c < 4; ++c) M[r / HY][r % HY][4 * v + 1 + c] = (uint8_t)(w[m] >> (8 * c));
    }
#pragma unroll
    for (int m = 0; m < kStageHalo; ++m) {
      const int e = stage_halo_id(m), r = e >> 1;
      if (e >= 2 * HX * HY) continue;
      const int i = x0 + r / HY - 1, j = y0 + r % HY - 1, kk = (e & 1) ? z0 + TZ : z0 - 1;
      uint8_t mc = CLS_SOLID;
      if ((unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && (unsigned)kk < (unsigned)n3)
        mc = src_cls[((int64_t)i * n2 + j) * n3 + kk];
      M[r / HY][r % HY][(e & 1) ? HZ - 1 : 0] = mc;
    }
  } else {
    const int v = threadIdx.x % NVR, k = z0 + 4 * v;
    // the interior in 3 batches of 3 vectors per channel, every load of a batch in flight together
#pragma unroll
    for (int b = 0; b < kStageVec / 3; ++b) {
      float4 ch[3][3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const int r = stage_vec_row(3 * b + m), i = x0 + r / HY - 1, j = y0 + r % HY - 1;
        const bool in = (unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && k < n3;
        const int64_t q = ((int64_t)i * n2 + j) * n3 + k;
#pragma unroll
        for (int s = 0; s < 3; ++s)
          ch[m][s] = in ? __ldg(reinterpret_cast<const float4 *>(img + s * n + q)) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const int r = stage_vec_row(3 * b + m);
#pragma unroll
        for (int c = 0; c < 4; ++c) M[r / HY][r % HY][4 * v + 1 + c] = material_at(ch[m][0], ch[m][1], ch[m][2], c);
      }
    }
#pragma unroll
    for (int m = 0; m < kStageHalo; ++m) {
      const int e = stage_halo_id(m), r = e >> 1;
      if (e >= 2 * HX * HY) continue;
      const int i = x0 + r / HY - 1, j = y0 + r % HY - 1, kk = (e & 1) ? z0 + TZ : z0 - 1;
      int mc = CLS_SOLID;
      if ((unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && (unsigned)kk < (unsigned)n3) {
        const int64_t q = ((int64_t)i * n2 + j) * n3 + kk;
        mc = material_of(img[q], img[n + q], img[2 * n + q]);
      }
      M[r / HY][r % HY][(e & 1) ? HZ - 1 : 0] = (uint8_t)mc;
    }
  }
  __syncthreads();
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int k0 = z0 + tz * 8, j = y0 + ty;
  int ngen = 0, nmixed = 0;
  uint32_t word[TX] = {CLS_SOLID, CLS_SOLID};
  bool mixed[TX] = {false, false};
  if (k0 < n3 && j < n2) {
#pragma unroll
    for (int tx = 0; tx < TX; ++tx) {
      const int i = x0 + tx;
      if (i >= n1) continue;
      // per cell: the set of material codes seen in its 3 x 3 x 3 neighbourhood, as bits
      uint32_t seen[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
      for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
          uint32_t rowbits[10];
#pragma unroll
          for (int c = 0; c < 10; ++c) rowbits[c] = 1u << M[tx + dx][ty + dy][tz * 8 + c];
#pragma unroll
          for (int c = 0; c < 8; ++c) seen[c] |= rowbits[c] | rowbits[c + 1] | rowbits[c + 2];
        }
      uint32_t w[2] = {0u, 0u}, all = 0u;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        // uniform: exactly one code seen, and it is not the general code
        const uint32_t sc = seen[c];
        const int cl = (__popc(sc) == 1 && !(sc & (1u << CLS_GENERAL))) ? (__ffs(sc) - 1) : CLS_GENERAL;
        w[c >> 2] |= (uint32_t)cl << (8 * (c & 3));
        ngen += cl == CLS_GENERAL;
        all |= 1u << cl;
      }
      *reinterpret_cast<uint2 *>(cls + ((int64_t)i * n2 + j) * n3 + k0) = make_uint2(w[0], w[1]);
      if (!FROM_CLS && pkeys) {
        // each general cell's neighbourhood pattern -- 27 material codes, 2 bits each -- into the table
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
          if (((w[c >> 2] >> (8 * (c & 3))) & 0xffu) != CLS_GENERAL) continue;
          unsigned long long key = 0;
          bool one_hot = true;
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
              for (int dz = 0; dz < 3; ++dz) {
                const uint32_t code = M[tx + dx][ty + dy][tz * 8 + c + dz];
                one_hot = one_hot && code != 3u;
                key |= (unsigned long long)(code & 3u) << (2 * (dx * 9 + dy * 3 + dz));
              }
          const uint32_t slot = one_hot ? pattern_insert(pkeys, key) : kNoPattern;
          if (slot == kNoPattern) atomicOr(pfail, 1u);
          cell_slot[((int64_t)i * n2 + j) * n3 + k0 + c] = slot;
        }
      }
      mixed[tx] = __popc(all) != 1 || (all & (1u << CLS_GENERAL));
      word[tx] = mixed[tx] ? kMixed : (uint32_t)(__ffs(all) - 1);
      nmixed += mixed[tx];
    }
  }
  int rtot, gtot;
  int pos = cta_excl_scan(nmixed, rtot);
  cta_excl_scan(ngen, gtot);
  if (k0 < n3 && j < n2) {
#pragma unroll
    for (int tx = 0; tx < TX; ++tx) {
      const int i = x0 + tx;
      if (i >= n1) continue;
      if (mixed[tx]) word[tx] |= (uint32_t)(pos++) << 2;
      rw[(((int64_t)i * n2 + j) * n3 + k0) >> 3] = word[tx];
    }
  }
  if (threadIdx.x == 0) {
    rcount[tile_id()] = (uint32_t)rtot;
    gcount[tile_id()] = (uint32_t)gtot;
  }
}

// exclusive prefix sum of the tile counts (one CTA of 1024 threads)
__global__ void __launch_bounds__(1024)
k_scan_tiles(const uint32_t *__restrict__ cnt, uint32_t *__restrict__ base, int ntiles) {
  dependent_launch_enter();
  __shared__ uint32_t ws[32];
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int start = 0; start < ntiles; start += 1024) {
    const int idx = start + threadIdx.x;
    const uint32_t v = idx < ntiles ? cnt[idx] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t s = ws[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      ws[lane] = s;
    }
    __syncthreads();
    const uint32_t prefix = carry + (w > 0 ? ws[w - 1] : 0u) + x - v;
    if (idx < ntiles) base[idx] = prefix;
    __syncthreads();
    if (threadIdx.x == 1023) carry = prefix + v;
    __syncthreads();
  }
}

// v rounded to the storage type of the first argument's pointee
__device__ __forceinline__ float round_as(const float *, float v) { return v; }
__device__ __forceinline__ float round_as(const __nv_bfloat16 *, float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

// The coefficient vector of each uniform material for every block of the
// model (blockIdx.x = parameter block b, at params + b * 2214), rounded like
// the stored dtype: thread (c, p) evaluates output p of material c in the
// material form of coeffs_of_patch_n (uniform_coeff), so it equals what that
// function yields on a patch of material c.  Block b's vectors go to slot b, and for
// the symmetric networks its transpose's, the reversed vector (tap 26 - p),
// to a second slot: kind MLPCG_PRECOND_SMALL_SPD (parameter blocks l0[0..n-1],
// l) puts l0[b] in slot b and its transpose in n + b, l in 2n and l_t in
// 2n + 1; kind MLPCG_PRECOND_SPD (blocks l0[0..n-1], l1[0..n-1], l) puts
// block b in slot b and its transpose in 2n + 1 + b.
template <typename KT>
__global__ void __launch_bounds__(3 * KREC)
k_kgen_uniform_all(const float *__restrict__ params, float *__restrict__ kuni, int n, int kind) {
  dependent_launch_enter();
  const int b = blockIdx.x, c = threadIdx.x / KREC, p = threadIdx.x % KREC;
  const float *W = params + (size_t)b * 2214, *bias = W + 2187;
  float acc = 0.f;
  if (p < 27) acc = round_as((const KT *)nullptr, uniform_coeff(W, bias, p, c));
  if (kind == MLPCG_PRECOND_SM) {
    kuni[(size_t)b * 3 * KREC + threadIdx.x] = acc;
    return;
  }
  int sf = b, sr = 2 * n + 1 + b;
  if (kind == MLPCG_PRECOND_SMALL_SPD) {
    sf = b < n ? b : 2 * n;
    sr = b < n ? n + b : 2 * n + 1;
  }
  kuni[(size_t)sf * 3 * KREC + threadIdx.x] = acc;
  kuni[(size_t)sr * 3 * KREC + c * KREC + (p < 27 ? 26 - p : p)] = acc;
}

// The linear index of every general cell, tile by tile in thread / run / cell
// order: list[gbase[tile] + rank] = q; and the run index (q / 8) of every
// mixed run at its record position: rlist[rbase[tile] + local index].
__global__ void __launch_bounds__(PT)
k_list_general(const uint8_t *__restrict__ cls, int n1, int n2, int n3, const uint32_t *__restrict__ gbase,
               uint32_t *__restrict__ list, const uint32_t *__restrict__ rw, const uint32_t *__restrict__ rbase,
               uint32_t *__restrict__ rlist) {
  dependent_launch_enter();
  const int k0 = blockIdx.x * TZ + run_tz(threadIdx.x) * 8, j = blockIdx.y * TY + run_ty(threadIdx.x);
  uint2 cw[TX];
  uint32_t gm[TX];
  int cnt = 0;
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = blockIdx.z * TX + tx;
    cw[tx] = make_uint2(0u, 0u);
    if (k0 < n3 && j < n2 && i < n1) {
      const int64_t q0 = ((int64_t)i * n2 + j) * n3 + k0;
      cw[tx] = __ldg(reinterpret_cast<const uint2 *>(cls + q0));
      const uint32_t word = __ldg(rw + (q0 >> 3));
      if ((word & 3u) == kMixed) rlist[__ldg(rbase + tile_id()) + (word >> 2)] = (uint32_t)(q0 >> 3);
    }
    gm[tx] = 0u;
#pragma unroll
    for (int c = 0; c < 8; ++c) gm[tx] |= (class_of(cw[tx], c) == CLS_GENERAL ? 1u : 0u) << c;
    cnt += __popc(gm[tx]);
  }
  int tot;
  uint32_t pos = __ldg(gbase + tile_id()) + (uint32_t)cta_excl_scan(cnt, tot);
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    if (!gm[tx]) continue;
    const uint32_t q0 = (uint32_t)((((int64_t)blockIdx.z * TX + tx) * n2 + j) * n3 + k0);
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (gm[tx] & (1u << c)) list[pos++] = q0 + c;
  }
}

// Where the coefficients of cell q (in a mixed run) live: coefficient p at
// offset + p * stride of the level's record array.
struct RecPos {
  size_t offset, stride;
};
__device__ __forceinline__ RecPos rec_pos(const uint32_t *__restrict__ rw, const uint32_t *__restrict__ rbase,
                                          const uint32_t *__restrict__ rcount, uint32_t q, int i, int j, int k,
                                          int n2, int n3) {
  const uint32_t tile = (uint32_t)(k / TZ) + (uint32_t)((n3 + TZ - 1) / TZ) *
                        ((uint32_t)(j / TY) + (uint32_t)((n2 + TY - 1) / TY) * (uint32_t)(i / TX));
  const size_t R = __ldg(rcount + tile);
  RecPos rp;
  rp.offset = (size_t)__ldg(rbase + tile) * RREC + (size_t)(__ldg(rw + (q >> 3)) >> 2) * 8 + (q & 7u);
  rp.stride = R * 8;
  return rp;
}

// ---------------------------------------------------------------------------
// Coefficient generation by neighbourhood pattern (level 0 of a one-hot image).
// There every general cell's coefficients depend only on the 27 material codes
// around it (the material form), and few distinct neighbourhoods occur: walls
// and sphere surfaces repeat them.  k_classify puts each general cell's 54-bit
// pattern into an open-addressed hash table (pattern_insert) and records its
// slot; k_pattern_coeffs evaluates every distinct pattern once with the
// arithmetic of the per-cell path into a table; k_fill_runs_pattern writes the
// records from it.  A cell whose patch is not one-hot, whose probe runs out, or
// whose pattern finds no table room (kPatMax) raises the failure flag and is
// evaluated by k_kgen_list as before.  The table order depends on the
// insertion race, the values do not.
// ---------------------------------------------------------------------------

// One warp per occupied hash slot: lane 0 takes the next table entry (while there is room), lane p
// (< 28) sums coefficient p of each block -- the bias, then the material table row of each position
// in order, as coeffs_of_materials_n does -- and stores it.
template <int NB>
__global__ void __launch_bounds__(256)
k_pattern_coeffs(const float *__restrict__ params, int b0, int b1, const unsigned long long *__restrict__ keys,
                 uint32_t *__restrict__ pidx, uint32_t *__restrict__ pcount, float *__restrict__ pcoef,
                 uint32_t *__restrict__ pfail) {
  dependent_launch_enter();
  __shared__ float4 sW[NB * kSW];
  __shared__ float4 sWm[NB * kSW];
  __shared__ float sb[NB * 28];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const float *W = params + (size_t)(b ? b1 : b0) * 2214;
    load_weights_smem(W, W + 2187, sW + b * kSW, sWm + b * kSW, sb + b * 28);
  }
  __syncthreads();
  const float *wm = reinterpret_cast<const float *>(sWm);
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = warp * 32; base < kPatSlots; base += nwarps * 32) {
    const unsigned long long kl = __ldg(keys + base + lane);
    uint32_t occ = __ballot_sync(0xffffffffu, kl != kPatEmpty);
    while (occ) {
      const int src = __ffs(occ) - 1;
      occ &= occ - 1;
      const unsigned long long key = __shfl_sync(0xffffffffu, kl, src);
      uint32_t idx = 0;
      if (lane == 0) idx = atomicAdd(pcount, 1u);
      idx = __shfl_sync(0xffffffffu, idx, 0);
      if (idx >= kPatMax) {
        if (lane == 0) {
          pidx[base + src] = kNoPattern;
          atomicOr(pfail, 1u);
        }
        continue;
      }
      if (lane < 28) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          float acc = sb[b * 28 + lane];
#pragma unroll
          for (int pos = 0; pos < 27; ++pos) {
            const int mt = (int)((key >> (2 * pos)) & 3u);
            acc = __fadd_rn(acc, wm[b * kSW * 4 + (mt * 27 + pos) * 28 + lane]);
          }
          pcoef[(size_t)idx * NB * 28 + b * 28 + lane] = acc;
        }
      }
      if (lane == 0) pidx[base + src] = idx;
    }
  }
}

// The uniform cells of every mixed run, for NB blocks (uniform vectors at
// kuni0 / kuni1): thread (p, e) writes tap p of the record of mixed run e --
// the run's 8 cells, contiguous in the record -- as one vector store, its
// uniform cells taking their material's value and its general cells 0 until
// k_kgen_list / k_kgen_t_list (launched after it) write theirs.  Consecutive
// threads take consecutive runs of one tap, which sit side by side in a tile's
// record block.  Run indices from rlist, their count read on the device.
template <typename KT, int NB>
__global__ void __launch_bounds__(256)
k_fill_runs(const uint8_t *__restrict__ cls, const uint32_t *__restrict__ rlist,
            const uint32_t *__restrict__ rlast_base, const uint32_t *__restrict__ rlast_count,
            const uint32_t *__restrict__ rw, const uint32_t *__restrict__ rbase, const uint32_t *__restrict__ rcount,
            int n2, int n3, const float *__restrict__ kuni0, const float *__restrict__ kuni1, KT *__restrict__ rec0,
            KT *__restrict__ rec1) {
  dependent_launch_enter();
  const uint64_t nrun = (uint64_t)__ldg(rlast_base) + __ldg(rlast_count);
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 27 * nrun;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const int p = (int)(t / nrun);
    const uint32_t e = (uint32_t)(t - (uint64_t)p * nrun);
    const uint32_t q = 8u * __ldg(rlist + e);
    const int k = (int)(q % (uint32_t)n3);
    const uint32_t r = q / (uint32_t)n3;
    const int j = (int)(r % (uint32_t)n2), i = (int)(r / (uint32_t)n2);
    const RecPos rp = rec_pos(rw, rbase, rcount, q, i, j, k, n2, n3);
    const uint2 cw = __ldg(reinterpret_cast<const uint2 *>(cls + q));
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const float *ku = (b ? kuni1 : kuni0) + p;
      float v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int cl = class_of(cw, c);
        v[c] = cl == CLS_GENERAL ? 0.f : __ldg(ku + cl * KREC);
      }
      st8((b ? rec1 : rec0) + rp.offset + (size_t)p * rp.stride, v);
    }
  }
}

// k_fill_runs with the pattern table (level 0): thread e writes the whole record of mixed run e,
// looking up its general cells' table entries once; for each tap, consecutive threads store
// consecutive runs' 16 bytes.  General cells without table values are written 0 (k_kgen_list
// evaluates them afterwards).
template <typename KT, int NB>
__global__ void __launch_bounds__(256)
k_fill_runs_pattern(const uint8_t *__restrict__ cls, const uint32_t *__restrict__ rlist,
                    const uint32_t *__restrict__ rlast_base, const uint32_t *__restrict__ rlast_count,
                    const uint32_t *__restrict__ rw, const uint32_t *__restrict__ rbase,
                    const uint32_t *__restrict__ rcount, int n2, int n3, const float *__restrict__ kuni0,
                    const float *__restrict__ kuni1, KT *__restrict__ rec0, KT *__restrict__ rec1,
                    const PatternArgs pat) {
  dependent_launch_enter();
  const uint32_t nrun = __ldg(rlast_base) + __ldg(rlast_count);
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nrun; e += gridDim.x * blockDim.x) {
    const uint32_t q = 8u * __ldg(rlist + e);
    const int k = (int)(q % (uint32_t)n3);
    const uint32_t r = q / (uint32_t)n3;
    const int j = (int)(r % (uint32_t)n2), i = (int)(r / (uint32_t)n2);
    const RecPos rp = rec_pos(rw, rbase, rcount, q, i, j, k, n2, n3);
    const uint2 cw = __ldg(reinterpret_cast<const uint2 *>(cls + q));
    // per cell: a material (0..2), or a table row (row + 3), or none (-1: written 0)
    int64_t src[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int cl = class_of(cw, c);
      src[c] = cl;
      if (cl == CLS_GENERAL) {
        src[c] = -1;
        const uint32_t slot = __ldg(pat.cell_slot + q + c);
        if (slot != kNoPattern) {
          const uint32_t idx = __ldg(pat.pidx + slot);
          if (idx != kNoPattern) src[c] = 3 + (int64_t)idx * NB * 28;
        }
      }
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const float *ku = b ? kuni1 : kuni0;
      KT *rec = (b ? rec1 : rec0) + rp.offset;
      // taps in groups of four: one 16-byte load per cell (uniform vectors: 32 floats per material;
      // table rows: 28 per block, both 16-byte aligned), then the four taps' stores
      for (int p0 = 0; p0 < 27; p0 += 4) {
        float4 g[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float *srcp = src[c] < 3 ? ku + src[c] * KREC + p0 : pat.pcoef + (src[c] - 3) + b * 28 + p0;
          g[c] = src[c] < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(reinterpret_cast<const float4 *>(srcp));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (p0 + u >= 27) break;
          float v[8];
#pragma unroll
          for (int c = 0; c < 8; ++c) v[c] = u == 0 ? g[c].x : (u == 1 ? g[c].y : (u == 2 ? g[c].z : g[c].w));
          st8(rec + (size_t)(p0 + u) * rp.stride, v);
        }
      }
    }
  }
}

// The coefficients of every general cell for NB blocks of one level at once
// (the pre- and post-block share the level's image and run words), written
// into the records of their runs.  Thread e of the grid-stride loop evaluates
// list[e]; the count of general cells is read on the device.
//
// With the pattern table (PatternArgs), k_fill_runs_pattern has already
// written the general cells whose pattern has table values; this kernel
// evaluates the others' patches (and returns at once when there are none).

template <typename KT, int NB>
__global__ void __launch_bounds__(PT)
k_kgen_list(const float *__restrict__ img, int n1, int n2, int n3, const float *__restrict__ params, int b0, int b1,
            const uint32_t *__restrict__ list, const uint32_t *__restrict__ glast_base,
            const uint32_t *__restrict__ glast_count, const uint32_t *__restrict__ rw,
            const uint32_t *__restrict__ rbase, const uint32_t *__restrict__ rcount, KT *__restrict__ rec0,
            KT *__restrict__ rec1, const PatternArgs pat) {
  dependent_launch_enter();
  if (pat.cell_slot && __ldg(pat.fail) == 0) return;  // k_fill_runs_pattern wrote every general cell
  __shared__ float4 sW[NB * kSW];
  __shared__ float4 sWm[NB * kSW];
  __shared__ float sb[NB * 28];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const float *W = params + (size_t)(b ? b1 : b0) * 2214;
    load_weights_smem(W, W + 2187, sW + b * kSW, sWm + b * kSW, sb + b * 28);
  }
  __syncthreads();
  const uint32_t G = __ldg(glast_base) + __ldg(glast_count);
  const FieldGeom g = FieldGeom::make(n1, n2, n3, 0);
  for (uint32_t e = blockIdx.x * PT + threadIdx.x; e < G; e += gridDim.x * PT) {
    const uint32_t q = __ldg(list + e);
    const int k = (int)(q % (uint32_t)n3);
    const uint32_t t = q / (uint32_t)n3;
    const int j = (int)(t % (uint32_t)n2), i = (int)(t / (uint32_t)n2);
    if (pat.cell_slot) {  // written by k_fill_runs when its pattern has table values
      const uint32_t slot = __ldg(pat.cell_slot + q);
      if (slot != kNoPattern && __ldg(pat.pidx + slot) != kNoPattern) continue;
    }
    float acc[NB][28];
    coeffs_of_patch_n<NB>(sW, sWm, sb, [&](int s, int m, int nn, int o) {
      return g.at(img + s * g.bstride, i + m - 1, j + nn - 1, k + o - 1);
    }, acc);
    const RecPos rp = rec_pos(rw, rbase, rcount, q, i, j, k, n2, n3);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      KT *r = (b ? rec1 : rec0) + rp.offset;
#pragma unroll
      for (int p = 0; p < 27; ++p) stf(r + p * rp.stride, acc[b][p]);
    }
  }
}

// The transposed block's coefficients at its general cells, gathered from
// the forward block of the same weights: B^T at cell q has, for tap p, the
// forward coefficient 26 - p of the neighbour r = q + offset(p) (its
// material's uniform value, or its record entry when r is general); 0 where
// r is outside the grid (the input is 0 there).  Written into q's record of
// the transposed block.  Thread e of the grid-stride loop takes list[e].
template <typename KT>
__global__ void __launch_bounds__(PT)
k_kgen_t_list(int n1, int n2, int n3, const uint32_t *__restrict__ list, const uint32_t *__restrict__ glast_base,
              const uint32_t *__restrict__ glast_count, const uint8_t *__restrict__ cls,
              const uint32_t *__restrict__ rw, const uint32_t *__restrict__ rbase, const uint32_t *__restrict__ rcount,
              const KT *__restrict__ rec, const float *__restrict__ kuni, const uint32_t *__restrict__ rwT,
              const uint32_t *__restrict__ rbaseT, const uint32_t *__restrict__ rcountT, KT *__restrict__ recT) {
  dependent_launch_enter();
  const uint32_t G = __ldg(glast_base) + __ldg(glast_count);
  for (uint32_t e = blockIdx.x * PT + threadIdx.x; e < G; e += gridDim.x * PT) {
    const uint32_t q = __ldg(list + e);
    const int k = (int)(q % (uint32_t)n3);
    const uint32_t t = q / (uint32_t)n3;
    const int j = (int)(t % (uint32_t)n2), i = (int)(t / (uint32_t)n2);
    const RecPos rt = rec_pos(rwT, rbaseT, rcountT, q, i, j, k, n2, n3);
#pragma unroll 3
    for (int p = 0; p < 27; ++p) {
      const int ii = i + tap_dx(p), jj = j + tap_dy(p), kk = k + tap_dz(p);
      float v = 0.f;
      if ((unsigned)ii < (unsigned)n1 && (unsigned)jj < (unsigned)n2 && (unsigned)kk < (unsigned)n3) {
        const uint32_t r = ((uint32_t)ii * (uint32_t)n2 + (uint32_t)jj) * (uint32_t)n3 + (uint32_t)kk;
        const int cl = __ldg(cls + r);
        if (cl != CLS_GENERAL) {
          v = __ldg(kuni + cl * KREC + 26 - p);
        } else {
          const RecPos rf = rec_pos(rw, rbase, rcount, r, ii, jj, kk, n2, n3);
          v = ldf(rec + rf.offset + (size_t)(26 - p) * rf.stride);
        }
      }
      stf(recT + rt.offset + (size_t)p * rt.stride, v);
    }
  }
}

// Dense planes of the transposed block: KT[p][q] = K[26 - p][q + offset(p)], 0 outside the grid.
template <typename KT>
__global__ void __launch_bounds__(256)
k_planes_transpose(const KT *__restrict__ K, KT *__restrict__ Kt, int64_t ps, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int64_t n = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2), i = (int)(t / n2);
#pragma unroll
  for (int p = 0; p < 27; ++p) {
    const int ii = i + tap_dx(p), jj = j + tap_dy(p), kk = k + tap_dz(p);
    float v = 0.f;
    if ((unsigned)ii < (unsigned)n1 && (unsigned)jj < (unsigned)n2 && (unsigned)kk < (unsigned)n3)
      v = ldf(K + (size_t)(26 - p) * ps + ((int64_t)ii * n2 + jj) * n3 + kk);
    stf(Kt + (size_t)p * ps + q, v);
  }
}

// c[e] = c[e]^2 (the SPD kind's c0^2, c1^2; sm_model_3d.py:421)
__global__ void k_square(float *__restrict__ c, int n) {
  dependent_launch_enter();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) c[e] = c[e] * c[e];
}

template <typename KT>
struct CoefArgs {
  const KT *K;             // dense: 27 planes ...
  int64_t ps;              // ... of this stride
  const KT *rec;           // classed: mixed-run records
  const KT *mrec;          // classed: a record for each material (its vector, each value 8 times)
  const float *kuni;       // classed: 3 x KREC uniform vectors
  const uint32_t *rw;      // classed: run words
  const uint32_t *rbase;   // classed: first record index per tile
  const uint32_t *rcount;  // classed: mixed runs per tile
};

// The material records of every block: block b, material m, coefficient p,
// cell c at mrec[((b * 3 + m) * 27 + p) * 8 + c] = kuni[b][m][p].
template <typename KT>
__global__ void __launch_bounds__(256) k_material_records(const float *__restrict__ kuni, KT *__restrict__ mrec) {
  dependent_launch_enter();
  const int b = blockIdx.x;
  for (int e = threadIdx.x; e < 3 * RREC; e += blockDim.x) {
    const int m = e / RREC, p = (e % RREC) / 8;
    stf(mrec + (size_t)b * 3 * RREC + e, kuni[((size_t)b * 3 + m) * KREC + p]);
  }
}

constexpr int KU = 33;  // row stride of the uniform vectors in shared memory (no bank conflicts)

// Shared memory of the classed path: the uniform vectors
struct ClsSmem {
  float Ku[3][KU];
};

// The thread's two runs (tx = 0, 1) against the staged tile, rows shared:
// plane pl = tx + dx of the tile serves run 0 as dx = pl and run 1 as
// dx = pl - 1, so each of the 12 input rows is read from shared memory once.
// Per cell the 27 taps are summed in the reference's order (dx, dy, dz).
// coef(tx, p, kv) yields the 8 coefficients of tap p for run tx.  OFF is the
// tile index of the run's z - 1 neighbour relative to 8 tz: 0 for the staged
// layout (interior from index 1), 3 for the TMA layout (interior from index 4;
// the row is then read as 16 values from 8 tz, all 16-byte aligned).
template <int OFF = 0, typename Coef>
__device__ __forceinline__ void apply_pair(const float (*S)[HY][HZP], int ty, int tz8, Coef coef, float acc[TX][8]) {
#pragma unroll
  for (int tx = 0; tx < TX; ++tx)
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[tx][c] = 0.f;
#pragma unroll
  for (int pl = 0; pl < TX + 2; ++pl)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      float xr[OFF ? 16 : 12];
      if constexpr (OFF != 0) ld_row16(&S[pl][ty + dy][tz8], xr);
      else ld_row12(&S[pl][ty + dy][tz8], xr);
#pragma unroll
      for (int tx = 0; tx < TX; ++tx) {
        const int dx = pl - tx;
        if (dx < 0 || dx > 2) continue;
#pragma unroll
        for (int dz = 0; dz < 3; ++dz) {
          float kv[8];
          coef(tx, dx * 9 + dy * 3 + dz, kv);
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[tx][c] = fmaf(kv[c], xr[c + dz + OFF], acc[tx][c]);
        }
      }
    }
}

// acc[tx][c] for the thread's two runs (tx = 0, 1).
// Dense: coefficient planes streamed from HBM.  Classed: a material run takes
// the material's uniform vector from shared memory, a mixed run streams its
// record like a dense run; warps with no mixed run skip the record path.
// rwd are the runs' words (load_run_words), trec the tile's first record and
// mixed-run count (load_tile_runs).
template <typename KT, bool CLS, int OFF = 0>
__device__ __forceinline__ void tile_apply(const float (*S)[HY][HZP], const ClsSmem *sm, const CoefArgs<KT> &C,
                                           const uint32_t rwd[TX], uint2 trec, const Tile &t, int n1, int n2,
                                           int n3, float acc[TX][8]) {
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int x0 = t.bz * TX, k0 = t.bx * TZ + tz * 8, j = t.by * TY + ty;
  const bool active = k0 < n3 && j < n2;
  bool valid[TX];
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) valid[tx] = active && x0 + tx < n1;
  if constexpr (!CLS) {
    int64_t q[TX];
#pragma unroll
    for (int tx = 0; tx < TX; ++tx) q[tx] = valid[tx] ? ((int64_t)(x0 + tx) * n2 + j) * n3 + k0 : 0;
    apply_pair<OFF>(S, ty, tz * 8, [&](int tx, int p, float kv[8]) {
      if (valid[tx]) ld8cs(C.K + p * C.ps + q[tx], kv);
      else {
#pragma unroll
        for (int c = 0; c < 8; ++c) kv[c] = 0.f;
      }
    }, acc);
    return;
  } else {
    bool mixed[TX];
#pragma unroll
    for (int tx = 0; tx < TX; ++tx) mixed[tx] = (rwd[tx] & 3u) == kMixed;
    if (!__any_sync(0xffffffffu, mixed[0] || mixed[1])) {
      const float *ku[TX];
#pragma unroll
      for (int tx = 0; tx < TX; ++tx) ku[tx] = sm->Ku[rwd[tx] & 3u];
      apply_pair<OFF>(S, ty, tz * 8, [&](int tx, int p, float kv[8]) {
        const float v = ku[tx][p];
#pragma unroll
        for (int c = 0; c < 8; ++c) kv[c] = v;
      }, acc);
    } else {
      // every lane streams a record: its run's, or its material's (cached), so
      // the loads carry no branch and issue ahead of the arithmetic
      const KT *rp[TX];
      uint32_t st[TX];
#pragma unroll
      for (int tx = 0; tx < TX; ++tx) {
        rp[tx] = mixed[tx] ? C.rec + (size_t)trec.x * RREC + (rwd[tx] >> 2) * 8 : C.mrec + (rwd[tx] & 3u) * RREC;
        st[tx] = mixed[tx] ? trec.y * 8 : 8;
      }
      apply_pair<OFF>(S, ty, tz * 8, [&](int tx, int p, float kv[8]) { ld8(rp[tx] + p * st[tx], kv); }, acc);
    }
  }
}

// tile_apply for the small levels (the grid fits in one wave, so registers do not limit the
// resident CTAs): each run's 27 coefficient vectors are loaded before any of them is used --
// one round of memory latency per run instead of one per group of taps -- and the runs are
// applied one after the other, each cell summing its taps in the same order with the same
// operands as tile_apply, so the results are identical.  BF16 coefficients (8 values per
// 16-byte load); warps without a mixed run take tile_apply's shared-memory path.
template <typename KT, bool CLS, int OFF = 0>
__device__ __forceinline__ void tile_apply_pref(const float (*S)[HY][HZP], const ClsSmem *sm, const CoefArgs<KT> &C,
                                                const uint32_t rwd[TX], uint2 trec, const Tile &t, int n1, int n2,
                                                int n3, float acc[TX][8]) {
  static_assert(sizeof(KT) == 2, "prefetched application: BF16 coefficients only");
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int x0 = t.bz * TX, k0 = t.bx * TZ + tz * 8, j = t.by * TY + ty;
  const bool active = k0 < n3 && j < n2;
  if constexpr (CLS) {
    const bool m0 = (rwd[0] & 3u) == kMixed, m1 = (rwd[1] & 3u) == kMixed;
    if (!__any_sync(0xffffffffu, m0 || m1)) {
      tile_apply<KT, CLS, OFF>(S, sm, C, rwd, trec, t, n1, n2, n3, acc);
      return;
    }
  }
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const bool valid = active && x0 + tx < n1;
    const KT *base;
    size_t st;
    bool load = true;
    if constexpr (CLS) {
      const bool mixed = (rwd[tx] & 3u) == kMixed;
      base = mixed ? C.rec + (size_t)trec.x * RREC + (rwd[tx] >> 2) * 8 : C.mrec + (rwd[tx] & 3u) * RREC;
      st = mixed ? (size_t)trec.y * 8 : 8;
    } else {
      base = C.K + (valid ? ((int64_t)(x0 + tx) * n2 + j) * n3 + k0 : 0);
      st = (size_t)C.ps;
      load = valid;
    }
    // all 27 loads issued before the first use (volatile: kept in this order, ahead of the FMAs)
    uint4 kr[27];
#pragma unroll
    for (int p = 0; p < 27; ++p) {
      kr[p] = make_uint4(0u, 0u, 0u, 0u);
      if (load)
        asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(kr[p].x), "=r"(kr[p].y), "=r"(kr[p].z), "=r"(kr[p].w)
                     : "l"(base + (size_t)p * st));
    }
    // keep every use after the last load: each vector passes through an (empty) volatile statement,
    // and those statements follow the loads in program order
#pragma unroll
    for (int p = 0; p < 27; ++p)
      asm volatile("" : "+r"(kr[p].x), "+r"(kr[p].y), "+r"(kr[p].z), "+r"(kr[p].w));
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[tx][c] = 0.f;
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
      for (int dy = 0; dy < 3; ++dy) {
        float xr[OFF ? 16 : 12];
        if constexpr (OFF != 0) ld_row16(&S[tx + dx][ty + dy][tz * 8], xr);
        else ld_row12(&S[tx + dx][ty + dy][tz * 8], xr);
#pragma unroll
        for (int dz = 0; dz < 3; ++dz) {
          const uint4 u = kr[dx * 9 + dy * 3 + dz];
          float kv[8];
          unpack_bf16x2(u.x, kv[0], kv[1]); unpack_bf16x2(u.y, kv[2], kv[3]);
          unpack_bf16x2(u.z, kv[4], kv[5]); unpack_bf16x2(u.w, kv[6], kv[7]);
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[tx][c] = fmaf(kv[c], xr[c + dz + OFF], acc[tx][c]);
        }
      }
  }
}

// uniform coefficient vectors of a classed block into shared memory
template <bool CLS>
__device__ __forceinline__ void stage_uniform(ClsSmem *sm, const float *__restrict__ kuni) {
  if constexpr (CLS) {
    for (int e = threadIdx.x; e < 3 * KREC; e += PT) sm->Ku[e / KREC][e % KREC] = __ldg(kuni + e);
  }
}

// the run words of the thread's runs and the tile's (first record, mixed runs) (classed only).
// The tile's mixed-run records are one contiguous block (tap-major across its runs); thread 0
// asks for the whole block to be brought into L2 with one bulk prefetch, so that the record
// loads of the block application, issued after the tile is staged, find it there.
template <typename KT, bool CLS>
__device__ __forceinline__ uint2 load_tile_runs(const CoefArgs<KT> &C, const Tile &t, int n1, int n2, int n3,
                                                uint32_t rwd[TX]) {
  if (!CLS) return make_uint2(0u, 0u);
  const uint2 tb = make_uint2(__ldg(C.rbase + t.id), __ldg(C.rcount + t.id));
  if (threadIdx.x == 0 && tb.y > 0) {
    // record block: RREC values per run, 16-byte aligned (RREC * sizeof(KT) is a multiple of 16)
    const size_t addr = __cvta_generic_to_global(C.rec + (size_t)tb.x * RREC);
    const uint32_t bytes = tb.y * (uint32_t)(RREC * sizeof(KT));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(addr), "r"(bytes) : "memory");
  }
  load_run_words(C.rw, t, n1, n2, n3, rwd);
  return tb;
}

// mask bytes of the thread's runs (all ones without a mask)
__device__ __forceinline__ void load_run_mask(const uint8_t *__restrict__ m, const Tile &t, int n1, int n2, int n3,
                                              uint2 mw[TX]) {
  const int k0 = t.bx * TZ + run_tz(threadIdx.x) * 8, j = t.by * TY + run_ty(threadIdx.x);
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = t.bz * TX + tx;
    mw[tx] = make_uint2(0xffffffffu, 0xffffffffu);
    if (m && k0 < n3 && j < n2 && i < n1) mw[tx] = __ldg(reinterpret_cast<const uint2 *>(m + ((int64_t)i * n2 + j) * n3 + k0));
  }
}
__device__ __forceinline__ void apply_run_mask(uint2 m, float acc[8]) {
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (!((c < 4 ? (m.x >> (8 * c)) : (m.y >> (8 * (c - 4)))) & 0xffu)) acc[c] = 0.f;
}

// ---------------------------------------------------------------------------
// pre-block (and the coarsest l-block): y = B(x), optional fused avg-pool
// ---------------------------------------------------------------------------
// Thread 0: initialise the tile's mbarrier (one arrival + the byte count) and have the
// tensor-memory accelerator copy the 4 x 18 x 76 FP32 box of the tile's input -- z from
// z0 - 4 (a multiple of 4 floats, 16 bytes), y from y0 - 1, x from x0 - 1, zero outside
// the grid -- into S (interior cell z0 + c at row index c + 4).
__device__ __forceinline__ void tma_tile_issue(float (*S)[HY][HZP], uint32_t bar, const CUtensorMap *tmap,
                                               const Tile &t) {
  if (threadIdx.x != 0) return;
  const int z0 = t.bx * TZ, y0 = t.by * TY, x0 = t.bz * TX;
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"((uint32_t)(HX * HY * HZP * sizeof(float))) : "memory");
  const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&S[0][0][0]);
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(z0 - 4), "r"(y0 - 1), "r"(x0 - 1), "r"(bar)
      : "memory");
}

// Shared state of a TMA-staged tile's wait: the copy's mbarrier, a second mbarrier that nothing
// ever arrives on (initialised for one arrival; the copy-stall test waits on it so that the bounded
// wait runs out while the real copy completes normally), and the CTA's copy-failed flag.
struct TileWait {
  uint64_t bar, never;
  int failed;
};

// Thread 0, before the __syncthreads that precedes tma_tile_wait: the second barrier and the flag.
__device__ __forceinline__ void tile_wait_init(TileWait &w) {
  if (threadIdx.x != 0) return;
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&w.never))
               : "memory");
  w.failed = 0;
}

__device__ __forceinline__ uint32_t mbar_poll(uint32_t bar, uint32_t limit) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < limit && !done; ++it)
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(bar) : "memory");
  return done;
}

// All threads, after a __syncthreads that follows tma_tile_issue and tile_wait_init: wait for the
// tile (phase 0) with a bounded poll (2^22 tries, about a second).  A thread whose poll runs out
// raises the CTA's flag and *err, then waits once more (bounded) so that a late copy lands before the
// CTA leaves; the CTA then agrees on the flag (one __syncthreads), so every thread returns the same
// verdict: true when the tile is in place.  err[1] != 0 (the copy-stall test knob) makes the first
// poll wait on the barrier that never completes, 256 tries, so the timeout path runs on an ordinary
// copy; the second poll then waits for the real copy as usual.
__device__ __forceinline__ bool tma_tile_wait(TileWait &w, int *err) {
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&w.bar);
  const bool stall = err[1] != 0;
  const uint32_t first = stall ? (uint32_t)__cvta_generic_to_shared(&w.never) : bar;
  if (!mbar_poll(first, stall ? 256u : (1u << 22))) {
    w.failed = 1;
    atomicExch(err, 1);
    mbar_poll(bar, 1u << 22);
  }
  __syncthreads();
  return !w.failed;
}

// Shared memory of the block bodies, one object per kernel whichever bodies it runs: the fine
// input tile, the classed path's uniform vectors, the tile copy's wait state and the post-block's
// coarse tile.  A kernel that runs several bodies one after the other (the coarse-level cluster
// kernel) reuses them, separating the bodies with barriers.
__device__ __forceinline__ float (*fine_tile_smem())[HY][HZP] {
  __shared__ __align__(128) float S[HX][HY][HZP];
  return S;
}
__device__ __forceinline__ ClsSmem *cls_smem() {
  __shared__ ClsSmem smc;
  return &smc;
}
__device__ __forceinline__ TileWait &tile_wait_smem() {
  __shared__ __align__(8) TileWait tw;
  return tw;
}
__device__ __forceinline__ float (*coarse_tile_smem())[CY][CZP] {
  __shared__ __align__(16) float Cs[CX][CY][CZP];
  return Cs;
}

// The body of the pre-block kernels.  Staged: every thread loads its share of
// the input tile (scaled by xscale) and stores it to shared memory.  TMA
// (XT = float): thread 0 has the tensor-memory accelerator copy the whole
// 4 x 18 x 76 box of the input (z from z0 - 4, outside the grid read as 0)
// into the tile, completing on an mbarrier; the scale is applied to the
// block's output instead (the block is linear in x).
template <typename KT, typename XT, typename YT, bool POOL, bool CLS, bool TMA, bool COH = false, bool PREF = false>
__device__ __forceinline__ void pre_fused_body(const CoefArgs<KT> &C, const XT *__restrict__ x,
                                               const float *__restrict__ xscale, YT *__restrict__ y,
                                               YT *__restrict__ ypool, const uint8_t *__restrict__ mask, int n1,
                                               int n2, int n3, const CUtensorMap *tmap, int *err, const Tile &t) {
  float(*S)[HY][HZP] = fine_tile_smem();
  ClsSmem *smc = CLS ? cls_smem() : nullptr;
  TileWait &tw = tile_wait_smem();
  const int z0 = t.bx * TZ, y0 = t.by * TY, x0 = t.bz * TX;
  const float sc = xscale ? __ldg(xscale) : 1.f;
  if constexpr (TMA) {
    tile_wait_init(tw);
    tma_tile_issue(S, (uint32_t)__cvta_generic_to_shared(&tw.bar), tmap, t);
  }
  uint32_t rwd[TX];
  uint2 mw[TX];
  const uint2 tb = load_tile_runs<KT, CLS>(C, t, n1, n2, n3, rwd);
  load_run_mask(mask, t, n1, n2, n3, mw);
  if constexpr (!TMA) {
    FineStage fs;
    stage_load(fs, t, n1, n2, n3,
               [&](int, int, int, int64_t q) {
                 const float4 v = ldv4c<COH>(x + q);
                 return make_float4(v.x * sc, v.y * sc, v.z * sc, v.w * sc);
               },
               [&](int, int, int, int64_t q) { return ldfc<COH>(x + q) * sc; });
    stage_put(S, fs);
  }
  stage_uniform<CLS>(smc, C.kuni);
  __syncthreads();  // also orders the mbarrier initialisation before the other threads' waits
  if constexpr (TMA) {
    if (!tma_tile_wait(tw, err)) return;
  }
  float acc[TX][8];
  if constexpr (PREF) tile_apply_pref<KT, CLS, TMA ? 3 : 0>(S, smc, C, rwd, tb, t, n1, n2, n3, acc);
  else tile_apply<KT, CLS, TMA ? 3 : 0>(S, smc, C, rwd, tb, t, n1, n2, n3, acc);
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int k0 = z0 + tz * 8, j = y0 + ty;
  const bool active = k0 < n3 && j < n2;  // n3 % 8 == 0: a run is all in or all out
  float pool[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = x0 + tx;
    if (!active || i >= n1) continue;
    const int64_t q = ((int64_t)i * n2 + j) * n3 + k0;
    if constexpr (TMA) {
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[tx][c] *= sc;
    }
    apply_run_mask(mw[tx], acc[tx]);
    if (y) st8(y + q, acc[tx]);  // y may be NULL when only the pooled output is wanted
    if (POOL) {
#pragma unroll
      for (int c = 0; c < 4; ++c) pool[c] += acc[tx][2 * c] + acc[tx][2 * c + 1];
    }
  }
  if (POOL) {
#pragma unroll
    for (int c = 0; c < 4; ++c) pool[c] += __shfl_xor_sync(0xffffffffu, pool[c], kTyPairLane);
    // (the cluster kernel also runs its coarsest block through this body, with no pooled output)
    if (active && (ty & 1) == 0 && (!COH || ypool)) {
      const int m2 = n2 / 2, m3 = n3 / 2;
      const int64_t qc = ((int64_t)(x0 / 2) * m2 + j / 2) * m3 + k0 / 2;
#pragma unroll
      for (int c = 0; c < 4; ++c) pool[c] *= 0.125f;
      st4(ypool + qc, pool);
    }
  }
}

// pre-block (and the coarsest l-block): y = B(x), optional fused avg-pool
template <typename KT, typename XT, typename YT, bool POOL, bool CLS>
__global__ void __launch_bounds__(PT)
k_pre_fused(const CoefArgs<KT> C, const XT *__restrict__ x,
            const float *__restrict__ xscale, YT *__restrict__ y, YT *__restrict__ ypool,
            const uint8_t *__restrict__ mask, int n1, int n2, int n3, const int *__restrict__ gate) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;  // batched solves: this system has stopped
  pre_fused_body<KT, XT, YT, POOL, CLS, false>(C, x, xscale, y, ypool, mask, n1, n2, n3, nullptr, nullptr,
                                              grid_tile());
}

// the small levels' pre-block: each run's coefficients loaded up front (tile_apply_pref); one
// CTA per SM is all such a grid needs, so the kernel may use the registers that takes
template <typename KT, typename XT, typename YT, bool POOL, bool CLS>
__global__ void __launch_bounds__(PT, 1)
k_pre_fused_small(const CoefArgs<KT> C, const XT *__restrict__ x, YT *__restrict__ y, YT *__restrict__ ypool,
                  int n1, int n2, int n3, const int *__restrict__ gate) {
  dependent_launch_enter();
  dependent_launch_trigger();
  if (gate && *gate != 0) return;
  pre_fused_body<KT, XT, YT, POOL, CLS, false, false, true>(C, x, nullptr, y, ypool, nullptr, n1, n2, n3, nullptr,
                                                            nullptr, grid_tile());
}

// the level-0 pre-block with its FP32 input tile loaded by TMA through tmap (x only for the
// pointer-free parts); err receives 1 if a tile copy did not complete
template <typename KT, typename YT, bool CLS>
__global__ void __launch_bounds__(PT)
k_pre_fused_tma(const CoefArgs<KT> C, const __grid_constant__ CUtensorMap tmap, const float *__restrict__ xscale,
                YT *__restrict__ y, YT *__restrict__ ypool, const uint8_t *__restrict__ mask, int n1, int n2, int n3,
                const int *__restrict__ gate, int *__restrict__ err) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;
  pre_fused_body<KT, float, YT, true, CLS, true>(C, nullptr, xscale, y, ypool, mask, n1, n2, n3, &tmap, err,
                                                grid_tile());
}

// ---------------------------------------------------------------------------
// post-block with fused trilinear prolongation and level combine
// ---------------------------------------------------------------------------
struct Lin1 { int i0, i1; float l0, l1; };
__device__ __forceinline__ Lin1 lin1(int f, int n) {
  float src = 0.5f * ((float)f + 0.5f) - 0.5f;
  if (src < 0.f) src = 0.f;
  Lin1 r;
  r.i0 = (int)src;
  r.i1 = r.i0 + (r.i0 < n - 1 ? 1 : 0);
  r.l1 = src - (float)r.i0;
  r.l0 = 1.f - r.l1;
  return r;
}

// trilinear prolongation at fine z index k from the staged coarse tile, the
// x / y weights (a, b) already relative to the tile
__device__ __forceinline__ float up_at(const float (*Cs)[CY][CZP], const Lin1 &a, const Lin1 &b, int k, int m3,
                                       int cz0) {
  const Lin1 c = lin1(k, m3);
  const int e0 = c.i0 - cz0, e1 = c.i1 - cz0;
  return a.l0 * (b.l0 * (c.l0 * Cs[a.i0][b.i0][e0] + c.l1 * Cs[a.i0][b.i0][e1]) +
                 b.l1 * (c.l0 * Cs[a.i0][b.i1][e0] + c.l1 * Cs[a.i0][b.i1][e1])) +
         a.l1 * (b.l0 * (c.l0 * Cs[a.i1][b.i0][e0] + c.l1 * Cs[a.i1][b.i0][e1]) +
                 b.l1 * (c.l0 * Cs[a.i1][b.i1][e0] + c.l1 * Cs[a.i1][b.i1][e1]));
}
__device__ __forceinline__ Lin1 lin1_rel(int f, int n, int base) {
  Lin1 r = lin1(f, n);
  r.i0 -= base;
  r.i1 -= base;
  return r;
}

constexpr int CNV = (TZ / 2) / 4;                 // coarse interior vectors per row
constexpr int kCoarseVec = (CX * CY * CNV + PT - 1) / PT;

// Stages the coarse tile of the CTA's fine tile (x_{l+1} with a one-cell
// halo; 0 outside the grid): every global load first, then the stores.
template <typename CT, bool COH = false>
__device__ __forceinline__ void stage_coarse(float (*Cs)[CY][CZP], const CT *__restrict__ xc, const Tile &t, int m1,
                                             int m2, int m3) {
  const int cx0 = t.bz * TX / 2 - 1, cy0 = t.by * TY / 2 - 1, cz0 = t.bx * TZ / 2 - 1;
  float4 cv[kCoarseVec];
  float ch = 0.f;
#pragma unroll
  for (int m = 0; m < kCoarseVec; ++m) {
    const int e = threadIdx.x + m * PT, r = e / CNV;
    const int i = cx0 + r / CY, j = cy0 + r % CY, k = cz0 + 1 + 4 * (e % CNV);
    cv[m] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e < CX * CY * CNV && (unsigned)i < (unsigned)m1 && (unsigned)j < (unsigned)m2 && k < m3)
      cv[m] = ldv4c<COH>(xc + ((int64_t)i * m2 + j) * m3 + k);
  }
  {
    const int e = threadIdx.x, r = e >> 1;
    const int i = cx0 + r / CY, j = cy0 + r % CY, k = (e & 1) ? cz0 + CZ - 1 : cz0;
    if (e < 2 * CX * CY && (unsigned)i < (unsigned)m1 && (unsigned)j < (unsigned)m2 && (unsigned)k < (unsigned)m3)
      ch = ldfc<COH>(xc + ((int64_t)i * m2 + j) * m3 + k);
  }
#pragma unroll
  for (int m = 0; m < kCoarseVec; ++m) {
    const int e = threadIdx.x + m * PT, r = e / CNV, v = e % CNV;
    if (e >= CX * CY * CNV) continue;
    float *row = &Cs[r / CY][r % CY][1 + 4 * v];
    row[0] = cv[m].x; row[1] = cv[m].y; row[2] = cv[m].z; row[3] = cv[m].w;
  }
  if (threadIdx.x < 2 * CX * CY) {
    const int r = threadIdx.x >> 1;
    Cs[r / CY][r % CY][(threadIdx.x & 1) ? CZ - 1 : 0] = ch;
  }
}

// The prolongation of a large level as its own bandwidth-bound pass: u =
// up(x_{l+1}) (with swap: c0 y_l + c1 up(x_{l+1})), one value per fine
// cell in the activation dtype, for the post-block kernel to stage like any
// input (its tile then needs no interpolation of the halo).  Same tile grid
// and run ownership as the block kernels.  up is the trilinear x2
// interpolation, or with NEAREST the SPD networks' nearest x2 / 8
// (F.interpolate(x, scale_factor=2) / 8, sm_model_3d.py:415).
template <typename CT, typename YT, typename UT, bool SWAP, bool NEAREST = false>
__global__ void __launch_bounds__(PT)
k_up_fine(const CT *__restrict__ xc, const YT *__restrict__ yl, const float *__restrict__ c0p,
          const float *__restrict__ c1p, UT *__restrict__ u, int n1, int n2, int n3, const int *__restrict__ gate) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;
  __shared__ __align__(16) float Cs[CX][CY][CZP];
  const int m1 = n1 / 2, m2 = n2 / 2, m3 = n3 / 2;
  const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TY, x0 = blockIdx.z * TX;
  const int cx0 = x0 / 2 - 1, cy0 = y0 / 2 - 1, cz0 = z0 / 2 - 1;
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int k0 = z0 + tz * 8, j = y0 + ty;
  const bool active = k0 < n3 && j < n2;
  float yv[TX][8];
  if (SWAP) {
#pragma unroll
    for (int tx = 0; tx < TX; ++tx)
      if (active && x0 + tx < n1) ld8(yl + ((int64_t)(x0 + tx) * n2 + j) * n3 + k0, yv[tx]);
  }
  stage_coarse(Cs, xc, grid_tile(), m1, m2, m3);
  __syncthreads();
  if (!active) return;
  const float c0 = SWAP ? __ldg(c0p) : 0.f, c1 = SWAP ? __ldg(c1p) : 0.f;
  if constexpr (NEAREST) {
    // fine cell (i, j, k0 + c) takes coarse cell (i/2, j/2, k0/2 + c/2): tile
    // indices (1, j/2 - cy0, k0/2 - cz0 + c/2)
    const float *row = &Cs[1][j / 2 - cy0][k0 / 2 - cz0];
#pragma unroll
    for (int tx = 0; tx < TX; ++tx) {
      const int i = x0 + tx;
      if (i >= n1) continue;
      float o[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        o[c] = row[c / 2] * 0.125f;
        if (SWAP) o[c] = __fadd_rn(__fmul_rn(c0, yv[tx][c]), __fmul_rn(c1, o[c]));
      }
      st8(u + ((int64_t)i * n2 + j) * n3 + k0, o);
    }
    return;
  }
  const Lin1 b = lin1_rel(j, m2, cy0);
  // The run's fine cells k0 .. k0 + 7 interpolate along z between the coarse
  // cells k0/2 - 1 .. k0/2 + 4 (tile z index 4 tz ..), with the weights of
  // lin1: (1/4, 3/4) for even k, (3/4, 1/4) for odd k; only the first cell
  // of the grid (clamped source) and the last (clamped upper neighbour)
  // differ, and take lin1's values.
  const Lin1 zf = lin1(k0, m3), zl = lin1(k0 + 7, m3);
  const bool first_lo = zf.i0 - (k0 / 2 - 1) == 1;  // k0 == 0: both taps one cell up
  const bool last_hi = zl.i1 == zl.i0;             // last cell of the grid: upper tap clamped
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = x0 + tx;
    if (i >= n1) continue;
    const Lin1 a = lin1_rel(i, m1, cx0);
    float R[2][2][6];
#pragma unroll
    for (int ia = 0; ia < 2; ++ia)
#pragma unroll
      for (int ib = 0; ib < 2; ++ib) {
        const float *row = &Cs[ia ? a.i1 : a.i0][ib ? b.i1 : b.i0][4 * tz];
        const float4 lo = *reinterpret_cast<const float4 *>(row);
        const float2 hi = *reinterpret_cast<const float2 *>(row + 4);
        R[ia][ib][0] = lo.x; R[ia][ib][1] = lo.y; R[ia][ib][2] = lo.z; R[ia][ib][3] = lo.w;
        R[ia][ib][4] = hi.x; R[ia][ib][5] = hi.y;
      }
    float o[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float l0 = (c & 1) ? 0.75f : 0.25f, l1 = (c & 1) ? 0.25f : 0.75f;
      if (c == 0) { l0 = zf.l0; l1 = zf.l1; }
      if (c == 7) { l0 = zl.l0; l1 = zl.l1; }
      const int r0 = (c & 1) ? c / 2 + 1 : c / 2, r1 = r0 + 1;
      float v[2][2][2];
#pragma unroll
      for (int ia = 0; ia < 2; ++ia)
#pragma unroll
        for (int ib = 0; ib < 2; ++ib) {
          float x0v = R[ia][ib][r0], x1v = R[ia][ib][r1];
          if (c == 0 && first_lo) { x0v = R[ia][ib][1]; x1v = R[ia][ib][2]; }
          if (c == 7 && last_hi) x1v = R[ia][ib][4];
          v[ia][ib][0] = x0v;
          v[ia][ib][1] = x1v;
        }
      o[c] = a.l0 * (b.l0 * (l0 * v[0][0][0] + l1 * v[0][0][1]) + b.l1 * (l0 * v[0][1][0] + l1 * v[0][1][1])) +
             a.l1 * (b.l0 * (l0 * v[1][0][0] + l1 * v[1][0][1]) + b.l1 * (l0 * v[1][1][0] + l1 * v[1][1][1]));
      if (SWAP) o[c] = __fadd_rn(__fmul_rn(c0, yv[tx][c]), __fmul_rn(c1, o[c]));
    }
    st8(u + ((int64_t)i * n2 + j) * n3 + k0, o);
  }
}

// The tile's share of the npsd products (ZDots): each thread's FP32 sums of its cells, added in
// FP64 across the CTA in a fixed order; thread 0 stores the tile's two values.
__device__ __forceinline__ void zdots_tile_store(float s0, float s1, const ZDots &zd, unsigned tile) {
  __shared__ double red[2][PT / 32];
  double v0 = s0, v1 = s1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = v0;
    red[1][threadIdx.x >> 5] = v1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int w = 0; w < PT / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    zd.partial[2 * (size_t)tile] = a;
    zd.partial[2 * (size_t)tile + 1] = b;
  }
}

// UPIN: xc is the level's prolongated input u of k_up_fine (already combined
// with y_l under swap), staged like a pre-block input.
// TMA (UPIN, CT = float): the FP32 input u arrives by the tensor-memory accelerator as in the
// level-0 pre-block (tma_tile_issue / tma_tile_wait).
// ZD (OT = float): the npsd products of the output with the solver's directions (ZDots) as an
// epilogue, while the output is still in registers.
template <typename KT, typename CT, typename YT, typename OT, bool SWAP, bool CLS, bool UPIN, bool TMA,
          bool COH = false, bool PREF = false, bool ZD = false>
__device__ __forceinline__ void post_fused_body(const CoefArgs<KT> &C, const CT *__restrict__ xc,
                                                const YT *__restrict__ yl, const float *__restrict__ c0p,
                                                const float *__restrict__ c1p, OT *__restrict__ out,
                                                const uint8_t *__restrict__ bmask,
                                                const uint8_t *__restrict__ omask, int n1, int n2, int n3,
                                                const CUtensorMap *tmap, int *err, const Tile &t,
                                                const ZDots *zd = nullptr) {
  static_assert(!TMA || UPIN, "TMA staging needs the prolongated input");
  float(*S)[HY][HZP] = fine_tile_smem();
  TileWait &tw = tile_wait_smem();
  if constexpr (TMA) {
    tile_wait_init(tw);
    tma_tile_issue(S, (uint32_t)__cvta_generic_to_shared(&tw.bar), tmap, t);
  }
  float(*Cs)[CY][CZP] = nullptr;
  if constexpr (!UPIN) Cs = coarse_tile_smem();
  ClsSmem *smc = CLS ? cls_smem() : nullptr;
  stage_uniform<CLS>(smc, C.kuni);
  const int z0 = t.bx * TZ, y0 = t.by * TY, x0 = t.bz * TX;
  const int m1 = n1 / 2, m2 = n2 / 2, m3 = n3 / 2;
  const int cx0 = x0 / 2 - 1, cy0 = y0 / 2 - 1, cz0 = z0 / 2 - 1;
  const float c0 = __ldg(c0p), c1 = __ldg(c1p);
  uint32_t rwd[TX];
  uint2 bw[TX], ow[TX];
  const uint2 tb = load_tile_runs<KT, CLS>(C, t, n1, n2, n3, rwd);
  load_run_mask(bmask, t, n1, n2, n3, bw);
  load_run_mask(omask, t, n1, n2, n3, ow);
  // ZD: products wanted (0, 1 or 2, the same for the whole CTA) and their vectors, whose segments
  // of the thread's runs are asked into L2 now so that the epilogue's loads find them there
  int nd = 0;
  const float *a1 = nullptr, *a0 = nullptr;
  if constexpr (ZD) {
    const int it = __ldg(zd->it), h = zd->single ? 0 : __ldg(zd->head);
    nd = zd->single ? 1 : (it < 2 ? it : 2);
    a1 = zd->ring + (size_t)h * zd->n;
    a0 = zd->ring + (size_t)((h + 2) % 3) * zd->n;
    const int pk = z0 + run_tz(threadIdx.x) * 8, pj = y0 + run_ty(threadIdx.x);
    if (nd > 0 && pk < n3 && pj < n2) {
#pragma unroll
      for (int tx = 0; tx < TX; ++tx) {
        if (x0 + tx >= n1) continue;
        const int64_t q = ((int64_t)(x0 + tx) * n2 + pj) * n3 + pk;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a1 + q));
        if (nd == 2) asm volatile("prefetch.global.L2 [%0];" ::"l"(a0 + q));
      }
    }
  }
  if (UPIN) {
    if constexpr (!TMA) {
      FineStage fs;
      stage_load(fs, t, n1, n2, n3, [&](int, int, int, int64_t q) { return ldv4c<COH>(xc + q); },
                 [&](int, int, int, int64_t q) { return ldfc<COH>(xc + q); });
      stage_put(S, fs);
    }
  } else {
    if (SWAP) {  // y_l goes straight into the fine tile; the combine below reads it back in place
      FineStage fs;
      stage_load(fs, t, n1, n2, n3, [&](int, int, int, int64_t q) { return ldv4c<COH>(yl + q); },
                 [&](int, int, int, int64_t q) { return ldfc<COH>(yl + q); });
      stage_put(S, fs);
    }
    stage_coarse<CT, COH>(Cs, xc, t, m1, m2, m3);
    __syncthreads();
    // the fine tile: up(x_{l+1}) (with swap: c0 y_l + c1 up(x_{l+1})); 0 outside the grid
    const int v = threadIdx.x % NVR;
#pragma unroll
    for (int m = 0; m < kStageVec; ++m) {
      const int r = stage_vec_row(m), i = x0 + r / HY - 1, j = y0 + r % HY - 1, k = z0 + 4 * v;
      float o[4] = {0.f, 0.f, 0.f, 0.f};
      float *row = &S[r / HY][r % HY][4 * v + 1];
      if ((unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && k < n3) {
        const Lin1 a = lin1_rel(i, m1, cx0), b = lin1_rel(j, m2, cy0);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          o[c] = up_at(Cs, a, b, k + c, m3, cz0);
          if (SWAP) o[c] = __fadd_rn(__fmul_rn(c0, row[c]), __fmul_rn(c1, o[c]));
        }
      }
      row[0] = o[0];
      *reinterpret_cast<float2 *>(row + 1) = make_float2(o[1], o[2]);
      row[3] = o[3];
    }
#pragma unroll
    for (int m = 0; m < kStageHalo; ++m) {
      const int e = stage_halo_id(m), r = e >> 1;
      if (e >= 2 * HX * HY) continue;
      const int i = x0 + r / HY - 1, j = y0 + r % HY - 1, k = (e & 1) ? z0 + TZ : z0 - 1;
      float o = 0.f;
      if ((unsigned)i < (unsigned)n1 && (unsigned)j < (unsigned)n2 && (unsigned)k < (unsigned)n3) {
        o = up_at(Cs, lin1_rel(i, m1, cx0), lin1_rel(j, m2, cy0), k, m3, cz0);
        if (SWAP) o = __fadd_rn(__fmul_rn(c0, S[r / HY][r % HY][(e & 1) ? HZ - 1 : 0]), __fmul_rn(c1, o));
      }
      S[r / HY][r % HY][(e & 1) ? HZ - 1 : 0] = o;
    }
  }
  __syncthreads();
  if constexpr (TMA) {
    if (!tma_tile_wait(tw, err)) return;
  }
  float accs[TX][8];
  if constexpr (PREF) tile_apply_pref<KT, CLS, TMA ? 3 : 0>(S, smc, C, rwd, tb, t, n1, n2, n3, accs);
  else tile_apply<KT, CLS, TMA ? 3 : 0>(S, smc, C, rwd, tb, t, n1, n2, n3, accs);
  const int tz = run_tz(threadIdx.x), ty = run_ty(threadIdx.x);
  const int k0 = z0 + tz * 8, j = y0 + ty;
  const bool active = k0 < n3 && j < n2;
  float s1 = 0.f, s0 = 0.f;
#pragma unroll
  for (int tx = 0; tx < TX; ++tx) {
    const int i = x0 + tx;
    if (!active || i >= n1) continue;
    const int64_t q = ((int64_t)i * n2 + j) * n3 + k0;
    float *acc = accs[tx];
    apply_run_mask(bw[tx], acc);
    if (!SWAP) {
      float yv[8];
      ld8c<COH>(yl + q, yv);
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = __fadd_rn(__fmul_rn(c0, yv[c]), __fmul_rn(c1, acc[c]));
    }
    apply_run_mask(ow[tx], acc);
    st8(out + q, acc);
    if constexpr (ZD) {
      if (nd >= 1) {
        float a[8];
        ld8(a1 + q, a);
#pragma unroll
        for (int c = 0; c < 8; ++c) s1 = fmaf(acc[c], a[c], s1);
      }
      if (nd == 2) {
        float a[8];
        ld8(a0 + q, a);
#pragma unroll
        for (int c = 0; c < 8; ++c) s0 = fmaf(acc[c], a[c], s0);
      }
    }
  }
  if constexpr (ZD) {
    if (nd > 0) zdots_tile_store(s1, s0, *zd, t.id);
  }
}

template <typename KT, typename CT, typename YT, typename OT, bool SWAP, bool CLS, bool UPIN>
__global__ void __launch_bounds__(PT)
k_post_fused(const CoefArgs<KT> C, const CT *__restrict__ xc, const YT *__restrict__ yl,
             const float *__restrict__ c0p, const float *__restrict__ c1p, OT *__restrict__ out,
             const uint8_t *__restrict__ bmask, const uint8_t *__restrict__ omask, int n1, int n2, int n3,
             const int *__restrict__ gate) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;
  post_fused_body<KT, CT, YT, OT, SWAP, CLS, UPIN, false>(C, xc, yl, c0p, c1p, out, bmask, omask, n1, n2, n3,
                                                          nullptr, nullptr, grid_tile());
}

// the small levels' post-block (fused prolongation and combine), coefficients loaded up front
template <typename KT, typename AT, bool SWAP, bool CLS>
__global__ void __launch_bounds__(PT, 1)
k_post_fused_small(const CoefArgs<KT> C, const AT *__restrict__ xc, const AT *__restrict__ yl,
                   const float *__restrict__ c0p, const float *__restrict__ c1p, AT *__restrict__ out, int n1,
                   int n2, int n3, const int *__restrict__ gate) {
  dependent_launch_enter();
  dependent_launch_trigger();
  if (gate && *gate != 0) return;
  post_fused_body<KT, AT, AT, AT, SWAP, CLS, false, false, false, true>(C, xc, yl, c0p, c1p, out, nullptr, nullptr,
                                                                        n1, n2, n3, nullptr, nullptr, grid_tile());
}

// the post-block on an FP32 prolongated input u loaded by TMA through tmap; ZD: with the npsd
// products of the output (zd)
template <typename KT, typename YT, typename OT, bool SWAP, bool CLS, bool ZD = false>
__global__ void __launch_bounds__(PT)
k_post_fused_tma(const CoefArgs<KT> C, const __grid_constant__ CUtensorMap tmap, const YT *__restrict__ yl,
                 const float *__restrict__ c0p, const float *__restrict__ c1p, OT *__restrict__ out,
                 const uint8_t *__restrict__ bmask, const uint8_t *__restrict__ omask, int n1, int n2, int n3,
                 const int *__restrict__ gate, int *__restrict__ err, const ZDots zd) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;
  post_fused_body<KT, float, YT, OT, SWAP, CLS, true, true, false, false, ZD>(
      C, nullptr, yl, c0p, c1p, out, bmask, omask, n1, n2, n3, &tmap, err, grid_tile(), &zd);
}

// ---------------------------------------------------------------------------
// The coarse levels of one application in one launch: one thread-block
// cluster (16 CTAs, or 8 where 16 are not available) runs the pre-blocks of
// levels lc .. L-1, the coarsest block and the post-blocks of levels L-1 .. lc
// (sm_model_3d.py:204-260 from level lc on) as stages separated by cluster
// barriers.  In a stage, CTA r takes the level's tiles r, r + 16, ... through
// the same bodies as the per-level kernels, so every value is computed by the
// same arithmetic; activations written by one stage are read by the next
// through L2 (the bodies' COH loads).  These levels hold at most a few tens
// of tiles each, so as separate kernels they cost a launch and one CTA's
// load -> compute chain apiece; here the chains follow each other inside one
// launch.  Only the SmallSMModelDn3D kind (SM) uses it.
// ---------------------------------------------------------------------------
constexpr int kCoarseMaxLev = 6;
template <typename KT, typename AT>
struct CoarseArgs {
  int nlev;                              // levels lc .. L (index i: level lc + i)
  int n1[kCoarseMaxLev], n2[kCoarseMaxLev], n3[kCoarseMaxLev];
  int tz[kCoarseMaxLev], ty[kCoarseMaxLev];  // tiles along z and y
  unsigned ntiles[kCoarseMaxLev];
  CoefArgs<KT> pre[kCoarseMaxLev];       // pre-blocks; pre[nlev - 1]: the coarsest block
  CoefArgs<KT> post[kCoarseMaxLev];      // post-blocks of levels lc .. L-1
  AT *x[kCoarseMaxLev];                  // pre-block inputs; x[0] written by the previous kernel
  AT *y[kCoarseMaxLev];                  // pre-block outputs
  AT *xo[kCoarseMaxLev];                 // post-block outputs; xo[nlev - 1]: the coarsest block's
  const float *c0[kCoarseMaxLev], *c1[kCoarseMaxLev];
};

__device__ __forceinline__ Tile tile_of(unsigned id, int tz, int ty) {
  return Tile{(int)(id % (unsigned)tz), (int)((id / (unsigned)tz) % (unsigned)ty), (int)(id / (unsigned)(tz * ty)),
              id};
}

// all threads of the cluster: the stage's global writes become visible to the next stage's reads
// (release / acquire at cluster scope; the next stage reads them through L2)
__device__ __forceinline__ void cluster_stage_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// one tile's mixed-run record block into L2 (classed levels)
template <typename KT>
__device__ __forceinline__ void prefetch_tile_records(const CoefArgs<KT> &C, unsigned tile) {
  const uint32_t base = __ldg(C.rbase + tile), cnt = __ldg(C.rcount + tile);
  if (cnt == 0) return;
  const size_t addr = __cvta_generic_to_global(C.rec + (size_t)base * RREC);
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(addr), "r"(cnt * (uint32_t)(RREC * sizeof(KT)))
               : "memory");
}

template <typename KT, typename AT, bool CLS, bool SWAP>
__global__ void __launch_bounds__(PT)
k_coarse_cluster(const __grid_constant__ CoarseArgs<KT, AT> A, const int *__restrict__ gate) {
  dependent_launch_enter();
  if (gate && *gate != 0) return;  // read alike by every CTA: the whole cluster leaves
  const unsigned r = blockIdx.x, nc = gridDim.x;
  if constexpr (CLS) {
    // the record blocks of every tile this CTA takes in any stage, asked into L2 up front (one
    // thread per block), so that the later stages' coefficient loads find them there
    int item = 0;
    for (int i = 0; i < A.nlev; ++i)
      for (unsigned id = r; id < A.ntiles[i]; id += nc) {
        if (item++ == (int)threadIdx.x) prefetch_tile_records(A.pre[i], id);
        if (i < A.nlev - 1 && item++ == (int)threadIdx.x) prefetch_tile_records(A.post[i], id);
      }
  }
  for (int i = 0; i < A.nlev; ++i) {
    const bool last = i == A.nlev - 1;
    for (unsigned id = r; id < A.ntiles[i]; id += nc) {
      pre_fused_body<KT, AT, AT, true, CLS, false, true>(A.pre[i], A.x[i], nullptr, last ? A.xo[i] : A.y[i],
                                                        last ? nullptr : A.x[i + 1], nullptr, A.n1[i], A.n2[i],
                                                        A.n3[i], nullptr, nullptr, tile_of(id, A.tz[i], A.ty[i]));
      __syncthreads();  // the next tile restages the shared tile
    }
    cluster_stage_barrier();
  }
  for (int i = A.nlev - 2; i >= 0; --i) {
    for (unsigned id = r; id < A.ntiles[i]; id += nc) {
      post_fused_body<KT, AT, AT, AT, SWAP, CLS, false, false, true>(
          A.post[i], A.xo[i + 1], A.y[i], A.c0[i], A.c1[i], A.xo[i], nullptr, nullptr, A.n1[i], A.n2[i], A.n3[i],
          nullptr, nullptr, tile_of(id, A.tz[i], A.ty[i]));
      __syncthreads();
    }
    if (i > 0) cluster_stage_barrier();
  }
}

// ---------------------------------------------------------------------------
// small helpers for the general (ragged-size) path and the plan setup
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_scale_copy(const float *__restrict__ x, const float *__restrict__ s, T *__restrict__ y, int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  stf(y + q, x[q] * (s ? s[0] : 1.f));
}

template <typename T>
__global__ void k_apply_mask(T *__restrict__ y, const uint8_t *__restrict__ m, int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (!m[q]) stf(y + q, 0.f);
}

template <typename TI, typename TO>
__global__ void k_convert(const TI *__restrict__ x, TO *__restrict__ y, int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  stf(y + q, ldf(x + q));
}

__global__ void k_fluid_mask(const float *__restrict__ img, uint8_t *__restrict__ m, int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  m[q] = img[n + q] != 0.f;  // channel 1 = fluid (the reference masks with image[1] == 0)
}
// the same, 16 cells per thread (n a multiple of 16: 16-byte loads of channel 1, one 16-byte store)
__global__ void k_fluid_mask16(const float *__restrict__ img, uint8_t *__restrict__ m, int64_t n) {
  dependent_launch_enter();
  const int64_t q = 16 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (q >= n) return;
  const float4 *f = reinterpret_cast<const float4 *>(img + n + q);
  uint32_t w[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float4 v = __ldg(f + u);
    w[u] = (v.x != 0.f ? 1u : 0u) | (v.y != 0.f ? 1u << 8 : 0u) | (v.z != 0.f ? 1u << 16 : 0u) |
           (v.w != 0.f ? 1u << 24 : 0u);
  }
  *reinterpret_cast<uint4 *>(m + q) = make_uint4(w[0], w[1], w[2], w[3]);
}

// ---------------------------------------------------------------------------
// the plan object (host side; all device memory is the caller's workspace)
// ---------------------------------------------------------------------------
int launch_stencil_gen(const float *, int, int, int, int, const float *, const float *, void *, int,
                       int64_t, cudaStream_t);
int launch_stencil_apply(const void *, int, int64_t, const void *, int, int, void *, int, int, int,
                         int, int, int, cudaStream_t);
int launch_avg_pool2(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_avg_pool2_adjoint(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_upsample2(const void *, void *, int, int, int, int, int, cudaStream_t);
int launch_axpby(const float *, const void *, const float *, const void *, void *, int, int64_t,
                 cudaStream_t);
int launch_linear_forward(const float *, int, int, int, const float *, const float *, int, float *,
                          float *, void *, size_t, cudaStream_t);
int launch_linear_forward_strided(const float *, int, int, int, const float *, int64_t, const float *, int64_t, int,
                                  float *, int64_t, float *, void *, size_t, cudaStream_t);
size_t linear_workspace();

struct PrecondPlan {
  int n1, n2, n3, L;          // fine sizes, number of levels n (blocks at levels 0..L)
  int kdt, adt;               // coefficient / activation storage dtypes
  int swap, mask;
  int kind;                   // MLPCG_PRECOND_SM, MLPCG_PRECOND_SMALL_SPD or MLPCG_PRECOND_SPD
  int layout;                 // MLPCG_COEFF_DENSE or MLPCG_COEFF_CLASSED
  struct Level { int n1, n2, n3; int64_t n, ps; bool fast, cls; unsigned ntiles; };
  std::vector<Level> lv;      // L + 1 levels
  // device pointers (inside the caller's workspace)
  std::vector<float *> img;   // level images, [0] unused (caller's image)
  float *Uall = nullptr;      // uniform vectors of all blocks
  void *Mrec = nullptr;       // material records of all blocks (block order of Uall)
  void *ufine = nullptr;      // level-0 prolongated post-block input
  uint32_t *glist = nullptr;  // general-cell list (setup scratch)
  uint32_t *rlist = nullptr;  // mixed-run list (setup scratch)
  // SmallSMModelDn3D kind: each classed level >= 1 builds its coefficients on a stream of its own,
  // with its own general-cell and mixed-run lists; each level's c0 / c1 pass its own workspace
  std::vector<uint32_t *> glists, rlists;
  std::vector<void *> lin_wss;
  // level-0 pattern table (classed level 0): hash keys, table index per slot, entries used,
  // coefficients per entry (2 blocks), pattern slot per general cell
  unsigned long long *pkeys = nullptr;
  uint32_t *pidx = nullptr, *pcount = nullptr, *cell_slot = nullptr;  // cell_slot: per level-0 cell
  float *pcoef = nullptr;
  // setup streams (SmallSMModelDn3D kind): level 0's coefficient chain runs on the caller's
  // stream; sides[0] builds the image pyramid (recording img_ev[l] as level l's image is ready)
  // and the coarse levels' c0 / c1; sides[l] (1 <= l <= L) level l's coefficients, then (l < L)
  // its c0 / c1; sides[L + 1] level 0's c0 / c1.  Forked with fork_ev, joined with join_evs.
  std::vector<cudaStream_t> sides;
  cudaEvent_t fork_ev = nullptr;
  std::vector<cudaEvent_t> img_ev, join_evs;
  std::vector<void *> Kpre, Kpost;   // dense planes, or mixed-run records on classed levels
  void *Kl = nullptr;
  std::vector<float *> Upre, Upost;  // classed levels: 3 x KREC uniform vectors per block
  float *Ul = nullptr;
  std::vector<uint8_t *> cls;        // classed levels: class byte per cell (setup)
  std::vector<uint32_t *> rw;        // classed levels: word per 8-cell run
  std::vector<uint32_t *> rcount, rbase, gcount, gbase;  // per tile: mixed runs, general cells
  // SPD kinds: the transposed blocks (l0_t, l1_t, coarsest l_t) have their own class map,
  // run words and per-tile counts per level (a cell is uniform when its 27 neighbours are)
  std::vector<uint8_t *> clsT;
  std::vector<uint32_t *> rwT, rcountT, rbaseT, gcountT, gbaseT;
  void *Klt = nullptr;        // coarsest transposed block
  float *Ult = nullptr;
  void *xtmp = nullptr;       // coarsest-level temporary between l and l_t (SMALL_SPD kind)
  // SPD kind (SPDSMModelDn3D): Kpre = l0, Kpost = l1 (forward); KpreT = l0_t, KpostT = l1_t
  std::vector<void *> KpreT, KpostT;
  std::vector<float *> UpreT, UpostT;
  void *v0 = nullptr;         // V's output on the finest level, the input of V^T
  std::vector<void *> y, xin, xout;  // y_l (pre out), x_l inputs (l >= 1), post outputs (l >= 1)
  float *coef = nullptr;      // c0[0..L-1], c1[0..L-1]
  uint8_t *fmask = nullptr;   // fluid mask of level 0
  void *lin_ws = nullptr;
  float *scratch = nullptr;   // 81 floats (linear means)
  int *err = nullptr;         // set to 1 by a level-0 TMA tile copy that did not complete
  bool coarse_cluster = false; // SM kind: the coarse levels in one cluster launch (off: slower, see notes)
  int small_tiles_per_sm = 2;  // a level with at most this many tiles per SM runs the prefetching kernels
  size_t bytes = 0;
  bool ready = false;
};

static size_t al256(size_t b) { return (b + 255) / 256 * 256; }

// multiprocessors of the current device (grid sizing of persistent kernels)
static int sm_count() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
    return 152;
  return v;
}

// CTAs of PT threads of kernel f resident per SM (at least 1)
template <typename F>
static int resident_ctas(F f) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, PT, 0) != cudaSuccess || nb < 1) return 1;
  return nb;
}
template <typename KT>
static KT *kgen_rec_type(void (*)(const float *, int, int, int, const float *, int, int, const uint32_t *,
                                  const uint32_t *, const uint32_t *, const uint32_t *, const uint32_t *,
                                  const uint32_t *, KT *, KT *, const PatternArgs));

// blocks with uniform vectors / material records: 2L + 1 forward, plus l_t (SMALL_SPD kind) or
// the 2L + 1 transposes (SPD kind)
static int uniform_blocks(const PrecondPlan &P) {
  if (P.kind == MLPCG_PRECOND_SMALL_SPD) return 2 * P.L + 2;
  if (P.kind == MLPCG_PRECOND_SPD) return 4 * P.L + 2;
  return 2 * P.L + 1;
}
static bool has_transposes(const PrecondPlan &P) { return P.kind != MLPCG_PRECOND_SM; }

static size_t plan_layout(PrecondPlan &P, char *base) {
  size_t off = 0;
  auto take = [&](size_t b) -> void * {
    void *p = base ? base + off : nullptr;
    off += al256(b);
    return p;
  };
  const size_t sk = dtype_size(P.kdt), sa = dtype_size(P.adt);
  P.img.assign(P.L + 1, nullptr);
  P.Kpre.assign(P.L, nullptr);
  P.Kpost.assign(P.L, nullptr);
  P.y.assign(P.L, nullptr);
  P.xin.assign(P.L + 1, nullptr);
  P.xout.assign(P.L + 1, nullptr);
  for (int l = 1; l <= P.L; ++l) P.img[l] = (float *)take(3 * P.lv[l].n * sizeof(float));
  // coefficient storage of one block: dense planes, or (worst case: every run mixed) run records
  auto kbytes = [&](int l) {
    const auto &v = P.lv[l];
    return v.cls ? (size_t)(v.n / 8) * RREC * sk : (size_t)27 * v.ps * sk;
  };
  for (int l = 0; l < P.L; ++l) {
    P.Kpre[l] = take(kbytes(l));
    P.Kpost[l] = take(kbytes(l));
  }
  P.Kl = take(kbytes(P.L));
  const bool spd = has_transposes(P), full = P.kind == MLPCG_PRECOND_SPD;
  P.Klt = spd ? take(kbytes(P.L)) : nullptr;
  P.KpreT.assign(P.L, nullptr);
  P.KpostT.assign(P.L, nullptr);
  for (int l = 0; full && l < P.L; ++l) {
    P.KpreT[l] = take(kbytes(l));
    P.KpostT[l] = take(kbytes(l));
  }
  P.Upre.assign(P.L, nullptr);
  P.Upost.assign(P.L, nullptr);
  P.cls.assign(P.L + 1, nullptr);
  P.rw.assign(P.L + 1, nullptr);
  P.rcount.assign(P.L + 1, nullptr);
  P.rbase.assign(P.L + 1, nullptr);
  P.gcount.assign(P.L + 1, nullptr);
  P.gbase.assign(P.L + 1, nullptr);
  // uniform vectors of all blocks (block b at U + 3 KREC b): pre[0..L-1], post[0..L-1], l
  // (the parameter block order), and for the SPD kind l_t after l
  const int nU = uniform_blocks(P);
  float *U = (float *)take((size_t)nU * 3 * KREC * sizeof(float));
  for (int l = 0; l < P.L; ++l) {
    P.Upre[l] = U + (size_t)l * 3 * KREC;
    P.Upost[l] = U + (size_t)(P.L + l) * 3 * KREC;
  }
  P.Ul = U + (size_t)2 * P.L * 3 * KREC;
  P.Ult = spd ? U + (size_t)(full ? 4 * P.L + 1 : 2 * P.L + 1) * 3 * KREC : nullptr;
  P.UpreT.assign(P.L, nullptr);
  P.UpostT.assign(P.L, nullptr);
  for (int l = 0; full && l < P.L; ++l) {
    P.UpreT[l] = U + (size_t)(2 * P.L + 1 + l) * 3 * KREC;
    P.UpostT[l] = U + (size_t)(3 * P.L + 1 + l) * 3 * KREC;
  }
  P.Uall = U;
  P.Mrec = take((size_t)nU * 3 * RREC * sk);
  int64_t nlist = 0;
  for (int l = 0; l <= P.L; ++l) {
    const auto &v = P.lv[l];
    if (!v.cls) continue;
    P.cls[l] = (uint8_t *)take(v.ps);
    P.rw[l] = (uint32_t *)take((v.n / 8) * sizeof(uint32_t));
    P.rcount[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.rbase[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.gcount[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.gbase[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    nlist = std::max<int64_t>(nlist, v.n);
  }
  P.clsT.assign(P.L + 1, nullptr);
  P.rwT.assign(P.L + 1, nullptr);
  P.rcountT.assign(P.L + 1, nullptr);
  P.rbaseT.assign(P.L + 1, nullptr);
  P.gcountT.assign(P.L + 1, nullptr);
  P.gbaseT.assign(P.L + 1, nullptr);
  for (int l = 0; spd && l <= P.L; ++l) {
    const auto &v = P.lv[l];
    if (!v.cls) continue;
    P.clsT[l] = (uint8_t *)take(v.ps);
    P.rwT[l] = (uint32_t *)take((v.n / 8) * sizeof(uint32_t));
    P.rcountT[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.rbaseT[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.gcountT[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
    P.gbaseT[l] = (uint32_t *)take(v.ntiles * sizeof(uint32_t));
  }
  // general-cell and mixed-run lists of one level at a time (setup only)
  P.glist = nlist ? (uint32_t *)take((size_t)nlist * sizeof(uint32_t)) : nullptr;
  P.rlist = nlist ? (uint32_t *)take((size_t)(nlist / 8 + 1) * sizeof(uint32_t)) : nullptr;
  // the lists of each classed level >= 1 (SmallSMModelDn3D kind), built on that level's stream
  P.glists.assign(P.L + 1, nullptr);
  P.rlists.assign(P.L + 1, nullptr);
  for (int l = 1; P.kind == MLPCG_PRECOND_SM && l <= P.L; ++l) {
    if (!P.lv[l].cls) continue;
    P.glists[l] = (uint32_t *)take((size_t)P.lv[l].n * sizeof(uint32_t));
    P.rlists[l] = (uint32_t *)take((size_t)(P.lv[l].n / 8 + 1) * sizeof(uint32_t));
  }
  if (P.lv[0].cls && nlist) {
    P.pkeys = (unsigned long long *)take((size_t)kPatSlots * sizeof(unsigned long long));
    P.pidx = (uint32_t *)take((size_t)kPatSlots * sizeof(uint32_t));
    P.pcount = (uint32_t *)take(2 * sizeof(uint32_t));  // [0] entries used, [1] failure flag
    P.pcoef = (float *)take((size_t)kPatMax * 2 * 28 * sizeof(float));
    P.cell_slot = (uint32_t *)take((size_t)P.lv[0].n * sizeof(uint32_t));
  }
  for (int l = 0; l < P.L; ++l) P.y[l] = take(P.lv[l].ps * sa);
  for (int l = 1; l <= P.L; ++l) {
    P.xin[l] = take(P.lv[l].ps * sa);
    P.xout[l] = take(P.lv[l].ps * sa);
  }
  // the finest level's prolongated input (fast path only; the SPD kind uses it on every level)
  P.ufine = P.lv[0].fast ? take(P.lv[0].ps * sizeof(float)) : nullptr;  // FP32 on level 0 (TMA-staged)
  P.xtmp = P.kind == MLPCG_PRECOND_SMALL_SPD ? take(P.lv[P.L].ps * sa) : nullptr;
  // FP32 on a tiled finest level (the V^T pre-block loads it by TMA), else the activation dtype
  P.v0 = full ? take(P.lv[0].ps * (P.lv[0].fast ? sizeof(float) : sa)) : nullptr;
  P.coef = (float *)take(2 * P.L * sizeof(float));
  P.fmask = (uint8_t *)take(P.lv[0].ps + 64);
  P.lin_ws = take(linear_workspace());
  P.lin_wss.assign(P.L, nullptr);
  for (int l = 0; P.kind == MLPCG_PRECOND_SM && l < P.L; ++l) P.lin_wss[l] = take(linear_workspace());
  P.err = (int *)take(2 * sizeof(int));  // [0]: a tile copy did not complete, [1]: copy-stall test knob
  // scratch last: the general path's temporaries (sized in the plan's byte count) follow it
  P.scratch = (float *)take(96 * sizeof(float));
  // scratch for the general path: level-0 scaled input and one activation-sized temp
  return off;
}

}  // namespace mlpcg

using namespace mlpcg;

typedef struct mlpcg_precond mlpcg_precond;
struct mlpcg_precond {
  PrecondPlan p;
  ~mlpcg_precond() {
    for (cudaStream_t s : p.sides) cudaStreamDestroy(s);
    if (p.fork_ev) cudaEventDestroy(p.fork_ev);
    for (cudaEvent_t e : p.img_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : p.join_evs) cudaEventDestroy(e);
  }
};

#define RET_IF(expr) do { int _r = (expr); if (_r != MLPCG_OK) return _r; } while (0)

// launch helpers for the fast kernels ------------------------------------------
static dim3 grid_of(const PrecondPlan::Level &v) {
  return dim3((unsigned)((v.n3 + TZ - 1) / TZ), (unsigned)((v.n2 + TY - 1) / TY), (unsigned)((v.n1 + TX - 1) / TX));
}

template <typename KT>
static CoefArgs<KT> coef_args(const PrecondPlan &P, int l, void *K, float *uni) {
  CoefArgs<KT> C;
  // the block's material records sit at the same block offset as its uniform vectors
  C.mrec = uni ? (const KT *)P.Mrec + (size_t)((uni - P.Uall) / (3 * KREC)) * 3 * RREC : nullptr;
  C.K = (const KT *)K;
  C.ps = P.lv[l].ps;
  C.rec = (const KT *)K;
  C.kuni = uni;
  C.rw = P.rw[l];
  C.rbase = P.rbase[l];
  C.rcount = P.rcount[l];
  return C;
}

// a transposed block of the SPD kind: its own run words and tile counts
template <typename KT>
static CoefArgs<KT> coef_args_t(const PrecondPlan &P, int l, void *K, float *uni) {
  CoefArgs<KT> C = coef_args<KT>(P, l, K, uni);
  C.rw = P.rwT[l];
  C.rbase = P.rbaseT[l];
  C.rcount = P.rcountT[l];
  return C;
}

namespace mlpcg {
// exclusive prefix sum of n uint32 counts (one CTA)
int launch_scan_u32(const uint32_t *cnt, uint32_t *base, int n, cudaStream_t st) {
  k_scan_tiles<<<1, 1024, 0, st>>>(cnt, base, n);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}
}  // namespace mlpcg

// cuTensorMapEncodeTiled of the driver, looked up once through the runtime (no link to libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

namespace mlpcg {
// Tensor map of an FP32 N1 x N2 x N3 grid vector (z fastest) for TMA tile loads of boxes
// box_z x box_y x box_x, zero fill outside the grid.  The callers' box z origins are multiples
// of 4 floats (16 bytes) as TMA requires; N3 % 4 == 0 makes the row strides multiples of 16
// bytes.  false if the encoder is unavailable or the base is not 16-byte aligned.
bool encode_grid_map(CUtensorMap *m, const float *base, int n1, int n2, int n3, int box_z, int box_y, int box_x) {
  const auto enc = tensor_map_encoder();
  if (!enc || ((uintptr_t)base & 15) || n3 % 4) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)n3, (cuuint64_t)n2, (cuuint64_t)n1};
  const cuuint64_t strides[2] = {(cuuint64_t)n3 * 4, (cuuint64_t)n3 * (cuuint64_t)n2 * 4};
  const cuuint32_t box[3] = {(cuuint32_t)box_z, (cuuint32_t)box_y, (cuuint32_t)box_x};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace mlpcg

// Tensor map of the FP32 fine-grid input r (or u) for the level-0 TMA tile loads: box
// 76 (z) x 18 (y) x 4 (x) = the shared tile.
static bool encode_input_map(CUtensorMap *m, const float *r, const PrecondPlan::Level &v) {
  return encode_grid_map(m, r, v.n1, v.n2, v.n3, HZP, HY, HX);
}

// The level-0 pre-block (FP32 input r, scaled by rscale): TMA-staged when the tensor map
// encodes, else the thread-staged kernel.
template <typename KT, typename AT>
static int launch_pre0(const PrecondPlan &P, const CoefArgs<KT> &C, const float *r, const float *rscale, AT *y,
                       AT *ypool, const uint8_t *mask, cudaStream_t st, const int *gate) {
  const auto &v = P.lv[0];
  const dim3 g = grid_of(v);
  CUtensorMap tm;
  if (encode_input_map(&tm, r, v)) {
    if (v.cls) k_pre_fused_tma<KT, AT, true><<<g, PT, 0, st>>>(C, tm, rscale, y, ypool, mask, v.n1, v.n2, v.n3, gate, P.err);
    else k_pre_fused_tma<KT, AT, false><<<g, PT, 0, st>>>(C, tm, rscale, y, ypool, mask, v.n1, v.n2, v.n3, gate, P.err);
  } else {
    if (v.cls) k_pre_fused<KT, float, AT, true, true><<<g, PT, 0, st>>>(C, r, rscale, y, ypool, mask, v.n1, v.n2, v.n3, gate);
    else k_pre_fused<KT, float, AT, true, false><<<g, PT, 0, st>>>(C, r, rscale, y, ypool, mask, v.n1, v.n2, v.n3, gate);
  }
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

// The finest level's post-block on its prolongated input u (FP32, in P.ufine): TMA-staged when
// the tensor map encodes, else the thread-staged kernel.
// zd (non-NULL only when precond_zdots_tiles allows it): the npsd products as the TMA kernel's
// epilogue.
template <typename KT, typename AT, typename OT, bool SWAP>
static int launch_post0(const PrecondPlan &P, const CoefArgs<KT> &C, const AT *yl, const float *c0, const float *c1,
                        OT *out, const uint8_t *bm, const uint8_t *om, cudaStream_t st, const int *gate,
                        const ZDots *zd = nullptr) {
  const auto &v = P.lv[0];
  const dim3 g = grid_of(v);
  const float *u = (const float *)P.ufine;
  CUtensorMap tm;
  if (encode_input_map(&tm, u, v)) {
    const ZDots z = zd ? *zd : ZDots{};
    if (zd && v.cls) k_post_fused_tma<KT, AT, OT, SWAP, true, true><<<g, PT, 0, st>>>(C, tm, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate, P.err, z);
    else if (zd) k_post_fused_tma<KT, AT, OT, SWAP, false, true><<<g, PT, 0, st>>>(C, tm, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate, P.err, z);
    else if (v.cls) k_post_fused_tma<KT, AT, OT, SWAP, true><<<g, PT, 0, st>>>(C, tm, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate, P.err, z);
    else k_post_fused_tma<KT, AT, OT, SWAP, false><<<g, PT, 0, st>>>(C, tm, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate, P.err, z);
  } else {
    MLPCG_REQUIRE(!zd, MLPCG_ERR_ARG, "precond apply: product epilogue without a TMA level-0 post-block");
    if (v.cls) k_post_fused<KT, float, AT, OT, SWAP, true, true><<<g, PT, 0, st>>>(C, u, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate);
    else k_post_fused<KT, float, AT, OT, SWAP, false, true><<<g, PT, 0, st>>>(C, u, yl, c0, c1, out, bm, om, v.n1, v.n2, v.n3, gate);
  }
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

// One application of the SPD kind (SPDSMModelDn3D.eval_forward, sm_model_3d.py:313-347): the
// V-cycle V (stages 0 .. 2L) into v0, then V^T (stages 2L + 1 .. 4L + 1) into z.
//   V:   y_l = l0[l](x_l), x_{l+1} = pool(y_l); x_L = l(x_L);
//        x_l = c0 y_l + c1 l1[l](P x_{l+1})                       (P = nearest x2 / 8)
//   V^T: w_0 = v0, w_{l+1} = pool(l1_t[l](w_l)); w_L = l_t(w_L);
//        w_l = l0_t[l](c0 w_l + c1 P w_{l+1})
// V^T's skip vector of level l is that level's input w_l (xin[l], v0 on level 0).
template <typename KT, typename AT>
static int run_apply_spd(const PrecondPlan &P, const float *r, const float *rscale, float *z, void *tmp0,
                         cudaStream_t st, int s0, int s1, const int *gate) {
  const int L = P.L;
  auto in_range = [&](int s) { return s >= s0 && s <= s1; };
  // ---- V: down sweep with l0, as the other networks' pre-blocks
  for (int l = 0; l < L; ++l) {
    if (!in_range(l)) continue;
    const auto &v = P.lv[l];
    if (v.fast) {
      const CoefArgs<KT> C = coef_args<KT>(P, l, P.Kpre[l], v.cls ? P.Upre[l] : nullptr);
      if (l == 0) {
        RET_IF((launch_pre0<KT, AT>(P, C, r, rscale, (AT *)P.y[0], (AT *)P.xin[1], nullptr, st, gate)));
      } else {
        if (v.cls)
          k_pre_fused<KT, AT, AT, true, true><<<grid_of(v), PT, 0, st>>>(
              C, (const AT *)P.xin[l], nullptr, (AT *)P.y[l], (AT *)P.xin[l + 1], nullptr, v.n1, v.n2, v.n3, gate);
        else
          k_pre_fused<KT, AT, AT, true, false><<<grid_of(v), PT, 0, st>>>(
              C, (const AT *)P.xin[l], nullptr, (AT *)P.y[l], (AT *)P.xin[l + 1], nullptr, v.n1, v.n2, v.n3, gate);
      }
      MLPCG_LAUNCH_CHECK();
    } else {
      const void *src = P.xin[l];
      if (l == 0) {
        k_scale_copy<AT><<<blocks_for(v.n, 256), 256, 0, st>>>(r, rscale, (AT *)tmp0, v.n);
        MLPCG_LAUNCH_CHECK();
        src = tmp0;
      }
      RET_IF(launch_stencil_apply(P.Kpre[l], P.kdt, v.ps, src, P.adt, 0, P.y[l], P.adt, 1, v.n1, v.n2, v.n3, 0, st));
      RET_IF(launch_avg_pool2(P.y[l], P.xin[l + 1], P.adt, 1, v.n1, v.n2, v.n3, st));
    }
  }
  // ---- coarsest block l (V), l_t (V^T): xin[L] -> xout[L]
  auto coarsest = [&](bool transposed) -> int {
    const auto &v = P.lv[L];
    if (v.fast) {
      const CoefArgs<KT> C = transposed ? coef_args_t<KT>(P, L, P.Klt, v.cls ? P.Ult : nullptr)
                                        : coef_args<KT>(P, L, P.Kl, v.cls ? P.Ul : nullptr);
      if (v.cls)
        k_pre_fused<KT, AT, AT, false, true><<<grid_of(v), PT, 0, st>>>(
            C, (const AT *)P.xin[L], nullptr, (AT *)P.xout[L], nullptr, nullptr, v.n1, v.n2, v.n3, gate);
      else
        k_pre_fused<KT, AT, AT, false, false><<<grid_of(v), PT, 0, st>>>(
            C, (const AT *)P.xin[L], nullptr, (AT *)P.xout[L], nullptr, nullptr, v.n1, v.n2, v.n3, gate);
      MLPCG_LAUNCH_CHECK();
      return MLPCG_OK;
    }
    return launch_stencil_apply(P.Kl, P.kdt, v.ps, P.xin[L], P.adt, 0, P.xout[L], P.adt, 1, v.n1, v.n2, v.n3,
                                transposed ? 1 : 0, st);
  };
  if (in_range(L)) RET_IF(coarsest(false));
  // ---- V: up sweep, x_l = c0 y_l + c1 l1[l](P x_{l+1}); level 0 into v0 (FP32 when tiled)
  for (int l = L - 1; l >= 0; --l) {
    if (!in_range(2 * L - l)) continue;
    const auto &v = P.lv[l];
    const float *c0 = P.coef + l, *c1 = P.coef + L + l;
    AT *o = (AT *)(l == 0 ? P.v0 : P.xout[l]);
    if (v.fast) {
      const CoefArgs<KT> C = coef_args<KT>(P, l, P.Kpost[l], v.cls ? P.Upost[l] : nullptr);
      const dim3 g = grid_of(v);
      if (l == 0) {
        k_up_fine<AT, AT, float, false, true><<<g, PT, 0, st>>>((const AT *)P.xout[1], (const AT *)P.y[0], c0, c1,
                                                                 (float *)P.ufine, v.n1, v.n2, v.n3, gate);
        MLPCG_LAUNCH_CHECK();
        RET_IF((launch_post0<KT, AT, float, false>(P, C, (const AT *)P.y[0], c0, c1, (float *)P.v0, nullptr, nullptr,
                                                    st, gate)));
      } else {
        AT *u = (AT *)P.ufine;
        k_up_fine<AT, AT, AT, false, true><<<g, PT, 0, st>>>((const AT *)P.xout[l + 1], (const AT *)P.y[l], c0, c1, u,
                                                              v.n1, v.n2, v.n3, gate);
        MLPCG_LAUNCH_CHECK();
        if (v.cls) k_post_fused<KT, AT, AT, AT, false, true, true><<<g, PT, 0, st>>>(C, u, (const AT *)P.y[l], c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        else k_post_fused<KT, AT, AT, AT, false, false, true><<<g, PT, 0, st>>>(C, u, (const AT *)P.y[l], c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        MLPCG_LAUNCH_CHECK();
      }
    } else {
      RET_IF(launch_avg_pool2_adjoint(P.xout[l + 1], tmp0, P.adt, 1, v.n1, v.n2, v.n3, st));
      RET_IF(launch_stencil_apply(P.Kpost[l], P.kdt, v.ps, tmp0, P.adt, 0, o, P.adt, 1, v.n1, v.n2, v.n3, 0, st));
      RET_IF(launch_axpby(c0, P.y[l], c1, o, o, P.adt, v.n, st));
    }
  }
  // ---- V^T: down sweep with l1_t from v0; only the pooled outputs are kept
  const int B = 2 * L + 1;
  for (int l = 0; l < L; ++l) {
    if (!in_range(B + l)) continue;
    const auto &v = P.lv[l];
    const AT *src = (const AT *)(l == 0 ? P.v0 : P.xin[l]);
    if (v.fast && l == 0) {  // v0 is FP32: the TMA-staged pre-block, unscaled
      const CoefArgs<KT> C = coef_args_t<KT>(P, 0, P.KpostT[0], v.cls ? P.UpostT[0] : nullptr);
      RET_IF((launch_pre0<KT, AT>(P, C, (const float *)P.v0, nullptr, (AT *)nullptr, (AT *)P.xin[1], nullptr, st,
                                  gate)));
    } else if (v.fast) {
      const CoefArgs<KT> C = coef_args_t<KT>(P, l, P.KpostT[l], v.cls ? P.UpostT[l] : nullptr);
      if (v.cls)
        k_pre_fused<KT, AT, AT, true, true><<<grid_of(v), PT, 0, st>>>(
            C, src, nullptr, (AT *)nullptr, (AT *)P.xin[l + 1], nullptr, v.n1, v.n2, v.n3, gate);
      else
        k_pre_fused<KT, AT, AT, true, false><<<grid_of(v), PT, 0, st>>>(
            C, src, nullptr, (AT *)nullptr, (AT *)P.xin[l + 1], nullptr, v.n1, v.n2, v.n3, gate);
      MLPCG_LAUNCH_CHECK();
    } else {
      RET_IF(launch_stencil_apply(P.Kpost[l], P.kdt, v.ps, src, P.adt, 0, tmp0, P.adt, 1, v.n1, v.n2, v.n3, 1, st));
      RET_IF(launch_avg_pool2(tmp0, P.xin[l + 1], P.adt, 1, v.n1, v.n2, v.n3, st));
    }
  }
  if (in_range(B + L)) RET_IF(coarsest(true));
  // ---- V^T: up sweep, w_l = l0_t[l](c0 w_l + c1 P w_{l+1}); level 0 into z, zero off the fluid cells
  for (int l = L - 1; l >= 0; --l) {
    if (!in_range(B + 2 * L - l)) continue;
    const auto &v = P.lv[l];
    const float *c0 = P.coef + l, *c1 = P.coef + L + l;
    const AT *skip = (const AT *)(l == 0 ? P.v0 : P.xin[l]);
    if (v.fast) {
      const CoefArgs<KT> C = coef_args_t<KT>(P, l, P.KpreT[l], v.cls ? P.UpreT[l] : nullptr);
      const dim3 g = grid_of(v);
      if (l == 0) {  // skip vector v0 in FP32
        k_up_fine<AT, float, float, true, true><<<g, PT, 0, st>>>((const AT *)P.xout[1], (const float *)P.v0, c0, c1,
                                                                   (float *)P.ufine, v.n1, v.n2, v.n3, gate);
        MLPCG_LAUNCH_CHECK();
        RET_IF((launch_post0<KT, AT, float, true>(P, C, (const AT *)nullptr, c0, c1, z, nullptr, P.fmask, st, gate)));
      } else {
        AT *u = (AT *)P.ufine;
        k_up_fine<AT, AT, AT, true, true><<<g, PT, 0, st>>>((const AT *)P.xout[l + 1], skip, c0, c1, u, v.n1, v.n2,
                                                             v.n3, gate);
        MLPCG_LAUNCH_CHECK();
        AT *o = (AT *)P.xout[l];
        if (v.cls) k_post_fused<KT, AT, AT, AT, true, true, true><<<g, PT, 0, st>>>(C, u, skip, c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        else k_post_fused<KT, AT, AT, AT, true, false, true><<<g, PT, 0, st>>>(C, u, skip, c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
      }
      MLPCG_LAUNCH_CHECK();
    } else {
      void *dst = (l == 0) ? (void *)z : P.xout[l];
      const int ddt = (l == 0) ? MLPCG_F32 : P.adt;
      RET_IF(launch_avg_pool2_adjoint(P.xout[l + 1], tmp0, P.adt, 1, v.n1, v.n2, v.n3, st));
      RET_IF(launch_axpby(c0, skip, c1, tmp0, tmp0, P.adt, v.n, st));
      RET_IF(launch_stencil_apply(P.Kpre[l], P.kdt, v.ps, tmp0, P.adt, 0, dst, ddt, 1, v.n1, v.n2, v.n3, 1, st));
      if (l == 0) {
        k_apply_mask<float><<<blocks_for(v.n, 256), 256, 0, st>>>((float *)dst, P.fmask, v.n);
        MLPCG_LAUNCH_CHECK();
      }
    }
  }
  return MLPCG_OK;
}

// Stages of one application, in launch order: 0..L-1 = pre-block of level s,
// L = coarsest block, L+1..2L = post-block of level 2L-s.  [s0, s1] selects a range.
// CTAs of the coarse-level cluster kernel this device runs as one cluster: 16 (non-portable
// size) or 8, 0 if neither (the per-level kernels are used then).  Looked up once per
// instantiation.
template <typename KT, typename AT, bool CLS, bool SWAP>
static int coarse_cluster_ctas() {
  static const int ctas = [] {
    auto kern = k_coarse_cluster<KT, AT, CLS, SWAP>;
    for (int c : {16, 8}) {
      if (c > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        (void)cudaGetLastError();
        continue;
      }
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)c);
      cfg.blockDim = dim3(PT);
      cudaLaunchAttribute at{};
      at.id = cudaLaunchAttributeClusterDimension;
      at.val.clusterDim.x = (unsigned)c;
      at.val.clusterDim.y = 1;
      at.val.clusterDim.z = 1;
      cfg.attrs = &at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n >= 1) return c;
      (void)cudaGetLastError();
    }
    return 0;
  }();
  return ctas;
}

// The first level of the coarse-level cluster kernel for a SmallSMModelDn3D plan: the smallest
// l >= 1 from which every level down to the coarsest runs the tiled kernels in one coefficient
// layout, with at most 4 tiles per CTA at level l; -1 when no two levels qualify.
static int coarse_cluster_level(const PrecondPlan &P, int ctas) {
  if (P.kind != MLPCG_PRECOND_SM || ctas <= 0) return -1;
  const int L = P.L;
  int lc = -1;
  for (int l = L - 1; l >= 1 && L - l + 1 <= kCoarseMaxLev; --l) {
    bool ok = true;
    for (int m = l; m <= L; ++m) ok = ok && P.lv[m].fast && P.lv[m].cls == P.lv[L].cls;
    if (!ok || P.lv[l].ntiles > (unsigned)(4 * ctas)) break;
    lc = l;
  }
  return lc;
}

template <typename KT, typename AT, bool CLS, bool SWAP>
static int launch_coarse_cluster(const PrecondPlan &P, int lc, int ctas, cudaStream_t st, const int *gate) {
  const int L = P.L;
  CoarseArgs<KT, AT> A{};
  A.nlev = L - lc + 1;
  for (int i = 0; i < A.nlev; ++i) {
    const int l = lc + i;
    const auto &v = P.lv[l];
    const dim3 g = grid_of(v);
    A.n1[i] = v.n1; A.n2[i] = v.n2; A.n3[i] = v.n3;
    A.tz[i] = (int)g.x; A.ty[i] = (int)g.y;
    A.ntiles[i] = v.ntiles;
    A.x[i] = (AT *)P.xin[l];
    A.xo[i] = (AT *)P.xout[l];
    if (l < L) {
      A.pre[i] = coef_args<KT>(P, l, P.Kpre[l], CLS ? P.Upre[l] : nullptr);
      A.post[i] = coef_args<KT>(P, l, P.Kpost[l], CLS ? P.Upost[l] : nullptr);
      A.y[i] = (AT *)P.y[l];
      A.c0[i] = P.coef + l;
      A.c1[i] = P.coef + L + l;
    } else {
      A.pre[i] = coef_args<KT>(P, L, P.Kl, CLS ? P.Ul : nullptr);
    }
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(PT);
  cfg.stream = st;
  cudaLaunchAttribute at{};
  at.id = cudaLaunchAttributeClusterDimension;
  at.val.clusterDim.x = (unsigned)ctas;
  at.val.clusterDim.y = 1;
  at.val.clusterDim.z = 1;
  cfg.attrs = &at;
  cfg.numAttrs = 1;
  MLPCG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, k_coarse_cluster<KT, AT, CLS, SWAP>, A, gate));
  return MLPCG_OK;
}

template <typename KT, typename AT>
static int run_coarse_cluster(const PrecondPlan &P, int lc, int ctas, cudaStream_t st, const int *gate) {
  const bool cls = P.lv[P.L].cls;
  if (P.swap) return cls ? launch_coarse_cluster<KT, AT, true, true>(P, lc, ctas, st, gate)
                         : launch_coarse_cluster<KT, AT, false, true>(P, lc, ctas, st, gate);
  return cls ? launch_coarse_cluster<KT, AT, true, false>(P, lc, ctas, st, gate)
             : launch_coarse_cluster<KT, AT, false, false>(P, lc, ctas, st, gate);
}

template <typename KT, typename AT>
static int cluster_ctas_for(const PrecondPlan &P) {
  const bool cls = P.lv[P.L].cls;
  if (P.swap) return cls ? coarse_cluster_ctas<KT, AT, true, true>() : coarse_cluster_ctas<KT, AT, false, true>();
  return cls ? coarse_cluster_ctas<KT, AT, true, false>() : coarse_cluster_ctas<KT, AT, false, false>();
}

// The small levels (their tiles fit in one wave of CTAs: at most P.small_tiles_per_sm per SM)
// run the block kernels' prefetching variant when the coefficients are BF16.
template <typename KT>
static bool small_level(const PrecondPlan &P, const PrecondPlan::Level &v) {
  return std::is_same<KT, __nv_bfloat16>::value &&
         v.ntiles <= (unsigned)P.small_tiles_per_sm * (unsigned)sm_count();
}

template <typename KT, typename AT, bool POOL, bool CLS>
static void launch_pre_level(const PrecondPlan &P, const PrecondPlan::Level &v, const CoefArgs<KT> &C, const AT *x,
                             AT *y, AT *yp, cudaStream_t st, const int *gate) {
  if constexpr (std::is_same<KT, __nv_bfloat16>::value) {
    if (small_level<KT>(P, v)) {
      k_pre_fused_small<KT, AT, AT, POOL, CLS><<<grid_of(v), PT, 0, st>>>(C, x, y, yp, v.n1, v.n2, v.n3, gate);
      return;
    }
  }
  k_pre_fused<KT, AT, AT, POOL, CLS><<<grid_of(v), PT, 0, st>>>(C, x, nullptr, y, yp, nullptr, v.n1, v.n2, v.n3,
                                                                gate);
}

template <typename KT, typename AT, bool SWAP, bool CLS>
static void launch_post_level(const PrecondPlan &P, const PrecondPlan::Level &v, const CoefArgs<KT> &C,
                              const AT *xc, const AT *yl, const float *c0, const float *c1, AT *o, cudaStream_t st,
                              const int *gate) {
  if constexpr (std::is_same<KT, __nv_bfloat16>::value) {
    if (small_level<KT>(P, v)) {
      k_post_fused_small<KT, AT, SWAP, CLS><<<grid_of(v), PT, 0, st>>>(C, xc, yl, c0, c1, o, v.n1, v.n2, v.n3,
                                                                         gate);
      return;
    }
  }
  k_post_fused<KT, AT, AT, AT, SWAP, CLS, false><<<grid_of(v), PT, 0, st>>>(C, xc, yl, c0, c1, o, nullptr, nullptr,
                                                                           v.n1, v.n2, v.n3, gate);
}

template <typename KT, typename AT>
static int run_apply(const PrecondPlan &P, const float *r, const float *rscale, float *z, void *tmp0,
                     cudaStream_t st, int s0 = 0, int s1 = 1 << 20, const int *gate = nullptr,
                     const ZDots *zd = nullptr) {
  if (P.kind == MLPCG_PRECOND_SPD) return run_apply_spd<KT, AT>(P, r, rscale, z, tmp0, st, s0, s1, gate);
  const int L = P.L;
  const uint8_t *m0 = P.mask ? P.fmask : nullptr;
  // levels lc .. L in one cluster launch when the range covers all of their stages
  const int ctas = P.kind == MLPCG_PRECOND_SM && P.coarse_cluster ? cluster_ctas_for<KT, AT>(P) : 0;
  const int lc = coarse_cluster_level(P, ctas);
  const bool cluster = lc > 0 && s0 <= lc && s1 >= 2 * L - lc;
  // ---- down sweep
  for (int l = 0; l < L; ++l) {
    const auto &v = P.lv[l];
    if (l < s0 || l > s1 || (cluster && l >= lc)) continue;
    if (v.fast) {
      const CoefArgs<KT> C = coef_args<KT>(P, l, P.Kpre[l], v.cls ? P.Upre[l] : nullptr);
      if (l == 0) {
        RET_IF((launch_pre0<KT, AT>(P, C, r, rscale, (AT *)P.y[0], (AT *)P.xin[1], m0, st, gate)));
      } else {
        if (v.cls)
          launch_pre_level<KT, AT, true, true>(P, v, C, (const AT *)P.xin[l], (AT *)P.y[l], (AT *)P.xin[l + 1], st, gate);
        else
          launch_pre_level<KT, AT, true, false>(P, v, C, (const AT *)P.xin[l], (AT *)P.y[l], (AT *)P.xin[l + 1], st,
                                                gate);
      }
      MLPCG_LAUNCH_CHECK();
    } else {
      const void *src = P.xin[l];
      int sdt = P.adt;
      if (l == 0) {
        k_scale_copy<AT><<<blocks_for(v.n, 256), 256, 0, st>>>(r, rscale, (AT *)tmp0, v.n);
        MLPCG_LAUNCH_CHECK();
        src = tmp0;
      }
      RET_IF(launch_stencil_apply(P.Kpre[l], P.kdt, v.ps, src, sdt, 0, P.y[l], P.adt, 1, v.n1, v.n2, v.n3, 0, st));
      if (l == 0 && m0) {
        k_apply_mask<AT><<<blocks_for(v.n, 256), 256, 0, st>>>((AT *)P.y[0], m0, v.n);
        MLPCG_LAUNCH_CHECK();
      }
      RET_IF(launch_avg_pool2(P.y[l], P.xin[l + 1], P.adt, 1, v.n1, v.n2, v.n3, st));
    }
  }
  if (cluster) RET_IF((run_coarse_cluster<KT, AT>(P, lc, ctas, st, gate)));
  // ---- coarsest block (SPD kind: l into xtmp, then l_t)
  const bool spd = P.kind == MLPCG_PRECOND_SMALL_SPD;
  if (L >= s0 && L <= s1 && !cluster) {
    const auto &v = P.lv[L];
    AT *cdst = (AT *)(spd ? P.xtmp : P.xout[L]);
    if (v.fast) {
      const CoefArgs<KT> C = coef_args<KT>(P, L, P.Kl, v.cls ? P.Ul : nullptr);
      if (v.cls) launch_pre_level<KT, AT, false, true>(P, v, C, (const AT *)P.xin[L], cdst, nullptr, st, gate);
      else launch_pre_level<KT, AT, false, false>(P, v, C, (const AT *)P.xin[L], cdst, nullptr, st, gate);
      MLPCG_LAUNCH_CHECK();
      if (spd) {
        const CoefArgs<KT> Ct = coef_args_t<KT>(P, L, P.Klt, v.cls ? P.Ult : nullptr);
        if (v.cls)
          k_pre_fused<KT, AT, AT, false, true><<<grid_of(v), PT, 0, st>>>(
              Ct, (const AT *)P.xtmp, nullptr, (AT *)P.xout[L], nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        else
          k_pre_fused<KT, AT, AT, false, false><<<grid_of(v), PT, 0, st>>>(
              Ct, (const AT *)P.xtmp, nullptr, (AT *)P.xout[L], nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        MLPCG_LAUNCH_CHECK();
      }
    } else {
      RET_IF(launch_stencil_apply(P.Kl, P.kdt, v.ps, P.xin[L], P.adt, 0, cdst, P.adt, 1, v.n1, v.n2, v.n3, 0, st));
      if (spd)
        RET_IF(launch_stencil_apply(P.Kl, P.kdt, v.ps, P.xtmp, P.adt, 0, P.xout[L], P.adt, 1, v.n1, v.n2, v.n3, 1, st));
    }
  }
  // ---- up sweep
  for (int l = L - 1; l >= 0; --l) {
    const auto &v = P.lv[l];
    if (2 * L - l < s0 || 2 * L - l > s1 || (cluster && l >= lc)) continue;
    const float *c0 = P.coef + l, *c1 = P.coef + L + l;
    const uint8_t *bm = (l == 0) ? m0 : nullptr;
    const uint8_t *om = (l == 0) ? P.fmask : nullptr;
    if (spd) {
      // u = c0^2 y_l + c1^2 (nearest x2 / 8)(x_{l+1}) (coef holds the squares), then the
      // transposed block l0_t on u (sm_model_3d.py:436-443)
      if (v.fast) {
        const CoefArgs<KT> C = coef_args_t<KT>(P, l, P.Kpost[l], v.cls ? P.Upost[l] : nullptr);
        const dim3 g = grid_of(v);
        if (l == 0) {
          k_up_fine<AT, AT, float, true, true><<<g, PT, 0, st>>>((const AT *)P.xout[1], (const AT *)P.y[0], c0, c1,
                                                                  (float *)P.ufine, v.n1, v.n2, v.n3, gate);
          MLPCG_LAUNCH_CHECK();
          RET_IF((launch_post0<KT, AT, float, true>(P, C, (const AT *)P.y[0], c0, c1, z, nullptr, om, st, gate, zd)));
        } else {
          AT *u = (AT *)P.ufine;
          k_up_fine<AT, AT, AT, true, true><<<g, PT, 0, st>>>((const AT *)P.xout[l + 1], (const AT *)P.y[l], c0, c1, u,
                                                               v.n1, v.n2, v.n3, gate);
          MLPCG_LAUNCH_CHECK();
          AT *o = (AT *)P.xout[l];
          if (v.cls) k_post_fused<KT, AT, AT, AT, true, true, true><<<g, PT, 0, st>>>(C, u, (const AT *)P.y[l], c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
          else k_post_fused<KT, AT, AT, AT, true, false, true><<<g, PT, 0, st>>>(C, u, (const AT *)P.y[l], c0, c1, o, nullptr, nullptr, v.n1, v.n2, v.n3, gate);
        }
        MLPCG_LAUNCH_CHECK();
      } else {
        void *up = tmp0;
        void *dst = (l == 0) ? (void *)z : P.xout[l];
        const int ddt = (l == 0) ? MLPCG_F32 : P.adt;
        RET_IF(launch_avg_pool2_adjoint(P.xout[l + 1], up, P.adt, 1, v.n1, v.n2, v.n3, st));
        RET_IF(launch_axpby(c0, P.y[l], c1, up, up, P.adt, v.n, st));
        RET_IF(launch_stencil_apply(P.Kpre[l], P.kdt, v.ps, up, P.adt, 0, dst, ddt, 1, v.n1, v.n2, v.n3, 1, st));
        if (l == 0) {
          k_apply_mask<float><<<blocks_for(v.n, 256), 256, 0, st>>>((float *)dst, P.fmask, v.n);
          MLPCG_LAUNCH_CHECK();
        }
      }
      continue;
    }
    if (v.fast) {
      const CoefArgs<KT> C = coef_args<KT>(P, l, P.Kpost[l], v.cls ? P.Upost[l] : nullptr);
      const AT *xc = (const AT *)P.xout[l + 1], *yl = (const AT *)P.y[l];
      const dim3 g = grid_of(v);
      if (l == 0) {
        // the finest level: prolongation as its own pass (FP32 u), then the block on u
        float *u = (float *)P.ufine;
        if (P.swap) {
          k_up_fine<AT, AT, float, true><<<g, PT, 0, st>>>(xc, yl, c0, c1, u, v.n1, v.n2, v.n3, gate);
          MLPCG_LAUNCH_CHECK();
          RET_IF((launch_post0<KT, AT, float, true>(P, C, yl, c0, c1, z, bm, om, st, gate, zd)));
        } else {
          k_up_fine<AT, AT, float, false><<<g, PT, 0, st>>>(xc, yl, c0, c1, u, v.n1, v.n2, v.n3, gate);
          MLPCG_LAUNCH_CHECK();
          RET_IF((launch_post0<KT, AT, float, false>(P, C, yl, c0, c1, z, bm, om, st, gate, zd)));
        }
      } else {
        AT *o = (AT *)P.xout[l];
        if (P.swap) {
          if (v.cls) launch_post_level<KT, AT, true, true>(P, v, C, xc, yl, c0, c1, o, st, gate);
          else launch_post_level<KT, AT, true, false>(P, v, C, xc, yl, c0, c1, o, st, gate);
        } else {
          if (v.cls) launch_post_level<KT, AT, false, true>(P, v, C, xc, yl, c0, c1, o, st, gate);
          else launch_post_level<KT, AT, false, false>(P, v, C, xc, yl, c0, c1, o, st, gate);
        }
      }
      MLPCG_LAUNCH_CHECK();
    } else {
      // general path: up -> (combine) -> block -> (combine) with level-sized temporaries
      void *up = tmp0;                                   // level-l sized, activation dtype
      void *dst = (l == 0) ? (void *)z : P.xout[l];
      const int ddt = (l == 0) ? MLPCG_F32 : P.adt;
      RET_IF(launch_upsample2(P.xout[l + 1], up, P.adt, 1, v.n1 / 2, v.n2 / 2, v.n3 / 2, st));
      if (P.swap) {
        RET_IF(launch_axpby(c0, P.y[l], c1, up, up, P.adt, v.n, st));
        RET_IF(launch_stencil_apply(P.Kpost[l], P.kdt, v.ps, up, P.adt, 0, dst, ddt, 1, v.n1, v.n2, v.n3, 0, st));
        if (bm) {
          k_apply_mask<float><<<blocks_for(v.n, 256), 256, 0, st>>>((float *)dst, bm, v.n);
          MLPCG_LAUNCH_CHECK();
        }
      } else {
        // t = B(up) into up's slot via dst, then combine into dst
        RET_IF(launch_stencil_apply(P.Kpost[l], P.kdt, v.ps, up, P.adt, 0, dst, ddt, 1, v.n1, v.n2, v.n3, 0, st));
        if (l == 0) {
          if (bm) {
            k_apply_mask<float><<<blocks_for(v.n, 256), 256, 0, st>>>((float *)dst, bm, v.n);
            MLPCG_LAUNCH_CHECK();
          }
          // y0 (activation dtype) -> F32 copy in tmp, then z = c0*y0 + c1*t
          k_convert<AT, float><<<blocks_for(v.n, 256), 256, 0, st>>>((const AT *)P.y[0], (float *)up, v.n);
          MLPCG_LAUNCH_CHECK();
          RET_IF(launch_axpby(c0, up, c1, dst, dst, MLPCG_F32, v.n, st));
        } else {
          RET_IF(launch_axpby(c0, P.y[l], c1, dst, dst, P.adt, v.n, st));
        }
      }
      if (l == 0) {
        k_apply_mask<float><<<blocks_for(v.n, 256), 256, 0, st>>>((float *)dst, P.fmask, v.n);
        MLPCG_LAUNCH_CHECK();
      }
    }
  }
  return MLPCG_OK;
}

namespace mlpcg {
// the plan's copy-failed word (device memory; valid once the plan is set up)
const int *precond_copy_flag(const mlpcg_precond *h) { return h->p.ready ? h->p.err : nullptr; }

int64_t precond_level0_tiles(const mlpcg_precond *h);

// Tiles of the finest level when the plan can compute the solver's products (ZDots) in its level-0
// post-block -- the SmallSMModelDn3D and SmallSPDSMModelDn3D kinds, whose finest post-block is
// the TMA kernel -- else 0.
int64_t precond_zdots_tiles(const mlpcg_precond *h) {
  const PrecondPlan &P = h->p;
  if (!P.ready || (P.kind != MLPCG_PRECOND_SM && P.kind != MLPCG_PRECOND_SMALL_SPD) || !P.lv[0].fast) return 0;
  CUtensorMap tm;
  if (!encode_input_map(&tm, (const float *)P.ufine, P.lv[0])) return 0;
  return precond_level0_tiles(h);
}

// tiles of the finest level's grid (known from creation on)
int64_t precond_level0_tiles(const mlpcg_precond *h) {
  const dim3 g = grid_of(h->p.lv[0]);
  return (int64_t)g.x * g.y * g.z;
}

// mlpcg_precond_apply whose fused kernels return at once while *gate != 0
// (the batched solver passes each system's status word); zd (only where precond_zdots_tiles > 0):
// the npsd products computed by the level-0 post-block
int precond_apply_gated(const mlpcg_precond *h, const float *r, const float *r_scale, float *z, const int *gate,
                        void *stream, const ZDots *zd) {
  const PrecondPlan &P = h->p;
  cudaStream_t st = as_stream(stream);
  void *tmp0 = (char *)P.scratch + al256(96 * sizeof(float));
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_BF16)
    return run_apply<__nv_bfloat16, __nv_bfloat16>(P, r, r_scale, z, tmp0, st, 0, 1 << 20, gate, zd);
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_F32)
    return run_apply<__nv_bfloat16, float>(P, r, r_scale, z, tmp0, st, 0, 1 << 20, gate, zd);
  if (P.kdt == MLPCG_F32 && P.adt == MLPCG_BF16)
    return run_apply<float, __nv_bfloat16>(P, r, r_scale, z, tmp0, st, 0, 1 << 20, gate, zd);
  return run_apply<float, float>(P, r, r_scale, z, tmp0, st, 0, 1 << 20, gate, zd);
}
}  // namespace mlpcg

extern "C" {

static int precond_create(int N1, int N2, int N3, int levels, int k_dtype, int act_dtype, int swap_sm_order,
                          int mask, int coeff_layout, int kind, mlpcg_precond **out) {
  MLPCG_REQUIRE(out != nullptr, MLPCG_ERR_ARG, "out must not be NULL");
  *out = nullptr;
  MLPCG_REQUIRE(levels >= 1 && levels <= 12, MLPCG_ERR_ARG, "levels %d out of [1, 12]", levels);
  MLPCG_REQUIRE(N1 >= 1 && N2 >= 1 && N3 >= 1, MLPCG_ERR_SHAPE, "grid sizes must be >= 1");
  const int f = 1 << levels;
  MLPCG_REQUIRE(N1 % f == 0 && N2 % f == 0 && N3 % f == 0, MLPCG_ERR_SHAPE,
                "grid %d x %d x %d must be divisible by 2^levels = %d", N1, N2, N3, f);
  MLPCG_REQUIRE((k_dtype == MLPCG_F32 || k_dtype == MLPCG_BF16) && (act_dtype == MLPCG_F32 || act_dtype == MLPCG_BF16),
                MLPCG_ERR_UNSUPPORTED, "coefficient / activation storage must be F32 or BF16");
  MLPCG_REQUIRE(coeff_layout == MLPCG_COEFF_DENSE || coeff_layout == MLPCG_COEFF_CLASSED, MLPCG_ERR_ARG,
                "coeff_layout must be MLPCG_COEFF_DENSE or MLPCG_COEFF_CLASSED");
  // classed levels index cells and records with 32-bit integers
  MLPCG_REQUIRE(coeff_layout == MLPCG_COEFF_DENSE || cells(N1, N2, N3) < ((int64_t)1 << 32), MLPCG_ERR_SHAPE,
                "the classed layout needs fewer than 2^32 cells (grid %d x %d x %d)", N1, N2, N3);
  auto *h = new mlpcg_precond();
  PrecondPlan &P = h->p;
  P.n1 = N1; P.n2 = N2; P.n3 = N3; P.L = levels;
  P.kdt = k_dtype; P.adt = act_dtype; P.swap = swap_sm_order ? 1 : 0; P.mask = mask ? 1 : 0;
  P.layout = coeff_layout;
  P.kind = kind;
  for (int l = 0; l <= levels; ++l) {
    PrecondPlan::Level v;
    v.n1 = N1 >> l; v.n2 = N2 >> l; v.n3 = N3 >> l;
    v.n = cells(v.n1, v.n2, v.n3);
    v.ps = (v.n + 63) / 64 * 64;
    v.fast = (v.n3 % 8 == 0);
    v.cls = v.fast && coeff_layout == MLPCG_COEFF_CLASSED;
    const dim3 g = grid_of(v);
    v.ntiles = g.x * g.y * g.z;
    P.lv.push_back(v);
  }
  P.bytes = plan_layout(P, nullptr);
  // temporaries of the general path: level-0 sized activation + F32 buffer
  P.bytes += al256(P.lv[0].ps * 4);
  *out = h;
  return MLPCG_OK;
}

int mlpcg_precond_create(int N1, int N2, int N3, int levels, int k_dtype, int act_dtype,
                         int swap_sm_order, int mask, int coeff_layout, mlpcg_precond **out) {
  clear_error();
  return precond_create(N1, N2, N3, levels, k_dtype, act_dtype, swap_sm_order, mask, coeff_layout,
                        MLPCG_PRECOND_SM, out);
}

int mlpcg_precond_create_spd(int N1, int N2, int N3, int levels, int k_dtype, int act_dtype, int coeff_layout,
                             mlpcg_precond **out) {
  clear_error();
  return precond_create(N1, N2, N3, levels, k_dtype, act_dtype, 0, 0, coeff_layout, MLPCG_PRECOND_SMALL_SPD, out);
}

int mlpcg_precond_create_kind(int N1, int N2, int N3, int levels, int kind, int k_dtype, int act_dtype,
                              int coeff_layout, mlpcg_precond **out) {
  clear_error();
  MLPCG_REQUIRE(kind == MLPCG_PRECOND_SMALL_SPD || kind == MLPCG_PRECOND_SPD, MLPCG_ERR_ARG,
                "precond_create_kind: kind must be MLPCG_PRECOND_SMALL_SPD or MLPCG_PRECOND_SPD");
  return precond_create(N1, N2, N3, levels, k_dtype, act_dtype, 0, 0, coeff_layout, kind, out);
}

size_t mlpcg_precond_workspace(const mlpcg_precond *h) { return h ? h->p.bytes : 0; }

void mlpcg_precond_destroy(mlpcg_precond *h) { delete h; }

int mlpcg_precond_setup(mlpcg_precond *h, void *workspace, size_t workspace_bytes, const float *image,
                        const float *params, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && workspace && image && params, MLPCG_ERR_ARG, "precond_setup: NULL argument");
  PrecondPlan &P = h->p;
  MLPCG_REQUIRE(workspace_bytes >= P.bytes, MLPCG_ERR_WORKSPACE, "precond workspace too small: %zu < %zu",
                workspace_bytes, P.bytes);
  MLPCG_REQUIRE(((uintptr_t)workspace & 255) == 0, MLPCG_ERR_ALIGN, "precond workspace must be 256-byte aligned");
  cudaStream_t st = as_stream(stream);
  plan_layout(P, (char *)workspace);
  MLPCG_CUDA_CHECK(cudaMemsetAsync(P.err, 0, 2 * sizeof(int), st));
  const int L = P.L;
  // parameter offsets: pre[0..L-1], post[0..L-1], l (2214 each), c0[0..L-1], c1[0..L-1] (82 each);
  // SPD kind: l0[0..L-1], l, then the linear blocks
  const bool spd = P.kind == MLPCG_PRECOND_SMALL_SPD;
  const int nblk = spd ? L + 1 : 2 * L + 1;  // SPD kind: l0, l1, l like pre, post, l
  auto blk_w = [&](int b) { return params + (size_t)b * 2214; };
  auto blk_b = [&](int b) { return params + (size_t)b * 2214 + 2187; };
  const float *linp = params + (size_t)nblk * 2214;
  // image pyramid (the SM kind's side stream builds it beside level 0's chain, below)
  const bool side_chain = P.kind == MLPCG_PRECOND_SM && L >= 1;
  auto pyramid = [&](cudaStream_t ps) -> int {
    for (int l = 1; l <= L; ++l) {
      const auto &v = P.lv[l - 1];
      const float *src = (l == 1) ? image : P.img[l - 1];
      RET_IF(launch_avg_pool2(src, P.img[l], MLPCG_F32, 3, v.n1, v.n2, v.n3, ps));
    }
    return MLPCG_OK;
  };
  auto fluid_mask = [&]() -> int {
    const int64_t n0 = P.lv[0].n;
    // 16-byte loads of channel 1 and stores of the mask when n0 is a multiple of 16 and the image
    // 16-byte aligned (the mask is 256-byte aligned)
    if (n0 % 16 == 0 && ((uintptr_t)image & 15) == 0)
      k_fluid_mask16<<<blocks_for(n0 / 16, 256), 256, 0, st>>>(image, P.fmask, n0);
    else
      k_fluid_mask<<<blocks_for(n0, 256), 256, 0, st>>>(image, P.fmask, n0);
    MLPCG_LAUNCH_CHECK();
    return MLPCG_OK;
  };
  if (!side_chain) {
    RET_IF(pyramid(st));
    RET_IF(fluid_mask());
  }
  // coefficients: dense planes, or class map + uniform vectors + general-cell records
  bool any_cls = false;
  for (int l = 0; l <= L; ++l) any_cls = any_cls || P.lv[l].cls;
  if (any_cls) {
    if (P.kdt == MLPCG_BF16) {
      k_kgen_uniform_all<__nv_bfloat16><<<nblk, 3 * KREC, 0, st>>>(params, P.Uall, L, P.kind);
      k_material_records<__nv_bfloat16><<<uniform_blocks(P), 256, 0, st>>>(P.Uall, (__nv_bfloat16 *)P.Mrec);
    } else {
      k_kgen_uniform_all<float><<<nblk, 3 * KREC, 0, st>>>(params, P.Uall, L, P.kind);
      k_material_records<float><<<uniform_blocks(P), 256, 0, st>>>(P.Uall, (float *)P.Mrec);
    }
    MLPCG_LAUNCH_CHECK();
  }
  // one level's blocks b0 (and b1 >= 0): dense planes, or class map + general-cell records;
  // their uniform vectors in slots u0s (and u1s), by default the block indices
  // c0 / c1 of every level (the linear blocks of sm_model_3d.py:236-239), on stream ls
  // c0[l] and c1[l] in one pass over the level image (their weights are L*82 floats apart), on
  // stream ls with workspace ws
  auto linear_level = [&](int l, cudaStream_t ls, void *ws) -> int {
    const auto &v = P.lv[l];
    const float *im = (l == 0) ? image : P.img[l];
    const float *w0 = linp + (size_t)l * 82;
    return launch_linear_forward_strided(im, v.n1, v.n2, v.n3, w0, (int64_t)L * 82, w0 + 81, (int64_t)L * 82, 2,
                                         P.coef + l, L, nullptr, ws, linear_workspace(), ls);
  };
  auto setup_linear = [&](cudaStream_t ls) -> int {
    for (int l = 0; l < L; ++l) RET_IF(linear_level(l, ls, P.lin_ws));
    return MLPCG_OK;
  };
  bool linear_done = false;
  // gen_level enqueues on gs with the list scratch gl / rl (level 0: the caller's stream and the
  // first lists; the SM kind's levels >= 1: the side stream and the second lists)
  cudaStream_t gs = st;
  uint32_t *gl = P.glist, *rl = P.rlist;
  auto gen_level = [&](int l, const float *im, int b0, void *K0, int b1, void *K1, int u0s = -1,
                       int u1s = -1) -> int {
    const auto &v = P.lv[l];
    if (!v.cls) {
      RET_IF(launch_stencil_gen(im, 0, v.n1, v.n2, v.n3, blk_w(b0), blk_b(b0), K0, P.kdt, v.ps, gs));
      if (b1 >= 0) RET_IF(launch_stencil_gen(im, 0, v.n1, v.n2, v.n3, blk_w(b1), blk_b(b1), K1, P.kdt, v.ps, gs));
      return MLPCG_OK;
    }
    // level 0 (one-hot image): classify also enters each general cell's neighbourhood pattern into
    // the pattern table, whose distinct patterns' coefficients are then evaluated once
    const bool use_pat = l == 0 && P.pkeys && gl == P.glist;
    if (use_pat) {
      MLPCG_CUDA_CHECK(cudaMemsetAsync(P.pkeys, 0xff, (size_t)kPatSlots * sizeof(unsigned long long), gs));
      MLPCG_CUDA_CHECK(cudaMemsetAsync(P.pcount, 0, 2 * sizeof(uint32_t), gs));  // entries used, failure flag
    }
    k_classify<false><<<grid_of(v), PT, 0, gs>>>(im, nullptr, v.n1, v.n2, v.n3, P.cls[l], P.rw[l], P.rcount[l],
                                                 P.gcount[l], use_pat ? P.pkeys : nullptr,
                                                 use_pat ? P.cell_slot : nullptr, use_pat ? P.pcount + 1 : nullptr);
    MLPCG_LAUNCH_CHECK();
    k_scan_tiles<<<1, 1024, 0, gs>>>(P.rcount[l], P.rbase[l], (int)v.ntiles);
    MLPCG_LAUNCH_CHECK();
    k_scan_tiles<<<1, 1024, 0, gs>>>(P.gcount[l], P.gbase[l], (int)v.ntiles);
    MLPCG_LAUNCH_CHECK();
    k_list_general<<<grid_of(v), PT, 0, gs>>>(P.cls[l], v.n1, v.n2, v.n3, P.gbase[l], gl, P.rw[l], P.rbase[l],
                                              rl);
    MLPCG_LAUNCH_CHECK();
    // general cells: one wave of CTAs (as many as fit on every SM), each looping over its share
    const uint32_t *lb = P.gbase[l] + v.ntiles - 1, *lc = P.gcount[l] + v.ntiles - 1;
    if (u0s < 0) u0s = b0;
    if (u1s < 0) u1s = b1 >= 0 ? b1 : b0;
    const float *u0 = P.Uall + (size_t)u0s * 3 * KREC, *u1 = P.Uall + (size_t)u1s * 3 * KREC;
    const int fgrid = (int)std::min<int64_t>((int64_t)sm_count() * 8, (27 * (v.n / 8) + 255) / 256);
    const uint32_t *rlb = P.rbase[l] + v.ntiles - 1, *rlc = P.rcount[l] + v.ntiles - 1;
    // the mixed runs' uniform cells first (whole taps per vector store), then the general cells
    PatternArgs pat{nullptr, nullptr, nullptr, nullptr};
    if (use_pat) {
      const int pgrid = sm_count() * 4;
      if (b1 >= 0)
        k_pattern_coeffs<2><<<pgrid, 256, 0, gs>>>(params, b0, b1, P.pkeys, P.pidx, P.pcount, P.pcoef, P.pcount + 1);
      else
        k_pattern_coeffs<1><<<pgrid, 256, 0, gs>>>(params, b0, b0, P.pkeys, P.pidx, P.pcount, P.pcoef, P.pcount + 1);
      MLPCG_LAUNCH_CHECK();
      pat = PatternArgs{P.cell_slot, P.pidx, P.pcoef, P.pcount + 1};
    }
    auto launch = [&](auto kern, auto fill, const void *r0, const void *r1) {
      using KT = typename std::remove_pointer<decltype(kgen_rec_type(kern))>::type;
      if (pat.cell_slot) {
        const int rgrid = (int)std::min<int64_t>((int64_t)sm_count() * 8, (v.n / 8 + 255) / 256);
        if (b1 >= 0)
          k_fill_runs_pattern<KT, 2><<<rgrid, 256, 0, gs>>>(P.cls[l], rl, rlb, rlc, P.rw[l], P.rbase[l], P.rcount[l],
                                                            v.n2, v.n3, u0, u1, (KT *)r0, (KT *)r1, pat);
        else
          k_fill_runs_pattern<KT, 1><<<rgrid, 256, 0, gs>>>(P.cls[l], rl, rlb, rlc, P.rw[l], P.rbase[l], P.rcount[l],
                                                            v.n2, v.n3, u0, u1, (KT *)r0, (KT *)r1, pat);
      } else {
        fill<<<fgrid, 256, 0, gs>>>(P.cls[l], rl, rlb, rlc, P.rw[l], P.rbase[l], P.rcount[l], v.n2, v.n3, u0, u1,
                                    (KT *)r0, (KT *)r1);
      }
      const int grid = (int)std::min<int64_t>((int64_t)sm_count() * resident_ctas(kern), (v.n + PT - 1) / PT);
      kern<<<grid, PT, 0, gs>>>(im, v.n1, v.n2, v.n3, params, b0, b1 >= 0 ? b1 : b0, gl, lb, lc, P.rw[l],
                                P.rbase[l], P.rcount[l], (KT *)r0, (KT *)r1, pat);
    };
    if (P.kdt == MLPCG_BF16) {
      if (b1 >= 0) launch(k_kgen_list<__nv_bfloat16, 2>, k_fill_runs<__nv_bfloat16, 2>, K0, K1);
      else launch(k_kgen_list<__nv_bfloat16, 1>, k_fill_runs<__nv_bfloat16, 1>, K0, nullptr);
    } else {
      if (b1 >= 0) launch(k_kgen_list<float, 2>, k_fill_runs<float, 2>, K0, K1);
      else launch(k_kgen_list<float, 1>, k_fill_runs<float, 1>, K0, nullptr);
    }
    MLPCG_LAUNCH_CHECK();
    return MLPCG_OK;
  };
  // The transposed blocks of level l.  classify_t: on a classed level, the class map of the
  // neighbourhoods (from the forward class bytes), its tile scans and general-cell / mixed-run
  // lists, shared by every transposed block of the level.  gather_t: the transposed block of
  // forward block (Kf, uniform slot uf) into Kt (slot ut) -- general cells gathered from the
  // forward records, the mixed runs' uniform cells filled; on a dense tiled level the planes
  // gathered; a general-path level applies the forward planes transposed and needs nothing.
  auto classify_t = [&](int l) -> int {
    const auto &v = P.lv[l];
    if (!v.cls) return MLPCG_OK;
    k_classify<true><<<grid_of(v), PT, 0, st>>>(nullptr, P.cls[l], v.n1, v.n2, v.n3, P.clsT[l], P.rwT[l],
                                                P.rcountT[l], P.gcountT[l], nullptr, nullptr, nullptr);
    MLPCG_LAUNCH_CHECK();
    k_scan_tiles<<<1, 1024, 0, st>>>(P.rcountT[l], P.rbaseT[l], (int)v.ntiles);
    MLPCG_LAUNCH_CHECK();
    k_scan_tiles<<<1, 1024, 0, st>>>(P.gcountT[l], P.gbaseT[l], (int)v.ntiles);
    MLPCG_LAUNCH_CHECK();
    k_list_general<<<grid_of(v), PT, 0, st>>>(P.clsT[l], v.n1, v.n2, v.n3, P.gbaseT[l], P.glist, P.rwT[l],
                                              P.rbaseT[l], P.rlist);
    MLPCG_LAUNCH_CHECK();
    return MLPCG_OK;
  };
  auto gather_t = [&](int l, void *Kf, int uf, void *Kt, int ut) -> int {
    const auto &v = P.lv[l];
    if (!v.fast) return MLPCG_OK;
    if (!v.cls) {
      if (P.kdt == MLPCG_BF16)
        k_planes_transpose<__nv_bfloat16><<<blocks_for(v.n, 256), 256, 0, st>>>(
            (const __nv_bfloat16 *)Kf, (__nv_bfloat16 *)Kt, v.ps, v.n1, v.n2, v.n3);
      else
        k_planes_transpose<float><<<blocks_for(v.n, 256), 256, 0, st>>>((const float *)Kf, (float *)Kt, v.ps, v.n1,
                                                                       v.n2, v.n3);
      MLPCG_LAUNCH_CHECK();
      return MLPCG_OK;
    }
    const uint32_t *lb = P.gbaseT[l] + v.ntiles - 1, *lc = P.gcountT[l] + v.ntiles - 1;
    const uint32_t *rlb = P.rbaseT[l] + v.ntiles - 1, *rlc = P.rcountT[l] + v.ntiles - 1;
    const float *kf = P.Uall + (size_t)uf * 3 * KREC, *kt = P.Uall + (size_t)ut * 3 * KREC;
    const int fgrid = (int)std::min<int64_t>((int64_t)sm_count() * 8, (27 * (v.n / 8) + 255) / 256);
    auto launch = [&](auto kern, auto fill, auto *kf_rec, auto *kt_rec) {
      fill<<<fgrid, 256, 0, st>>>(P.clsT[l], P.rlist, rlb, rlc, P.rwT[l], P.rbaseT[l], P.rcountT[l], v.n2, v.n3, kt,
                                  kt, kt_rec, kt_rec);
      const int grid = (int)std::min<int64_t>((int64_t)sm_count() * resident_ctas(kern), (v.n + PT - 1) / PT);
      kern<<<grid, PT, 0, st>>>(v.n1, v.n2, v.n3, P.glist, lb, lc, P.cls[l], P.rw[l], P.rbase[l], P.rcount[l], kf_rec,
                                kf, P.rwT[l], P.rbaseT[l], P.rcountT[l], kt_rec);
    };
    if (P.kdt == MLPCG_BF16)
      launch(k_kgen_t_list<__nv_bfloat16>, k_fill_runs<__nv_bfloat16, 1>, (const __nv_bfloat16 *)Kf,
             (__nv_bfloat16 *)Kt);
    else
      launch(k_kgen_t_list<float>, k_fill_runs<float, 1>, (const float *)Kf, (float *)Kt);
    MLPCG_LAUNCH_CHECK();
    return MLPCG_OK;
  };
  if (P.kind == MLPCG_PRECOND_SMALL_SPD) {
    // l0[l] forward (slot l) and transposed (slot L + l); l forward (slot 2L) and transposed (2L + 1)
    for (int l = 0; l < L; ++l) {
      RET_IF(gen_level(l, (l == 0) ? image : P.img[l], l, P.Kpre[l], -1, nullptr));
      RET_IF(classify_t(l));
      RET_IF(gather_t(l, P.Kpre[l], l, P.Kpost[l], L + l));
    }
    RET_IF(gen_level(L, P.img[L], L, P.Kl, -1, nullptr, 2 * L));
    RET_IF(classify_t(L));
    RET_IF(gather_t(L, P.Kl, 2 * L, P.Klt, 2 * L + 1));
  } else if (side_chain) {
    // the chains of the coarse levels are short and latency-bound: each on a stream of its own
    // (the highest priority, so that their CTAs start as soon as level 0's free a slot)
    const int ns = L + 2;
    if ((int)P.sides.size() != ns) {
      int lo = 0, hi = 0;
      MLPCG_CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      P.sides.assign(ns, nullptr);
      P.img_ev.assign(L + 1, nullptr);
      P.join_evs.assign(ns, nullptr);
      for (int i = 0; i < ns; ++i) {
        MLPCG_CUDA_CHECK(cudaStreamCreateWithPriority(&P.sides[i], cudaStreamNonBlocking, hi));
        MLPCG_CUDA_CHECK(cudaEventCreateWithFlags(&P.join_evs[i], cudaEventDisableTiming));
      }
      for (int l = 0; l <= L; ++l) MLPCG_CUDA_CHECK(cudaEventCreateWithFlags(&P.img_ev[l], cudaEventDisableTiming));
      MLPCG_CUDA_CHECK(cudaEventCreateWithFlags(&P.fork_ev, cudaEventDisableTiming));
    }
    MLPCG_CUDA_CHECK(cudaEventRecord(P.fork_ev, st));
    for (int i = 0; i < ns; ++i) MLPCG_CUDA_CHECK(cudaStreamWaitEvent(P.sides[i], P.fork_ev, 0));
    // the pyramid on sides[0], level by level, each level's image announced
    for (int l = 1; l <= L; ++l) {
      const auto &v = P.lv[l - 1];
      const float *src = (l == 1) ? image : P.img[l - 1];
      RET_IF(launch_avg_pool2(src, P.img[l], MLPCG_F32, 3, v.n1, v.n2, v.n3, P.sides[0]));
      MLPCG_CUDA_CHECK(cudaEventRecord(P.img_ev[l], P.sides[0]));
    }
    // level l's coefficients (and, for l < L, its c0 / c1) on sides[l]
    for (int l = 1; l <= L; ++l) {
      MLPCG_CUDA_CHECK(cudaStreamWaitEvent(P.sides[l], P.img_ev[l], 0));
      gs = P.sides[l];
      gl = P.glists[l];
      rl = P.rlists[l];
      if (l < L) RET_IF(gen_level(l, P.img[l], l, P.Kpre[l], L + l, P.Kpost[l]));
      else RET_IF(gen_level(L, P.img[L], 2 * L, P.Kl, -1, nullptr));
      if (l < L) RET_IF(linear_level(l, P.sides[l], P.lin_wss[l]));
    }
    // level 0's c0 / c1 needs only the caller's image
    RET_IF(linear_level(0, P.sides[L + 1], P.lin_wss[0]));
    for (int i = 0; i < ns; ++i) MLPCG_CUDA_CHECK(cudaEventRecord(P.join_evs[i], P.sides[i]));
    gs = st;
    gl = P.glist;
    rl = P.rlist;
    RET_IF(fluid_mask());
    RET_IF(gen_level(0, image, 0, P.Kpre[0], L, P.Kpost[0]));
    for (int i = 0; i < ns; ++i) MLPCG_CUDA_CHECK(cudaStreamWaitEvent(st, P.join_evs[i], 0));
    linear_done = true;
  } else {
    for (int l = 0; l < L; ++l) RET_IF(gen_level(l, (l == 0) ? image : P.img[l], l, P.Kpre[l], L + l, P.Kpost[l]));
    RET_IF(gen_level(L, P.img[L], 2 * L, P.Kl, -1, nullptr));
    if (P.kind == MLPCG_PRECOND_SPD) {
      // l0[l] (slot l) -> l0_t (slot 2L + 1 + l); l1[l] (slot L + l) -> l1_t (3L + 1 + l); l -> l_t (4L + 1)
      for (int l = 0; l < L; ++l) {
        RET_IF(classify_t(l));
        RET_IF(gather_t(l, P.Kpre[l], l, P.KpreT[l], 2 * L + 1 + l));
        RET_IF(gather_t(l, P.Kpost[l], L + l, P.KpostT[l], 3 * L + 1 + l));
      }
      RET_IF(classify_t(L));
      RET_IF(gather_t(L, P.Kl, 2 * L, P.Klt, 4 * L + 1));
    }
  }
  if (!linear_done) RET_IF(setup_linear(st));
  if (spd) {
    k_square<<<1, 64, 0, st>>>(P.coef, 2 * L);
    MLPCG_LAUNCH_CHECK();
  }
  P.ready = true;
  return MLPCG_OK;
}

int mlpcg_precond_apply(const mlpcg_precond *h, const float *r, const float *r_scale, float *z, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && r && z, MLPCG_ERR_ARG, "precond_apply: NULL argument");
  MLPCG_REQUIRE(((uintptr_t)r & 15) == 0 && ((uintptr_t)z & 31) == 0, MLPCG_ERR_ALIGN,
                "precond_apply: r must be 16-byte and z 32-byte aligned");
  const PrecondPlan &P = h->p;
  MLPCG_REQUIRE(P.ready, MLPCG_ERR_ARG, "precond_apply: plan not set up");
  cudaStream_t st = as_stream(stream);
  void *tmp0 = (char *)P.scratch + al256(96 * sizeof(float));
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_BF16) return run_apply<__nv_bfloat16, __nv_bfloat16>(P, r, r_scale, z, tmp0, st);
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_F32) return run_apply<__nv_bfloat16, float>(P, r, r_scale, z, tmp0, st);
  if (P.kdt == MLPCG_F32 && P.adt == MLPCG_BF16) return run_apply<float, __nv_bfloat16>(P, r, r_scale, z, tmp0, st);
  return run_apply<float, float>(P, r, r_scale, z, tmp0, st);
}

int mlpcg_precond_apply_stages(const mlpcg_precond *h, int first, int last, const float *r, const float *r_scale,
                               float *z, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && r && z, MLPCG_ERR_ARG, "precond_apply_stages: NULL argument");
  MLPCG_REQUIRE(((uintptr_t)r & 15) == 0 && ((uintptr_t)z & 31) == 0, MLPCG_ERR_ALIGN,
                "precond_apply_stages: r must be 16-byte and z 32-byte aligned");
  const PrecondPlan &P = h->p;
  MLPCG_REQUIRE(P.ready, MLPCG_ERR_ARG, "precond_apply_stages: plan not set up");
  const int last_stage = P.kind == MLPCG_PRECOND_SPD ? 4 * P.L + 1 : 2 * P.L;
  MLPCG_REQUIRE(first >= 0 && last <= last_stage && first <= last, MLPCG_ERR_ARG,
                "precond_apply_stages: stage range [%d, %d] outside [0, %d]", first, last, last_stage);
  cudaStream_t st = as_stream(stream);
  void *tmp0 = (char *)P.scratch + al256(96 * sizeof(float));
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_BF16)
    return run_apply<__nv_bfloat16, __nv_bfloat16>(P, r, r_scale, z, tmp0, st, first, last);
  if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_F32) return run_apply<__nv_bfloat16, float>(P, r, r_scale, z, tmp0, st, first, last);
  if (P.kdt == MLPCG_F32 && P.adt == MLPCG_BF16) return run_apply<float, __nv_bfloat16>(P, r, r_scale, z, tmp0, st, first, last);
  return run_apply<float, float>(P, r, r_scale, z, tmp0, st, first, last);
}

static int class_counts(const mlpcg_precond *h, int level, bool transposed, int64_t *general_cells,
                        int64_t *mixed_runs, void *stream) {
  MLPCG_REQUIRE(h && general_cells && mixed_runs && level >= 0 && level <= h->p.L, MLPCG_ERR_ARG,
                "precond_class_counts: bad argument");
  const PrecondPlan &P = h->p;
  MLPCG_REQUIRE(P.ready, MLPCG_ERR_ARG, "precond_class_counts: plan not set up");
  MLPCG_REQUIRE(!transposed || has_transposes(P), MLPCG_ERR_ARG,
                "precond_class_counts_transposed: the plan has no transposed blocks");
  const auto &v = P.lv[level];
  if (!v.cls) {
    *general_cells = *mixed_runs = -1;
    return MLPCG_OK;
  }
  uint32_t last[4] = {0, 0, 0, 0};
  cudaStream_t st = as_stream(stream);
  const uint32_t *src[4] = {P.gbase[level], P.gcount[level], P.rbase[level], P.rcount[level]};
  if (transposed) {
    src[0] = P.gbaseT[level];
    src[1] = P.gcountT[level];
    src[2] = P.rbaseT[level];
    src[3] = P.rcountT[level];
  }
  for (int t = 0; t < 4; ++t)
    MLPCG_CUDA_CHECK(cudaMemcpyAsync(&last[t], src[t] + v.ntiles - 1, 4, cudaMemcpyDeviceToHost, st));
  MLPCG_CUDA_CHECK(cudaStreamSynchronize(st));
  *general_cells = (int64_t)last[0] + last[1];
  *mixed_runs = (int64_t)last[2] + last[3];
  return MLPCG_OK;
}

int mlpcg_precond_class_counts(const mlpcg_precond *h, int level, int64_t *general_cells, int64_t *mixed_runs,
                               void *stream) {
  clear_error();
  return class_counts(h, level, false, general_cells, mixed_runs, stream);
}

int mlpcg_precond_class_counts_transposed(const mlpcg_precond *h, int level, int64_t *general_cells,
                                          int64_t *mixed_runs, void *stream) {
  clear_error();
  return class_counts(h, level, true, general_cells, mixed_runs, stream);
}

int mlpcg_precond_check(const mlpcg_precond *h, int *copy_failed, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && copy_failed && h->p.ready, MLPCG_ERR_ARG, "precond_check: bad argument");
  cudaStream_t st = as_stream(stream);
  int v = 0;
  MLPCG_CUDA_CHECK(cudaMemcpyAsync(&v, h->p.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  MLPCG_CUDA_CHECK(cudaStreamSynchronize(st));
  *copy_failed = v;
  return MLPCG_OK;
}

int mlpcg_precond_set_small_levels(mlpcg_precond *h, int tiles_per_sm) {
  clear_error();
  MLPCG_REQUIRE(h, MLPCG_ERR_ARG, "precond_set_small_levels: NULL plan");
  MLPCG_REQUIRE(tiles_per_sm >= 0 && tiles_per_sm <= 64, MLPCG_ERR_ARG,
                "precond_set_small_levels: tiles_per_sm %d out of [0, 64]", tiles_per_sm);
  h->p.small_tiles_per_sm = tiles_per_sm;
  return MLPCG_OK;
}

int mlpcg_precond_set_coarse_cluster(mlpcg_precond *h, int on) {
  clear_error();
  MLPCG_REQUIRE(h, MLPCG_ERR_ARG, "precond_set_coarse_cluster: NULL plan");
  h->p.coarse_cluster = on != 0;
  return MLPCG_OK;
}

int mlpcg_precond_coarse_cluster(const mlpcg_precond *h, int *first_level, int *ctas) {
  clear_error();
  MLPCG_REQUIRE(h && first_level, MLPCG_ERR_ARG, "precond_coarse_cluster: NULL argument");
  const PrecondPlan &P = h->p;
  int c = 0;
  if (P.kind == MLPCG_PRECOND_SM && P.coarse_cluster) {
    if (P.kdt == MLPCG_BF16 && P.adt == MLPCG_BF16) c = cluster_ctas_for<__nv_bfloat16, __nv_bfloat16>(P);
    else if (P.kdt == MLPCG_BF16) c = cluster_ctas_for<__nv_bfloat16, float>(P);
    else if (P.adt == MLPCG_BF16) c = cluster_ctas_for<float, __nv_bfloat16>(P);
    else c = cluster_ctas_for<float, float>(P);
  }
  *first_level = coarse_cluster_level(P, c);
  if (ctas) *ctas = *first_level > 0 ? c : 0;
  return MLPCG_OK;
}

int mlpcg_precond_set_copy_stall(mlpcg_precond *h, int on, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && h->p.ready, MLPCG_ERR_ARG, "precond_set_copy_stall: plan not set up");
  // clears the copy-failed word and sets (any non-zero byte pattern) or clears the knob
  cudaStream_t st = as_stream(stream);
  MLPCG_CUDA_CHECK(cudaMemsetAsync(h->p.err, 0, sizeof(int), st));
  MLPCG_CUDA_CHECK(cudaMemsetAsync(h->p.err + 1, on ? 1 : 0, sizeof(int), st));
  return MLPCG_OK;
}

int mlpcg_precond_level_info(const mlpcg_precond *h, int level, int *n1, int *n2, int *n3, int *fast) {
  clear_error();
  MLPCG_REQUIRE(h && level >= 0 && level <= h->p.L, MLPCG_ERR_ARG, "precond_level_info: bad level");
  const auto &v = h->p.lv[level];
  if (n1) *n1 = v.n1;
  if (n2) *n2 = v.n2;
  if (n3) *n3 = v.n3;
  if (fast) *fast = v.fast ? 1 : 0;
  return MLPCG_OK;
}

int mlpcg_precond_coefficients(const mlpcg_precond *h, float *c_out, void *stream) {
  clear_error();
  MLPCG_REQUIRE(h && c_out && h->p.ready, MLPCG_ERR_ARG, "precond_coefficients: bad argument");
  MLPCG_CUDA_CHECK(cudaMemcpyAsync(c_out, h->p.coef, 2 * h->p.L * sizeof(float), cudaMemcpyDeviceToDevice,
                                   as_stream(stream)));
  return MLPCG_OK;
}

}  // extern "C"
