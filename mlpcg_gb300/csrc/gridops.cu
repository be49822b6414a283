// Level transfer (restriction / prolongation / combine), the per-level linear
// coefficients (sm_linear_3d) and the matrix-free mixed-boundary Laplacian.
#include "common.cuh"

#include <algorithm>

namespace mlpcg {

// ---------------------------------------------------------------------------
// avg_pool3d(x, 2) and its adjoint.  Sum in (a, b, c) loop order, then / 8.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_avg_pool2(const T *__restrict__ x, T *__restrict__ y, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int c1 = n1 / 2, c2 = n2 / 2, c3 = n3 / 2;
  const int64_t nc = cells(c1, c2, c3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nc) return;
  const int b = blockIdx.y;
  const int k = (int)(q % c3);
  const int64_t t = q / c3;
  const int j = (int)(t % c2);
  const int i = (int)(t / c2);
  const T *xb = x + (int64_t)b * cells(n1, n2, n3);
  float s = 0.f;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int bb = 0; bb < 2; ++bb)
#pragma unroll
      for (int c = 0; c < 2; ++c)
        s += ldf(xb + ((int64_t)(2 * i + a) * n2 + (2 * j + bb)) * n3 + (2 * k + c));
  stf(y + (int64_t)b * nc + q, s / 8.f);
}

template <typename T>
__global__ void k_avg_pool2_adjoint(const T *__restrict__ y, T *__restrict__ x, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int64_t n = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int b = blockIdx.y;
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2);
  const int i = (int)(t / n2);
  const int c2 = n2 / 2, c3 = n3 / 2;
  const int64_t nc = cells(n1 / 2, c2, c3);
  const float v = ldf(y + (int64_t)b * nc + ((int64_t)(i / 2) * c2 + j / 2) * c3 + k / 2);
  stf(x + (int64_t)b * n + q, v / 8.f);
}

// ---------------------------------------------------------------------------
// Trilinear x2 interpolation, align_corners=False (the semantics of
// F.interpolate(scale_factor=2, mode='trilinear')): per axis the source
// coordinate is max(0, 0.5*(f+0.5)-0.5), i0 = floor, i1 = min(i0+1, n-1),
// weights (1-l, l).
// ---------------------------------------------------------------------------
struct Lin1 {
  int i0, i1;
  float l0, l1;
};
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

template <typename T>
__global__ void k_upsample2(const T *__restrict__ x, T *__restrict__ y, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int f1 = 2 * n1, f2 = 2 * n2, f3 = 2 * n3;
  const int64_t nf = cells(f1, f2, f3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nf) return;
  const int b = blockIdx.y;
  const int k = (int)(q % f3);
  const int64_t t = q / f3;
  const int j = (int)(t % f2);
  const int i = (int)(t / f2);
  const Lin1 a = lin1(i, n1), bb = lin1(j, n2), c = lin1(k, n3);
  const T *xb = x + (int64_t)b * cells(n1, n2, n3);
  auto X = [&](int ii, int jj, int kk) { return ldf(xb + ((int64_t)ii * n2 + jj) * n3 + kk); };
  const float v =
      a.l0 * (bb.l0 * (c.l0 * X(a.i0, bb.i0, c.i0) + c.l1 * X(a.i0, bb.i0, c.i1)) +
              bb.l1 * (c.l0 * X(a.i0, bb.i1, c.i0) + c.l1 * X(a.i0, bb.i1, c.i1))) +
      a.l1 * (bb.l0 * (c.l0 * X(a.i1, bb.i0, c.i0) + c.l1 * X(a.i1, bb.i0, c.i1)) +
              bb.l1 * (c.l0 * X(a.i1, bb.i1, c.i0) + c.l1 * X(a.i1, bb.i1, c.i1)));
  stf(y + (int64_t)b * nf + q, v);
}

// Adjoint: each coarse cell gathers the weighted fine values that read it.
// Along one axis, coarse index c is read by fine f in {2c-1, 2c, 2c+1, 2c+2}
// (clamped at the ends); gathering keeps the kernel deterministic.
template <typename T>
__global__ void k_upsample2_adjoint(const T *__restrict__ y, T *__restrict__ x, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int f1 = 2 * n1, f2 = 2 * n2, f3 = 2 * n3;
  const int64_t nc = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nc) return;
  const int b = blockIdx.y;
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2);
  const int i = (int)(t / n2);
  const T *yb = y + (int64_t)b * cells(f1, f2, f3);
  // weights of coarse index c in fine index f along an axis of coarse size n
  auto wt = [](int f, int c, int n) -> float {
    const Lin1 l = lin1(f, n);
    float w = 0.f;
    if (l.i0 == c) w += l.l0;
    if (l.i1 == c) w += l.l1;
    return w;
  };
  float acc = 0.f;
  for (int fi = 2 * i - 1; fi <= 2 * i + 2; ++fi) {
    if (fi < 0 || fi >= f1) continue;
    const float wi = wt(fi, i, n1);
    if (wi == 0.f) continue;
    for (int fj = 2 * j - 1; fj <= 2 * j + 2; ++fj) {
      if (fj < 0 || fj >= f2) continue;
      const float wj = wt(fj, j, n2);
      if (wj == 0.f) continue;
      for (int fk = 2 * k - 1; fk <= 2 * k + 2; ++fk) {
        if (fk < 0 || fk >= f3) continue;
        const float wk = wt(fk, k, n3);
        if (wk == 0.f) continue;
        acc += wi * wj * wk * ldf(yb + ((int64_t)fi * f2 + fj) * f3 + fk);
      }
    }
  }
  stf(x + (int64_t)b * nc + q, acc);
}

// out = c0*x + c1*y, the two products rounded separately like torch's
// c0 * x + c1 * y.
template <typename T>
__global__ void k_axpby(const float *__restrict__ c0, const T *__restrict__ x,
                        const float *__restrict__ c1, const T *__restrict__ y, T *__restrict__ out,
                        int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float a = __fmul_rn(c0[0], ldf(x + q));
  const float b = __fmul_rn(c1[0], ldf(y + q));
  stf(out + q, __fadd_rn(a, b));
}

// ---------------------------------------------------------------------------
// sm_linear_3d: the 81 shifted means of the 3 image channels.
// Every cell belongs to one of 27 boundary classes (per axis: first plane,
// interior, last plane).  Each shifted sum is a sum of class sums, so one
// pass computes 27 x 3 class sums and the 81 shifted sums follow by
// inclusion (deterministic: per-block FP64 partials summed in fixed order).
// ---------------------------------------------------------------------------
constexpr int kLinBlocks = 1216;
constexpr int kLinThreads = 256;
constexpr int kLinWarps = kLinThreads / 32;

// boundary class of coordinate c on an axis of n cells: first plane 0,
// interior 1, last plane 2 (a single plane is class 0)
__device__ __forceinline__ int axis_class(int c, int n) { return c == 0 ? 0 : (c == n - 1 ? 2 : 1); }

// Per-block partial sums (double-float pairs) of the 3 image channels over
// each of the 27 classes.  Warps take whole z-rows (i, j), which share the
// row class (x class, y class); a lane sums its cells by z class in FP32
// across the rows of one row class, and the sums go through a double-float
// warp reduction into the warp's slots whenever the row class changes.
// Deterministic: the row assignment and every reduction order are fixed.
__global__ void __launch_bounds__(kLinThreads)
k_class_sums(const float *__restrict__ img, int n1, int n2, int n3, float2 *__restrict__ partial) {
  dependent_launch_enter();
  __shared__ float2 ws[kLinWarps][81];  // per warp: (class * 3 + channel)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int e = lane; e < 81; e += 32) ws[w][e] = make_float2(0.f, 0.f);
  __syncwarp();
  const int64_t n = cells(n1, n2, n3);
  const int64_t rows = (int64_t)n1 * n2;
  const bool vec = (n3 % 4) == 0 && ((uintptr_t)img & 15) == 0;
  float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // [channel][z class]
  int key = -1;  // current row class (x class * 3 + y class), warp-uniform
  auto flush = [&]() {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int cz = 0; cz < 3; ++cz) {
        float2 d = make_float2(a[ch][cz], 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d = df_add(d, df_shfl_xor(d, o));
        if (lane == 0) ws[w][(key * 3 + cz) * 3 + ch] = df_add(ws[w][(key * 3 + cz) * 3 + ch], d);
        a[ch][cz] = 0.f;
      }
  };
  auto add = [&](int k, float v0, float v1, float v2) {
    const int cz = axis_class(k, n3);
    if (cz == 1) { a[0][1] += v0; a[1][1] += v1; a[2][1] += v2; }
    else if (cz == 0) { a[0][0] += v0; a[1][0] += v1; a[2][0] += v2; }
    else { a[0][2] += v0; a[1][2] += v1; a[2][2] += v2; }
  };
  for (int64_t r = (int64_t)blockIdx.x * kLinWarps + w; r < rows; r += (int64_t)gridDim.x * kLinWarps) {
    const int i = (int)(r / n2), j = (int)(r % n2);
    const int nk = axis_class(i, n1) * 3 + axis_class(j, n2);
    if (nk != key) {
      if (key >= 0) flush();
      key = nk;
    }
    const float *p = img + r * n3;
    if (vec) {
      for (int k = 4 * lane; k < n3; k += 128) {
        const float4 x0 = __ldg(reinterpret_cast<const float4 *>(p + k));
        const float4 x1 = __ldg(reinterpret_cast<const float4 *>(p + n + k));
        const float4 x2 = __ldg(reinterpret_cast<const float4 *>(p + 2 * n + k));
        add(k, x0.x, x1.x, x2.x);
        add(k + 1, x0.y, x1.y, x2.y);
        add(k + 2, x0.z, x1.z, x2.z);
        add(k + 3, x0.w, x1.w, x2.w);
      }
    } else {
      for (int k = lane; k < n3; k += 32) add(k, __ldg(p + k), __ldg(p + n + k), __ldg(p + 2 * n + k));
    }
  }
  if (key >= 0) flush();
  __syncthreads();
  if (threadIdx.x < 81) {
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int ww = 0; ww < kLinWarps; ++ww) s = df_add(s, ws[ww][threadIdx.x]);
    partial[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = s;
  }
}

// One block of 1024 threads: class sums -> 81 shifted means y -> nlin outputs z.
// Output j uses weights W + j*wstride (81 values), bias[j*bstride], and goes to z[j*zstride].
// cs[c] (c = cls * 3 + channel) = the sum of the blocks' partials of value c: one CTA per value,
// double-float, in a fixed order (thread t takes blocks t, t + 256, ..., then a fixed tree).
__global__ void __launch_bounds__(256) k_linear_reduce(const float2 *__restrict__ partial, int nblk,
                                                       double *__restrict__ cs) {
  dependent_launch_enter();
  __shared__ float2 ws[8];
  const int c = blockIdx.x, t = threadIdx.x;
  float2 v[(kLinBlocks + 255) / 256];
#pragma unroll
  for (int u = 0; u < (kLinBlocks + 255) / 256; ++u) {
    const int b = t + 256 * u;
    v[u] = b < nblk ? partial[(int64_t)c * nblk + b] : make_float2(0.f, 0.f);
  }
  float2 s = v[0];
#pragma unroll
  for (int u = 1; u < (kLinBlocks + 255) / 256; ++u) s = df_add(s, v[u]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
  if ((t & 31) == 0) ws[t >> 5] = s;
  __syncthreads();
  if (t == 0) {
    float2 a = ws[0];
    for (int w = 1; w < 8; ++w) a = df_add(a, ws[w]);
    cs[c] = df_to_double(a);
  }
}

__global__ void k_linear_finalize(const double *__restrict__ cs_g, int n1, int n2, int n3,
                                  const float *__restrict__ W, int64_t wstride, const float *__restrict__ bias,
                                  int64_t bstride, int nlin, float *__restrict__ z, int64_t zstride,
                                  float *__restrict__ yout) {
  dependent_launch_enter();
  __shared__ double cs[27 * 3];
  __shared__ double ym[81];
  const int t = threadIdx.x;
  if (t < 81) cs[t] = cs_g[t];
  __syncthreads();
  // shift index k in {0,1,2} (offset k-1) keeps classes: k=0 -> {0,1}, k=1 -> all, k=2 -> {1,2};
  // for an axis of size 1 the single plane is class 0 and only k=1 keeps it.
  auto keep = [](int k, int cls, int n) -> bool {
    if (n == 1) return k == 1 && cls == 0;
    if (k == 0) return cls != 2;
    if (k == 2) return cls != 0;
    return true;
  };
  const double inv_n = 1.0 / (double)cells(n1, n2, n3);
  if (t < 81) {
    const int s = t / 27, kk = (t / 9) % 3, ll = (t / 3) % 3, oo = t % 3;
    double acc = 0.0;
    for (int cx = 0; cx < 3; ++cx) {
      if (!keep(kk, cx, n1)) continue;
      for (int cy = 0; cy < 3; ++cy) {
        if (!keep(ll, cy, n2)) continue;
        for (int cz = 0; cz < 3; ++cz) {
          if (!keep(oo, cz, n3)) continue;
          acc += cs[(cx * 9 + cy * 3 + cz) * 3 + s];
        }
      }
    }
    ym[t] = acc * inv_n;
    if (yout) yout[t] = (float)(acc * inv_n);
  }
  __syncthreads();
  // z_j = w_j . y + b_j   (w . y in float like the reference's dot, then + bias)
  if (t < nlin) {
    double acc = 0.0;
    for (int e = 0; e < 81; ++e) acc += (double)W[t * wstride + e] * ym[e];
    z[t * zstride] = (float)(acc + (double)bias[t * bstride]);
  }
}

__global__ void k_linear_backward(const float *__restrict__ g, const float *__restrict__ y,
                                  float *__restrict__ gw, float *__restrict__ gb) {
  dependent_launch_enter();
  const int t = threadIdx.x;
  if (t < 81) gw[t] = y[t] * g[0];
  if (t == 0) gb[0] = g[0];
}

// d z / d img(s, c) = g/N * sum over shifts d with c - d in grid of w[s][d]
__global__ void k_linear_image_grad(const float *__restrict__ g, const float *__restrict__ W, int n1,
                                    int n2, int n3, float *__restrict__ gimg) {
  dependent_launch_enter();
  const int64_t n = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2);
  const int i = (int)(t / n2);
  const float scale = g[0] / (float)n;
  for (int s = 0; s < 3; ++s) {
    float acc = 0.f;
    for (int o = 0; o < 27; ++o) {
      // y[s][o] sums img(q + d_o) over q in grid: img cell c is counted iff c - d_o in grid
      const int ii = i - (o / 9 - 1), jj = j - ((o / 3) % 3 - 1), kk = k - (o % 3 - 1);
      if ((unsigned)ii < (unsigned)n1 && (unsigned)jj < (unsigned)n2 && (unsigned)kk < (unsigned)n3)
        acc += W[s * 27 + o];
    }
    gimg[s * n + q] = acc * scale;
  }
}

// ---------------------------------------------------------------------------
// Matrix-free mixed-boundary 7-point operator.  Neighbours are visited in
// the column order of the assembled CSR row (i-1, j-1, k-1, centre, k+1,
// j+1, i+1).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_laplacian(const uint8_t *__restrict__ flags, const T *__restrict__ x,
                            T *__restrict__ y, int n1, int n2, int n3) {
  dependent_launch_enter();
  const int64_t n = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (flags[q] != MLPCG_FLUID) { y[q] = T(0); return; }
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2);
  const int i = (int)(t / n2);
  const int64_t sx = (int64_t)n2 * n3, sy = n3;
  T off = T(0);
  int d = 0;
  auto visit = [&](bool inside, int64_t nb) {
    if (!inside) return;
    const uint8_t f = flags[nb];
    if (f == MLPCG_FLUID) { off += x[nb]; ++d; }
    else if (f == MLPCG_AIR) { ++d; }
  };
  visit(i > 0, q - sx);
  visit(j > 0, q - sy);
  visit(k > 0, q - 1);
  visit(k < n3 - 1, q + 1);
  visit(j < n2 - 1, q + sy);
  visit(i < n1 - 1, q + sx);
  y[q] = T(d) * x[q] - off;
}

// [air, fluid, non-solid] channels from flag codes
__global__ void k_flags_to_image(const uint8_t *__restrict__ flags, float *__restrict__ img, int64_t n) {
  dependent_launch_enter();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint8_t f = flags[q];
  img[q] = f == MLPCG_AIR ? 1.f : 0.f;
  img[n + q] = f == MLPCG_FLUID ? 1.f : 0.f;
  img[2 * n + q] = f > MLPCG_SOLID ? 1.f : 0.f;
}

// ---------------------------------------------------------------------------
// Fluid-DOF vectors: the values of the fluid cells in flat cell order (the
// reference's compressed solver vectors).  Cells are taken in blocks of
// kFluidBlock; block_base[b] = number of fluid cells before block b, and a
// cell's position is its block's base plus its rank among the block's fluid
// cells (recomputed by a block scan in each pass).
// ---------------------------------------------------------------------------
constexpr int kFluidThreads = 256, kFluidPer = 4, kFluidBlock = kFluidThreads * kFluidPer;
// CTAs per SM of a scatter whose values are read from host memory
constexpr int kHostScatterCtasPerSm = 2;

// exclusive scan of one int per thread over a 256-thread block
__device__ __forceinline__ int block256_excl_scan(int v, int &total) {
  __shared__ int ws[kFluidThreads / 32];
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
  for (int i = 0; i < kFluidThreads / 32; ++i) {
    if (i < w) off += ws[i];
    tot += ws[i];
  }
  total = tot;
  return off + x - v;
}

// fluid bits of the thread's kFluidPer cells
__device__ __forceinline__ unsigned fluid_bits(const uint8_t *__restrict__ flags, int64_t n, int64_t q0) {
  unsigned m = 0;
#pragma unroll
  for (int u = 0; u < kFluidPer; ++u)
    if (q0 + u < n && flags[q0 + u] == MLPCG_FLUID) m |= 1u << u;
  return m;
}

__global__ void __launch_bounds__(kFluidThreads)
k_fluid_counts(const uint8_t *__restrict__ flags, int64_t n, uint32_t *__restrict__ cnt) {
  dependent_launch_enter();
  const int64_t q0 = (int64_t)blockIdx.x * kFluidBlock + kFluidPer * threadIdx.x;
  int tot;
  block256_excl_scan(__popc(fluid_bits(flags, n, q0)), tot);
  if (threadIdx.x == 0) cnt[blockIdx.x] = (uint32_t)tot;
}

// grid = the fluid values scattered to their cells, 0 elsewhere (and for
// positions beyond the m values given).  A block's values are one contiguous
// range of vals: the block reads it with consecutive lanes on consecutive
// values into shared memory (few, full transactions also when vals is host
// memory read over the host link), then places them.  Blocks step through the
// cell blocks by the grid size, so that a scatter from host memory can run on
// a few CTAs per SM beside other work: its speed is the host link's, and a
// full grid would hold every SM while its loads wait on the link.
__global__ void __launch_bounds__(kFluidThreads)
k_scatter_fluid(const double *__restrict__ vals, int64_t m, const uint8_t *__restrict__ flags,
                const uint32_t *__restrict__ base, int64_t n, double *__restrict__ grid) {
  dependent_launch_enter();
  __shared__ double sv[kFluidBlock];
  const int64_t nb = (n + kFluidBlock - 1) / kFluidBlock;
  for (int64_t blk = blockIdx.x; blk < nb; blk += gridDim.x) {
    const int64_t q0 = blk * kFluidBlock + kFluidPer * threadIdx.x;
    const unsigned fm = fluid_bits(flags, n, q0);
    int tot;
    const int64_t b0 = (int64_t)__ldg(base + blk);
    // the scan's barrier also orders this block's sv writes after the previous pass's reads
    int pos = block256_excl_scan(__popc(fm), tot);
    for (int i = threadIdx.x; i < tot; i += kFluidThreads) sv[i] = b0 + i < m ? vals[b0 + i] : 0.0;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kFluidPer; ++u)
      if (q0 + u < n) {
        const bool f = (fm >> u) & 1u;
        grid[q0 + u] = f ? sv[pos] : 0.0;
        pos += f;
      }
  }
}

// vals = the grid's values on the fluid cells (the first m of them), placed in
// shared memory first so that the block writes its contiguous range of vals
// with consecutive lanes on consecutive values (full transactions also when
// vals is host memory written over the host link)
__global__ void __launch_bounds__(kFluidThreads)
k_gather_fluid(const double *__restrict__ grid, const uint8_t *__restrict__ flags,
               const uint32_t *__restrict__ base, int64_t n, double *__restrict__ vals, int64_t m) {
  dependent_launch_enter();
  __shared__ double sv[kFluidBlock];
  const int64_t q0 = (int64_t)blockIdx.x * kFluidBlock + kFluidPer * threadIdx.x;
  const unsigned fm = fluid_bits(flags, n, q0);
  int tot;
  const int64_t b0 = (int64_t)__ldg(base + blockIdx.x);
  int pos = block256_excl_scan(__popc(fm), tot);
#pragma unroll
  for (int u = 0; u < kFluidPer; ++u)
    if ((fm >> u) & 1u) sv[pos++] = grid[q0 + u];
  __syncthreads();
  for (int i = threadIdx.x; i < tot && b0 + i < m; i += kFluidThreads) vals[b0 + i] = sv[i];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_flags_to_image(const uint8_t *flags, float *img, int64_t n, cudaStream_t st) {
  k_flags_to_image<<<blocks_for(n, 256), 256, 0, st>>>(flags, img, n);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

#define MLPCG_DISPATCH_DT(dt, T, ...)                                   \
  do {                                                                  \
    if ((dt) == MLPCG_F32) { using T = float; __VA_ARGS__; }            \
    else if ((dt) == MLPCG_BF16) { using T = __nv_bfloat16; __VA_ARGS__; } \
    else { using T = double; __VA_ARGS__; }                             \
  } while (0)

int launch_scan_u32(const uint32_t *cnt, uint32_t *base, int n, cudaStream_t st);  // precond.cu

int64_t fluid_blocks(int64_t n) { return (n + kFluidBlock - 1) / kFluidBlock; }

int launch_fluid_order(const uint8_t *flags, int64_t n, uint32_t *base, cudaStream_t st) {
  const int64_t nb = fluid_blocks(n);
  MLPCG_REQUIRE(nb < (1ll << 31), MLPCG_ERR_SHAPE, "fluid_order: too many cells");
  uint32_t *cnt = base + nb;  // second half of the caller's array
  k_fluid_counts<<<(unsigned)nb, kFluidThreads, 0, st>>>(flags, n, cnt);
  MLPCG_LAUNCH_CHECK();
  return launch_scan_u32(cnt, base, (int)nb, st);
}

int launch_scatter_fluid(const double *vals, int64_t m, const uint8_t *flags, const uint32_t *base, int64_t n,
                         double *grid, cudaStream_t st) {
  int64_t blocks = fluid_blocks(n);
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, vals);
  if (e != cudaSuccess) cudaGetLastError();
  if (e == cudaSuccess && a.type == cudaMemoryTypeHost) {  // read over the host link: a few CTAs per SM
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
      sms = 152;
    blocks = std::min<int64_t>(blocks, (int64_t)kHostScatterCtasPerSm * sms);
  }
  k_scatter_fluid<<<(unsigned)blocks, kFluidThreads, 0, st>>>(vals, m, flags, base, n, grid);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_gather_fluid(const double *grid, const uint8_t *flags, const uint32_t *base, int64_t n, double *vals,
                        int64_t m, cudaStream_t st) {
  k_gather_fluid<<<(unsigned)fluid_blocks(n), kFluidThreads, 0, st>>>(grid, flags, base, n, vals, m);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_avg_pool2(const void *x, void *y, int dt, int B, int n1, int n2, int n3, cudaStream_t st) {
  dim3 grid(blocks_for(cells(n1 / 2, n2 / 2, n3 / 2), 256), B);
  MLPCG_DISPATCH_DT(dt, T, k_avg_pool2<T><<<grid, 256, 0, st>>>((const T *)x, (T *)y, n1, n2, n3));
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_avg_pool2_adjoint(const void *y, void *x, int dt, int B, int n1, int n2, int n3,
                             cudaStream_t st) {
  dim3 grid(blocks_for(cells(n1, n2, n3), 256), B);
  MLPCG_DISPATCH_DT(dt, T, k_avg_pool2_adjoint<T><<<grid, 256, 0, st>>>((const T *)y, (T *)x, n1, n2, n3));
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_upsample2(const void *x, void *y, int dt, int B, int n1, int n2, int n3, cudaStream_t st) {
  dim3 grid(blocks_for(cells(2 * n1, 2 * n2, 2 * n3), 256), B);
  MLPCG_DISPATCH_DT(dt, T, k_upsample2<T><<<grid, 256, 0, st>>>((const T *)x, (T *)y, n1, n2, n3));
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_upsample2_adjoint(const void *y, void *x, int dt, int B, int n1, int n2, int n3,
                             cudaStream_t st) {
  dim3 grid(blocks_for(cells(n1, n2, n3), 256), B);
  MLPCG_DISPATCH_DT(dt, T, k_upsample2_adjoint<T><<<grid, 256, 0, st>>>((const T *)y, (T *)x, n1, n2, n3));
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_axpby(const float *c0, const void *x, const float *c1, const void *y, void *out, int dt,
                 int64_t n, cudaStream_t st) {
  MLPCG_DISPATCH_DT(dt, T, k_axpby<T><<<blocks_for(n, 256), 256, 0, st>>>(c0, (const T *)x, c1,
                                                                            (const T *)y, (T *)out, n));
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

// the blocks' partials (81 x kLinBlocks double-float pairs), then the 81 reduced sums (FP64)
size_t linear_workspace() { return (size_t)27 * 3 * kLinBlocks * sizeof(float2) + 81 * sizeof(double); }

int launch_linear_forward_strided(const float *img, int n1, int n2, int n3, const float *W, int64_t wstride,
                                  const float *bias, int64_t bstride, int nlin, float *z, int64_t zstride, float *y,
                                  void *ws, size_t ws_bytes, cudaStream_t st) {
  MLPCG_REQUIRE(ws_bytes >= linear_workspace(), MLPCG_ERR_WORKSPACE,
                "sm_linear_3d workspace too small: %zu < %zu", ws_bytes, linear_workspace());
  k_class_sums<<<kLinBlocks, kLinThreads, 0, st>>>(img, n1, n2, n3, (float2 *)ws);
  MLPCG_LAUNCH_CHECK();
  double *cs = reinterpret_cast<double *>((char *)ws + (size_t)27 * 3 * kLinBlocks * sizeof(float2));
  k_linear_reduce<<<81, 256, 0, st>>>((const float2 *)ws, kLinBlocks, cs);
  MLPCG_LAUNCH_CHECK();
  k_linear_finalize<<<1, 128, 0, st>>>(cs, n1, n2, n3, W, wstride, bias, bstride, nlin, z, zstride, y);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_linear_forward(const float *img, int n1, int n2, int n3, const float *W, const float *bias,
                          int nlin, float *z, float *y, void *ws, size_t ws_bytes, cudaStream_t st) {
  return launch_linear_forward_strided(img, n1, n2, n3, W, 81, bias, 1, nlin, z, 1, y, ws, ws_bytes, st);
}

int launch_linear_backward(const float *g, const float *y, float *gw, float *gb, cudaStream_t st) {
  k_linear_backward<<<1, 96, 0, st>>>(g, y, gw, gb);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_linear_image_grad(const float *g, const float *W, float *gimg, int n1, int n2, int n3,
                             cudaStream_t st) {
  k_linear_image_grad<<<blocks_for(cells(n1, n2, n3), 256), 256, 0, st>>>(g, W, n1, n2, n3, gimg);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_laplacian(const uint8_t *flags, const void *x, void *y, int dt, int n1, int n2, int n3,
                     cudaStream_t st) {
  const int64_t n = cells(n1, n2, n3);
  if (dt == MLPCG_F32)
    k_laplacian<float><<<blocks_for(n, 256), 256, 0, st>>>(flags, (const float *)x, (float *)y, n1, n2, n3);
  else if (dt == MLPCG_F64)
    k_laplacian<double><<<blocks_for(n, 256), 256, 0, st>>>(flags, (const double *)x, (double *)y, n1, n2, n3);
  else {
    set_error("laplacian: dtype must be F32 or F64");
    return MLPCG_ERR_UNSUPPORTED;
  }
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

}  // namespace mlpcg
