// Per-cell stencil coefficients (K) and their application.
//
// The reference's sm_block_3d kernels evaluate, for every output cell and on
// every call, 27 coefficients K_p = bias_p + (3->27 3x3x3 conv of the image)
// and then y = sum_p K_p x(q+off_p)  (torch_extension/sm_block_3d_kernel.cu:45-70).
// Here the two halves are separate kernels: K is generated once per
// (image, weights) into 27 planes, and the application is a bandwidth-bound
// 27-coefficient variable stencil.  The kernels in this file are the general
// ones (any size, padded or unpadded inputs, any batch); the fused solve
// path uses the tiled kernels of precond.cu.
#include "common.cuh"

namespace mlpcg {

// ---------------------------------------------------------------------------
// K generation
// ---------------------------------------------------------------------------
// sW[so][p] holds weight[p][so] (so = s*27 + tap of the image patch) with p
// padded to 28 so that one (s,o) row is seven float4 loads.  All threads of a
// warp read the same row: a shared-memory broadcast.
constexpr int kGenThreads = 128;

template <typename KT>
__global__ void __launch_bounds__(kGenThreads)
k_stencil_gen(const float *__restrict__ img, FieldGeom g, const float *__restrict__ W,
              const float *__restrict__ bias, KT *__restrict__ K, int64_t ps) {
  dependent_launch_enter();
  __shared__ float4 sW[kSW];
  __shared__ float4 sWm[kSW];
  __shared__ float sb[28];
  load_weights_smem(W, bias, sW, sWm, sb);
  __syncthreads();

  const int64_t n = cells(g.n1, g.n2, g.n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int k = (int)(q % g.n3);
  const int64_t t = q / g.n3;
  const int j = (int)(t % g.n2);
  const int i = (int)(t / g.n2);

  float acc[28];
  coeffs_of_patch(sW, sWm, sb, [&](int s, int m, int nn, int o) {
    return g.at(img + s * g.bstride, i + m - 1, j + nn - 1, k + o - 1);
  }, acc);
#pragma unroll
  for (int p = 0; p < 27; ++p) stf(K + p * ps + q, acc[p]);
}

// ---------------------------------------------------------------------------
// K application, forward and transposed (general kernel: one thread per
// output cell, blockIdx.y = batch item)
// ---------------------------------------------------------------------------
template <typename KT, typename XT, typename YT, bool TRANS>
__global__ void __launch_bounds__(256)
k_stencil_apply(const KT *__restrict__ K, int64_t ps, const XT *__restrict__ x, FieldGeom gx,
                YT *__restrict__ y) {
  dependent_launch_enter();
  const int64_t n = cells(gx.n1, gx.n2, gx.n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int b = blockIdx.y;
  const int k = (int)(q % gx.n3);
  const int64_t t = q / gx.n3;
  const int j = (int)(t % gx.n2);
  const int i = (int)(t / gx.n2);
  const XT *xb = x + b * gx.bstride;
  float acc = 0.f;
#pragma unroll
  for (int p = 0; p < 27; ++p) {
    const int di = tap_dx(p), dj = tap_dy(p), dk = tap_dz(p);
    if (!TRANS) {
      acc = fmaf(ldf(K + p * ps + q), gx.at(xb, i + di, j + dj, k + dk), acc);
    } else {
      const int ii = i - di, jj = j - dj, kk = k - dk;
      if ((unsigned)ii < (unsigned)gx.n1 && (unsigned)jj < (unsigned)gx.n2 &&
          (unsigned)kk < (unsigned)gx.n3) {
        const int64_t qs = ((int64_t)ii * gx.n2 + jj) * gx.n3 + kk;
        acc = fmaf(ldf(K + p * ps + qs), gx.at(xb, ii, jj, kk), acc);
      }
    }
  }
  stf(y + (int64_t)b * n + q, acc);
}

// ---------------------------------------------------------------------------
// dK (coefficient gradient, summed over the batch)
// ---------------------------------------------------------------------------
template <bool TRANS>
__global__ void __launch_bounds__(256)
k_coeff_grad(const float *__restrict__ g, const float *__restrict__ x, FieldGeom gx, int B,
             float *__restrict__ dK, int64_t ps) {
  dependent_launch_enter();
  const int64_t n = cells(gx.n1, gx.n2, gx.n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int k = (int)(q % gx.n3);
  const int64_t t = q / gx.n3;
  const int j = (int)(t % gx.n2);
  const int i = (int)(t / gx.n2);
  float acc[27];
#pragma unroll
  for (int p = 0; p < 27; ++p) acc[p] = 0.f;
  for (int b = 0; b < B; ++b) {
    const float *xb = x + b * gx.bstride;
    const float *gb = g + b * n;
    if (!TRANS) {
      const float gv = gb[q];
#pragma unroll
      for (int p = 0; p < 27; ++p)
        acc[p] = fmaf(gv, gx.at(xb, i + tap_dx(p), j + tap_dy(p), k + tap_dz(p)), acc[p]);
    } else {
      const float xv = gx.at(xb, i, j, k);
#pragma unroll
      for (int p = 0; p < 27; ++p) {
        const int ii = i + tap_dx(p), jj = j + tap_dy(p), kk = k + tap_dz(p);
        float gv = 0.f;
        if ((unsigned)ii < (unsigned)gx.n1 && (unsigned)jj < (unsigned)gx.n2 &&
            (unsigned)kk < (unsigned)gx.n3)
          gv = gb[((int64_t)ii * gx.n2 + jj) * gx.n3 + kk];
        acc[p] = fmaf(gv, xv, acc[p]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < 27; ++p) dK[p * ps + q] = acc[p];
}

// ---------------------------------------------------------------------------
// dW / db: grad_w[p][so] = sum_q dK_p(q) * patch_so(q),  grad_b[p] = sum_q dK_p(q)
// Block = 256 threads; tile of kWgTile cells staged in shared memory; each
// thread owns a 3 (p) x 3 (column) register tile of the 27 x 84 output
// (columns: 81 image taps, 1 bias column of ones, 2 zero pads).  FP32 within
// a tile, FP64 across tiles; one FP64 partial row per block, summed in a fixed
// order by k_wgrad_finalize (deterministic).
// ---------------------------------------------------------------------------
constexpr int kWgTile = 64;
constexpr int kWgCols = 84;
constexpr int kWgBlocksMax = 608;  // 4 x 152 SMs
constexpr int kWgOut = 27 * kWgCols;

__global__ void __launch_bounds__(256)
k_wgrad_partial(const float *__restrict__ dK, int64_t ps, const float *__restrict__ img,
                FieldGeom g, double *__restrict__ partial) {
  dependent_launch_enter();
  __shared__ float sdK[27][kWgTile];
  __shared__ float sP[kWgCols][kWgTile];
  const int64_t n = cells(g.n1, g.n2, g.n3);
  const int tid = threadIdx.x;
  const int tp = tid / 28;        // 0..8  (p tile), tid 252..255 idle in compute
  const int tc = tid % 28;        // 0..27 (column tile)
  const bool active = tid < 252;
  double accd[9];
#pragma unroll
  for (int r = 0; r < 9; ++r) accd[r] = 0.0;

  for (int64_t base = (int64_t)blockIdx.x * kWgTile; base < n; base += (int64_t)gridDim.x * kWgTile) {
    __syncthreads();
    // stage dK and patches of kWgTile cells
    for (int e = tid; e < 27 * kWgTile; e += blockDim.x) {
      const int p = e / kWgTile, c = e % kWgTile;
      const int64_t q = base + c;
      sdK[p][c] = q < n ? dK[p * ps + q] : 0.f;
    }
    for (int e = tid; e < kWgCols * kWgTile; e += blockDim.x) {
      const int col = e / kWgTile, c = e % kWgTile;
      const int64_t q = base + c;
      float v = 0.f;
      if (q < n) {
        if (col < 81) {
          const int s = col / 27, o = col % 27;
          const int k = (int)(q % g.n3);
          const int64_t t = q / g.n3;
          const int j = (int)(t % g.n2);
          const int i = (int)(t / g.n2);
          v = g.at(img + s * g.bstride, i + o / 9 - 1, j + (o / 3) % 3 - 1, k + o % 3 - 1);
        } else if (col == 81) {
          v = 1.f;
        }
      }
      sP[col][c] = v;
    }
    __syncthreads();
    if (active) {
      float acc[9];
#pragma unroll
      for (int r = 0; r < 9; ++r) acc[r] = 0.f;
#pragma unroll 4
      for (int c = 0; c < kWgTile; ++c) {
        const float d0 = sdK[tp * 3 + 0][c], d1 = sdK[tp * 3 + 1][c], d2 = sdK[tp * 3 + 2][c];
        const float p0 = sP[tc * 3 + 0][c], p1 = sP[tc * 3 + 1][c], p2 = sP[tc * 3 + 2][c];
        acc[0] = fmaf(d0, p0, acc[0]); acc[1] = fmaf(d0, p1, acc[1]); acc[2] = fmaf(d0, p2, acc[2]);
        acc[3] = fmaf(d1, p0, acc[3]); acc[4] = fmaf(d1, p1, acc[4]); acc[5] = fmaf(d1, p2, acc[5]);
        acc[6] = fmaf(d2, p0, acc[6]); acc[7] = fmaf(d2, p1, acc[7]); acc[8] = fmaf(d2, p2, acc[8]);
      }
#pragma unroll
      for (int r = 0; r < 9; ++r) accd[r] += (double)acc[r];
    }
  }
  if (active) {
    double *row = partial + (int64_t)blockIdx.x * kWgOut;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) row[(tp * 3 + a) * kWgCols + tc * 3 + c] = accd[a * 3 + c];
  }
}

__global__ void k_wgrad_finalize(const double *__restrict__ partial, int nblk,
                                 float *__restrict__ gw, float *__restrict__ gb) {
  dependent_launch_enter();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 27 * 82) return;
  const int p = e / 82, col = e % 82;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += partial[(int64_t)b * kWgOut + p * kWgCols + col];
  if (col < 81) gw[p * 81 + col] = (float)s;
  else gb[p] = (float)s;
}

// ---------------------------------------------------------------------------
// d image: grad_img(s, c) = sum_p sum_o W[p][s][o] dK_p(c - (o - 1))
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
k_image_grad(const float *__restrict__ dK, int64_t ps, const float *__restrict__ W, int n1,
             int n2, int n3, float *__restrict__ gimg) {
  dependent_launch_enter();
  __shared__ float sW[27 * 81];
  for (int t = threadIdx.x; t < 27 * 81; t += blockDim.x) sW[t] = W[t];
  __syncthreads();
  const int64_t n = cells(n1, n2, n3);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int k = (int)(q % n3);
  const int64_t t = q / n3;
  const int j = (int)(t % n2);
  const int i = (int)(t / n2);
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  for (int o = 0; o < 27; ++o) {
    const int ii = i - (o / 9 - 1), jj = j - ((o / 3) % 3 - 1), kk = k - (o % 3 - 1);
    if ((unsigned)ii >= (unsigned)n1 || (unsigned)jj >= (unsigned)n2 || (unsigned)kk >= (unsigned)n3)
      continue;
    const int64_t qs = ((int64_t)ii * n2 + jj) * n3 + kk;
#pragma unroll 9
    for (int p = 0; p < 27; ++p) {
      const float d = __ldg(dK + p * ps + qs);
      a0 = fmaf(sW[p * 81 + 0 * 27 + o], d, a0);
      a1 = fmaf(sW[p * 81 + 1 * 27 + o], d, a1);
      a2 = fmaf(sW[p * 81 + 2 * 27 + o], d, a2);
    }
  }
  gimg[q] = a0;
  gimg[n + q] = a1;
  gimg[2 * n + q] = a2;
}

// ---------------------------------------------------------------------------
// host launchers (used by capi.cu and precond.cu)
// ---------------------------------------------------------------------------
int launch_stencil_gen(const float *image, int image_padded, int n1, int n2, int n3,
                       const float *W, const float *bias, void *K, int kdt, int64_t ps,
                       cudaStream_t st) {
  FieldGeom g = FieldGeom::make(n1, n2, n3, image_padded);
  const int64_t n = cells(n1, n2, n3);
  dim3 grid(blocks_for(n, kGenThreads));
  if (kdt == MLPCG_F32)
    k_stencil_gen<float><<<grid, kGenThreads, 0, st>>>(image, g, W, bias, (float *)K, ps);
  else
    k_stencil_gen<__nv_bfloat16><<<grid, kGenThreads, 0, st>>>(image, g, W, bias, (__nv_bfloat16 *)K, ps);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

template <typename KT, typename XT, typename YT>
static void apply_dispatch3(const void *K, int64_t ps, const void *x, FieldGeom gx, void *y, int B,
                            int trans, cudaStream_t st) {
  const int64_t n = cells(gx.n1, gx.n2, gx.n3);
  dim3 grid(blocks_for(n, 256), B);
  if (trans)
    k_stencil_apply<KT, XT, YT, true><<<grid, 256, 0, st>>>((const KT *)K, ps, (const XT *)x, gx, (YT *)y);
  else
    k_stencil_apply<KT, XT, YT, false><<<grid, 256, 0, st>>>((const KT *)K, ps, (const XT *)x, gx, (YT *)y);
}

template <typename KT, typename XT>
static void apply_dispatch2(const void *K, int64_t ps, const void *x, FieldGeom gx, void *y, int ydt,
                            int B, int trans, cudaStream_t st) {
  if (ydt == MLPCG_F32) apply_dispatch3<KT, XT, float>(K, ps, x, gx, y, B, trans, st);
  else apply_dispatch3<KT, XT, __nv_bfloat16>(K, ps, x, gx, y, B, trans, st);
}

template <typename KT>
static void apply_dispatch1(const void *K, int64_t ps, const void *x, int xdt, FieldGeom gx, void *y,
                            int ydt, int B, int trans, cudaStream_t st) {
  if (xdt == MLPCG_F32) apply_dispatch2<KT, float>(K, ps, x, gx, y, ydt, B, trans, st);
  else apply_dispatch2<KT, __nv_bfloat16>(K, ps, x, gx, y, ydt, B, trans, st);
}

int launch_stencil_apply(const void *K, int kdt, int64_t ps, const void *x, int xdt, int x_padded,
                         void *y, int ydt, int B, int n1, int n2, int n3, int trans,
                         cudaStream_t st) {
  FieldGeom gx = FieldGeom::make(n1, n2, n3, x_padded);
  if (kdt == MLPCG_F32) apply_dispatch1<float>(K, ps, x, xdt, gx, y, ydt, B, trans, st);
  else apply_dispatch1<__nv_bfloat16>(K, ps, x, xdt, gx, y, ydt, B, trans, st);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_coeff_grad(const float *g, const float *x, int x_padded, float *dK, int64_t ps, int B,
                      int n1, int n2, int n3, int trans, cudaStream_t st) {
  FieldGeom gx = FieldGeom::make(n1, n2, n3, x_padded);
  dim3 grid(blocks_for(cells(n1, n2, n3), 256));
  if (trans) k_coeff_grad<true><<<grid, 256, 0, st>>>(g, x, gx, B, dK, ps);
  else k_coeff_grad<false><<<grid, 256, 0, st>>>(g, x, gx, B, dK, ps);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

size_t wgrad_workspace(int n1, int n2, int n3) {
  const int64_t n = cells(n1, n2, n3);
  int64_t nblk = (n + kWgTile - 1) / kWgTile;
  if (nblk > kWgBlocksMax) nblk = kWgBlocksMax;
  if (nblk < 1) nblk = 1;
  return (size_t)nblk * kWgOut * sizeof(double);
}

int launch_wgrad(const float *dK, int64_t ps, const float *image, int image_padded, int n1, int n2,
                 int n3, float *gw, float *gb, void *ws, size_t ws_bytes, cudaStream_t st) {
  const int64_t n = cells(n1, n2, n3);
  int64_t nblk = (n + kWgTile - 1) / kWgTile;
  if (nblk > kWgBlocksMax) nblk = kWgBlocksMax;
  if (nblk < 1) nblk = 1;
  MLPCG_REQUIRE(ws_bytes >= (size_t)nblk * kWgOut * sizeof(double), MLPCG_ERR_WORKSPACE,
                "wgrad workspace too small: %zu < %zu", ws_bytes,
                (size_t)nblk * kWgOut * sizeof(double));
  FieldGeom g = FieldGeom::make(n1, n2, n3, image_padded);
  k_wgrad_partial<<<(unsigned)nblk, 256, 0, st>>>(dK, ps, image, g, (double *)ws);
  MLPCG_LAUNCH_CHECK();
  k_wgrad_finalize<<<blocks_for(27 * 82, 128), 128, 0, st>>>((const double *)ws, (int)nblk, gw, gb);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int launch_image_grad(const float *dK, int64_t ps, const float *W, float *gimg, int n1, int n2,
                      int n3, cudaStream_t st) {
  k_image_grad<<<blocks_for(cells(n1, n2, n3), 128), 128, 0, st>>>(dK, ps, W, n1, n2, n3, gimg);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

}  // namespace mlpcg
