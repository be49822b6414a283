// Fused neural-preconditioned solve: the whole iteration on the GPU inside one
// CUDA graph whose conditional WHILE node loops until convergence, breakdown
// or max_it -- no host synchronisation per iteration (the reference syncs on
// .item() every iteration, cg_tests.py:90,266).
//
// Two iteration forms with the reference's recurrences:
//   NPSD (cg_tests.py:189-284): q = M r, A-orthogonalised against the last two
//        directions, x += (q.r / q.Aq) q.
//   NPCG (cg_tests.py:26-101): textbook PCG with the network as M.
// Precision: vectors r, z, p, Ap in FP32 on the full grid (zero off-fluid);
// the iterate x and the right-hand side b as double-float pairs (hi + lo,
// two floats, about 48 significant bits) updated with error-free FP32
// transformations -- GB300's FP64 pipe runs at a small fraction of its FP32
// rate, so FP64 arithmetic is used only to convert b and x in and x out once
// per solve; every dot product is summed per thread with a compensated FP32
// sum and reduced in FP64 across threads and, in fixed order, across blocks;
// the residual is recomputed as r = b - A x in double-float every
// `true_every` iterations and before declaring convergence (the reference
// recomputes it every iteration, cg_tests.py:83,260).
//
// Every reduction kernel ends with a "last block" step: block partials go to
// scratch, the last block to finish (atomic ticket) sums them in block order
// and updates the solver state.  Each loop iteration increments the
// iteration counter unconditionally and the loop stops at max_it, so the
// WHILE node always terminates.
#include <cuda.h>

#include <algorithm>
#include <vector>
#include "common.cuh"

struct mlpcg_precond;
namespace mlpcg {
int precond_apply_gated(const mlpcg_precond *, const float *, const float *, float *, const int *, void *,
                        const ZDots *);
int64_t precond_zdots_tiles(const mlpcg_precond *);
int64_t precond_level0_tiles(const mlpcg_precond *);
const int *precond_copy_flag(const mlpcg_precond *);
bool encode_grid_map(CUtensorMap *m, const float *base, int n1, int n2, int n3, int box_z, int box_y, int box_x);
}

namespace mlpcg {

enum { ST_RUNNING = 0, ST_CONVERGED = 1, ST_MAXIT = 2, ST_BREAKDOWN = 3, ST_NONFINITE = 4, ST_COPYFAIL = 5 };
enum { M_NPSD = 0, M_NPCG = 1 };

constexpr int RT = 256;          // threads per reduction block
constexpr int RB_MAX = 1216;     // blocks per reduction kernel at most (8 per SM): one ticket atomic each
constexpr int NRED = 3;          // dot products per kernel at most

struct State {
  int it, status, need_true, head;    // head: ring slot of the most recent direction
  int pp;                             // NPCG: index of the current p buffer
  int max_it, true_every, method;
  double tol, bb, rr, rr_true, rel;
  double alpha[3];                    // NPSD: p_j . A p_j per ring slot
  double e_last;                      // NPSD: p_recent . A p_previous
  double c0, c1, beta, rz_old, rz;
  float beta_hi, beta_lo;             // beta as a double-float pair
  float rscale;                       // 1/||r|| fed to the preconditioner
  // x is updated every other iteration: the pending term beta_k d_k (pend = 1) is added together
  // with the next iteration's (same double-float operations, same order), or on the fly by the
  // true residual and the final conversion; d_k stays in its buffer slot pend_buf until then
  int pend, pend_buf;
  float pend_hi, pend_lo;
  int stall_copies;                   // copy-stall test knob: the SpMV's first tile wait runs out
  unsigned ticket[4];
};

// q / d for q < 2^31 by multiply and shift (Granlund & Montgomery 1994, fig. 4.1)
struct FastDiv {
  uint32_t m, s1, s2;
};

struct Vecs {
  FastDiv fd3, fd2;  // division by N3 and by N2
  uint32_t ngroups;  // n / 4
  const uint8_t *flags;
  uint8_t *code;     // per cell: fluid -> diagonal (fluid + air neighbours), else kNotFluid
  const double *b;   // caller's right-hand side (FP64), read once per solve
  double *x;         // caller's iterate (FP64), read at the start and written at the end of a solve
  float2 *xd, *bd;   // x and b as double-float pairs (x zero off the fluid cells)
  float *r, *z;
  float *p;        // 3 slots (NPSD ring) or 2 (NPCG ping-pong), n each
  float *Ap;       // 3 slots (NPSD) or 1 (NPCG)
  double *part;    // NRED * RB_MAX partial sums
  double *zpart;   // NPSD: 2 per finest-level tile, the products z . Ap from the preconditioner's epilogue
  int64_t ztiles;  // tiles summed by k_sd_dots_tiles
  double *hist;    // max_it + 1 relative residuals
  State *st;
  const int *perr; // the preconditioner plan's copy-failed word (its level-0 TMA tiles)
  int zero_guess;  // x0 = 0: k_prepare does not read x, k_finalize writes every cell (0 off the fluid)
  int n1, n2, n3;
  int64_t n;
  int nblk;
};

// ---- block reduction of NR values into partials, last block finalises ----
template <int NR>
__device__ __forceinline__ bool reduce_last(double (&v)[NR], const Vecs &V, int slot, double (&out)[NR]) {
  __shared__ double red[NR][RT / 32];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < NR; ++r)
    for (int o = 16; o > 0; o >>= 1) v[r] += __shfl_xor_sync(0xffffffffu, v[r], o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
#pragma unroll
    for (int r = 0; r < NR; ++r) red[r][w] = v[r];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      double s = 0.0;
      for (int ww = 0; ww < RT / 32; ++ww) s += red[r][ww];
      V.part[r * RB_MAX + blockIdx.x] = s;
    }
    __threadfence();
    const unsigned t = atomicAdd(&V.st->ticket[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  // last block: fixed-order sum of the partials
  __threadfence();
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) s += __ldcg(&V.part[r * RB_MAX + b]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) red[r][w] = s;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    double s = 0.0;
    for (int ww = 0; ww < RT / 32; ++ww) s += red[r][ww];
    out[r] = s;
  }
  if (threadIdx.x == 0) V.st->ticket[slot] = 0u;
  return true;
}

// ---------------------------------------------------------------------------
// Cells are processed in groups of 4 consecutive z cells (N3 % 4 == 0): one
// 16-byte load per FP32 vector (two for FP64), one 4-byte load of flags.
// (i, j, k0) of a group come from a multiply-shift division by N3 and N2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  const uint32_t t = __umulhi(f.m, n);
  return (t + ((n - t) >> f.s1)) >> f.s2;
}

__device__ __forceinline__ uint32_t gstride() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ void ld4(const float *p, float v[4]) {
  const float4 a = *reinterpret_cast<const float4 *>(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void st4(float *p, const float v[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void ld4(const double *p, double v[4]) {
  const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(double *p, const double v[4]) {
  reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void ld4(const float2 *p, float2 v[4]) {
  const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
  v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w); v[2] = make_float2(b.x, b.y); v[3] = make_float2(b.z, b.w);
}
__device__ __forceinline__ void st4(float2 *p, const float2 v[4]) {
  reinterpret_cast<float4 *>(p)[0] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
  reinterpret_cast<float4 *>(p)[1] = make_float4(v[2].x, v[2].y, v[3].x, v[3].y);
}
__device__ __forceinline__ uchar4 ldflags4(const uint8_t *p) { return *reinterpret_cast<const uchar4 *>(p); }
__device__ __forceinline__ uint8_t lane(const uchar4 f, int c) {
  return c == 0 ? f.x : (c == 1 ? f.y : (c == 2 ? f.z : f.w));
}

// sources of the vector a stencil is applied to
struct SrcF32 {
  const float *a;
  __device__ __forceinline__ void load4(uint32_t q, float v[4]) const { ld4(a + q, v); }
  __device__ __forceinline__ float load1(uint32_t q) const { return a[q]; }
};
struct SrcZero {  // no values: loads only the flags of a neighbourhood
  __device__ __forceinline__ void load4(uint32_t, float v[4]) const { v[0] = v[1] = v[2] = v[3] = 0.f; }
  __device__ __forceinline__ float load1(uint32_t) const { return 0.f; }
};
// p_new = z + beta * p_old, evaluated on the fly (first iteration: p_new = z)
struct SrcAxpy {
  const float *z, *p;
  float beta;
  bool first;
  __device__ __forceinline__ void load4(uint32_t q, float v[4]) const {
    ld4(z + q, v);
    if (!first) {
      float w[4];
      ld4(p + q, w);
#pragma unroll
      for (int c = 0; c < 4; ++c) v[c] = fmaf(beta, w[c], v[c]);
    }
  }
  __device__ __forceinline__ float load1(uint32_t q) const { return first ? z[q] : fmaf(beta, p[q], z[q]); }
};

// Everything the 7-point operator needs on one 4-cell group, loaded before
// any arithmetic so that all of a thread's loads are in flight together.
// Missing neighbours (outside the grid) get SOLID flags.
template <typename T>
struct Nbr4 {
  uchar4 fc, fxm, fym, fyp, fxp;
  uint8_t fzm, fzp;
  T c[4], xm[4], ym[4], yp[4], xp[4];
  T zm, zp;
};

template <typename T, typename S>
__device__ __forceinline__ void nbr_load(const Vecs &V, uint32_t q, int i, int j, int k0, const S &src, Nbr4<T> &N) {
  const uint32_t sy = (uint32_t)V.n3, sx = (uint32_t)V.n2 * (uint32_t)V.n3;
  const uchar4 solid = make_uchar4(MLPCG_SOLID, MLPCG_SOLID, MLPCG_SOLID, MLPCG_SOLID);
  N.fc = ldflags4(V.flags + q);
  src.load4(q, N.c);
  N.fxm = N.fym = N.fyp = N.fxp = solid;
  N.fzm = N.fzp = MLPCG_SOLID;
#pragma unroll
  for (int c = 0; c < 4; ++c) N.xm[c] = N.ym[c] = N.yp[c] = N.xp[c] = T(0);
  N.zm = N.zp = T(0);
  if (i > 0) { N.fxm = ldflags4(V.flags + q - sx); src.load4(q - sx, N.xm); }
  if (j > 0) { N.fym = ldflags4(V.flags + q - sy); src.load4(q - sy, N.ym); }
  if (k0 > 0) { N.fzm = V.flags[q - 1]; N.zm = src.load1(q - 1); }
  if (k0 + 4 < V.n3) { N.fzp = V.flags[q + 4]; N.zp = src.load1(q + 4); }
  if (j < V.n2 - 1) { N.fyp = ldflags4(V.flags + q + sy); src.load4(q + sy, N.yp); }
  if (i < V.n1 - 1) { N.fxp = ldflags4(V.flags + q + sx); src.load4(q + sx, N.xp); }
}

// (A v) on the group from its loaded neighbourhood.  Neighbours are summed in
// the column order of the assembled CSR row: i-1, j-1, k-1, k+1, j+1, i+1.
template <typename T>
__device__ __forceinline__ void nbr_apply(const Nbr4<T> &N, T out[4]) {
  T off[4] = {T(0), T(0), T(0), T(0)};
  int d[4] = {0, 0, 0, 0};
  auto take = [&](int c, uint8_t f, T v) {
    if (f == MLPCG_FLUID) { off[c] += v; ++d[c]; }
    else if (f == MLPCG_AIR) { ++d[c]; }
  };
#pragma unroll
  for (int c = 0; c < 4; ++c) take(c, lane(N.fxm, c), N.xm[c]);
#pragma unroll
  for (int c = 0; c < 4; ++c) take(c, lane(N.fym, c), N.ym[c]);
  take(0, N.fzm, N.zm);
#pragma unroll
  for (int c = 1; c < 4; ++c) take(c, lane(N.fc, c - 1), N.c[c - 1]);
#pragma unroll
  for (int c = 0; c < 3; ++c) take(c, lane(N.fc, c + 1), N.c[c + 1]);
  take(3, N.fzp, N.zp);
#pragma unroll
  for (int c = 0; c < 4; ++c) take(c, lane(N.fyp, c), N.yp[c]);
#pragma unroll
  for (int c = 0; c < 4; ++c) take(c, lane(N.fxp, c), N.xp[c]);
#pragma unroll
  for (int c = 0; c < 4; ++c) out[c] = lane(N.fc, c) == MLPCG_FLUID ? T(d[c]) * N.c[c] - off[c] : T(0);
}

// The operator on vectors that vanish off the fluid cells (every CG vector
// r, z, p, q, Ap does): a fluid cell's row is d v_c - (sum of the 6
// neighbours), the non-fluid neighbours contributing their zeros, so the
// stencil needs only the cell's code -- d, the number of fluid or air
// neighbours (the CSR diagonal), or kNotFluid.  Same terms, same order as
// nbr_apply.
constexpr uint8_t kNotFluid = 0x80;

template <typename S>
__device__ __forceinline__ void lap4_code(const Vecs &V, uint32_t q, int i, int j, int k0, const S &src,
                                          float out[4], float cen[4]) {
  const uint32_t sy = (uint32_t)V.n3, sx = (uint32_t)V.n2 * (uint32_t)V.n3;
  float xm[4] = {0.f, 0.f, 0.f, 0.f}, ym[4] = {0.f, 0.f, 0.f, 0.f};
  float yp[4] = {0.f, 0.f, 0.f, 0.f}, xp[4] = {0.f, 0.f, 0.f, 0.f};
  float zm = 0.f, zp = 0.f;
  const uchar4 cd = ldflags4(V.code + q);
  src.load4(q, cen);
  if (i > 0) src.load4(q - sx, xm);
  if (j > 0) src.load4(q - sy, ym);
  if (k0 > 0) zm = src.load1(q - 1);
  if (k0 + 4 < V.n3) zp = src.load1(q + 4);
  if (j < V.n2 - 1) src.load4(q + sy, yp);
  if (i < V.n1 - 1) src.load4(q + sx, xp);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float off = 0.f;
    off += xm[c];
    off += ym[c];
    off += c == 0 ? zm : cen[c - 1];
    off += c == 3 ? zp : cen[c + 1];
    off += yp[c];
    off += xp[c];
    const uint8_t k = lane(cd, c);
    out[c] = (k & kNotFluid) ? 0.f : (float)k * cen[c] - off;
  }
}

constexpr int UNR = 2;  // groups per thread per loop pass in the streaming kernels

__device__ __forceinline__ void group_coords(const Vecs &V, uint32_t g, uint32_t &q, int &i, int &j, int &k0) {
  q = 4u * g;
  const uint32_t rowi = fdiv(q, V.fd3);
  k0 = (int)(q - rowi * (uint32_t)V.n3);
  const uint32_t ii = fdiv(rowi, V.fd2);
  j = (int)(rowi - ii * (uint32_t)V.n2);
  i = (int)ii;
}

// ---------------------------------------------------------------------------
// setup: state reset, then r = b - A x (FP64), bb = b.b, rr = r.r
// ---------------------------------------------------------------------------
__global__ void k_reset(State *st, int max_it, int true_every, int method, double tol, int stall_copies) {
  dependent_launch_enter();
  if (threadIdx.x != 0) return;
  State S{};
  S.max_it = max_it;
  S.true_every = true_every;
  S.method = method;
  S.tol = tol;
  S.stall_copies = stall_copies;
  *st = S;
}

// Once per solve, before the residual: every cell's operator code (see
// lap4_code), and x, b as double-float pairs on the fluid cells (zero
// elsewhere; the operator never reads x off the fluid cells).  The
// conversions use integer operations (df_from_double_bits); cells whose value
// is exactly zero skip them.
__global__ void __launch_bounds__(RT) k_prepare(Vecs V) {
  dependent_launch_enter();
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    uint32_t q; int i, j, k0;
    group_coords(V, g, q, i, j, k0);
    Nbr4<float> N;
    nbr_load<float>(V, q, i, j, k0, SrcZero{}, N);
    uint8_t cd[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      auto open = [](uint8_t f) { return f == MLPCG_FLUID || f == MLPCG_AIR ? 1 : 0; };
      const int d = open(lane(N.fxm, c)) + open(lane(N.fym, c)) + open(c == 0 ? N.fzm : lane(N.fc, c - 1)) +
                    open(c == 3 ? N.fzp : lane(N.fc, c + 1)) + open(lane(N.fyp, c)) + open(lane(N.fxp, c));
      cd[c] = lane(N.fc, c) == MLPCG_FLUID ? (uint8_t)d : kNotFluid;
    }
    *reinterpret_cast<uchar4 *>(V.code + q) = make_uchar4(cd[0], cd[1], cd[2], cd[3]);
    double xq[4] = {0.0, 0.0, 0.0, 0.0}, bq[4];
    if (!V.zero_guess) ld4(V.x + q, xq);
    ld4(V.b + q, bq);
    float2 xd[4], bd[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const bool fl = !(cd[c] & kNotFluid);
      // zero tests on the bit patterns (integer ops), so zero cells cost no FP64 work
      xd[c] = (fl && (__double_as_longlong(xq[c]) << 1)) ? df_from_double_bits(xq[c]) : make_float2(0.f, 0.f);
      bd[c] = (fl && (__double_as_longlong(bq[c]) << 1)) ? df_from_double_bits(bq[c]) : make_float2(0.f, 0.f);
    }
    st4(V.xd + q, xd);
    st4(V.bd + q, bd);
  }
}

// r = b - A x in double-float arithmetic (x, b as pairs, zero off the fluid
// cells), stored rounded to FP32; accumulates sum r^2 (and, with BB, sum b^2)
// with compensated FP32 sums.  The neighbours are added in the column order
// of the assembled CSR row (i-1, j-1, k-1, k+1, j+1, i+1).
// x with a pending update beta_p d_p (pd == nullptr: none), per cell exactly as k_update adds it
struct XEff {
  const float2 *x;
  const float *pd;
  float2 bp;
  __device__ __forceinline__ float2 at(uint32_t q) const {
    return pd ? df_add(x[q], df_mul_f(bp, pd[q])) : x[q];
  }
  __device__ __forceinline__ void at4(uint32_t q, float2 v[4]) const {
    ld4(x + q, v);
    if (pd) {
      float d[4];
      ld4(pd + q, d);
#pragma unroll
      for (int c = 0; c < 4; ++c) v[c] = df_add(v[c], df_mul_f(bp, d[c]));
    }
  }
};
__device__ __forceinline__ XEff x_eff(const Vecs &V) {
  const State &S = *V.st;
  XEff e{V.xd, S.pend ? V.p + (size_t)S.pend_buf * V.n : nullptr, make_float2(S.pend_hi, S.pend_lo)};
  return e;
}

template <bool BB>
__device__ __forceinline__ void residual_pass(const Vecs &V, CSum &bb, CSum &rr) {
  const uint32_t sy = (uint32_t)V.n3, sx = (uint32_t)V.n2 * (uint32_t)V.n3;
  const float2 zero = make_float2(0.f, 0.f);
  const XEff X = x_eff(V);
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    uint32_t q; int i, j, k0;
    group_coords(V, g, q, i, j, k0);
    float2 cen[4], xm[4], ym[4], yp[4], xp[4], bq[4];
    float2 zm = zero, zp = zero;
#pragma unroll
    for (int c = 0; c < 4; ++c) xm[c] = ym[c] = yp[c] = xp[c] = zero;
    const uchar4 cd = ldflags4(V.code + q);
    X.at4(q, cen);
    ld4(V.bd + q, bq);
    if (i > 0) X.at4(q - sx, xm);
    if (j > 0) X.at4(q - sy, ym);
    if (k0 > 0) zm = X.at(q - 1);
    if (k0 + 4 < V.n3) zp = X.at(q + 4);
    if (j < V.n2 - 1) X.at4(q + sy, yp);
    if (i < V.n1 - 1) X.at4(q + sx, xp);
    float rf[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const uint8_t k = lane(cd, c);
      rf[c] = 0.f;
      if (k & kNotFluid) continue;
      float2 off = df_add(xm[c], ym[c]);
      off = df_add(off, c == 0 ? zm : cen[c - 1]);
      off = df_add(off, c == 3 ? zp : cen[c + 1]);
      off = df_add(off, yp[c]);
      off = df_add(off, xp[c]);
      const float2 ax = df_add(df_mul_f(cen[c], (float)k), df_neg(off));
      const float2 rv = df_add(bq[c], df_neg(ax));
      rf[c] = __fadd_rn(rv.x, rv.y);
      rr.add(__fmul_rn(rf[c], rf[c]));
      if (BB) bb.add(__fmul_rn(bq[c].x, bq[c].x));
    }
    st4(V.r + q, rf);
  }
}

// The caller's x from the pairs, on the fluid cells (the others keep their values)
__global__ void __launch_bounds__(RT) k_finalize(Vecs V) {
  dependent_launch_enter();
  const XEff X = x_eff(V);  // with a still pending update of the iterate
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    const uint32_t q = 4u * g;
    const uchar4 cd = ldflags4(V.code + q);
    float2 xd[4];
    X.at4(q, xd);
    const bool all_fluid = !((cd.x | cd.y | cd.z | cd.w) & kNotFluid);
    if (all_fluid) {  // the common case: two 16-byte stores
      double2 *o = reinterpret_cast<double2 *>(V.x + q);
      o[0] = make_double2(df_to_double_bits(xd[0]), df_to_double_bits(xd[1]));
      o[1] = make_double2(df_to_double_bits(xd[2]), df_to_double_bits(xd[3]));
    } else if (V.zero_guess) {  // x was not read: every cell is written, 0 off the fluid
      double v[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) v[c] = (lane(cd, c) & kNotFluid) ? 0.0 : df_to_double_bits(xd[c]);
      double2 *o = reinterpret_cast<double2 *>(V.x + q);
      o[0] = make_double2(v[0], v[1]);
      o[1] = make_double2(v[2], v[3]);
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (!(lane(cd, c) & kNotFluid)) V.x[q + c] = df_to_double_bits(xd[c]);
    }
  }
}

// The initial residual from x0 = 0: residual_pass's arithmetic with every x value zero (A x is
// then the pair (0, 0) exactly), without reading x -- the same bits.
__device__ __forceinline__ void residual_pass_zero_x(const Vecs &V, CSum &bb, CSum &rr) {
  const float2 nz = make_float2(-0.f, -0.f);  // df_neg of A x = (0, 0)
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    const uint32_t q = 4u * g;
    const uchar4 cd = ldflags4(V.code + q);
    float2 bq[4];
    ld4(V.bd + q, bq);
    float rf[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      rf[c] = 0.f;
      if (lane(cd, c) & kNotFluid) continue;
      const float2 rv = df_add(bq[c], nz);
      rf[c] = __fadd_rn(rv.x, rv.y);
      rr.add(__fmul_rn(rf[c], rf[c]));
      bb.add(__fmul_rn(bq[c].x, bq[c].x));
    }
    st4(V.r + q, rf);
  }
}

__global__ void __launch_bounds__(RT) k_init(Vecs V) {
  dependent_launch_enter();
  CSum bb, rr;
  if (V.zero_guess) residual_pass_zero_x(V, bb, rr);
  else residual_pass<true>(V, bb, rr);
  double v[2] = {bb.get(), rr.get()};
  double o[2];
  if (reduce_last<2>(v, V, 0, o) && threadIdx.x == 0) {
    State &S = *V.st;
    S.bb = o[0];
    S.rr = o[1];
    S.it = 0;
    S.head = 2;
    S.pp = 0;
    S.need_true = 0;
    if (!isfinite(o[0]) || !isfinite(o[1])) {
      S.rel = o[1];
      S.status = ST_NONFINITE;
    } else {
      S.rel = (o[0] > 0.0) ? sqrt(o[1] / o[0]) : 0.0;
      S.status = (o[0] > 0.0 && S.rel >= S.tol) ? ST_RUNNING : ST_CONVERGED;
    }
    S.rscale = (o[1] > 0.0) ? (float)(1.0 / sqrt((double)(float)o[1])) : 1.f;
    S.alpha[0] = S.alpha[1] = S.alpha[2] = 0.0;
    S.e_last = 0.0;
    S.beta = S.c0 = S.c1 = 0.0;
    S.beta_hi = S.beta_lo = 0.f;
    S.rz_old = 0.0;
    V.hist[0] = S.rel;
  }
}

// ---------------------------------------------------------------------------
// NPSD
// ---------------------------------------------------------------------------
// d1 = z . A p_recent, d0 = z . A p_previous  ->  c1, c0 of
// q = z - c1 p_recent - c0 p_previous  (the two sequential projections of
// cg_tests.py:226-233, with q.A p_previous expanded as d0 - c1 e_last).
__global__ void __launch_bounds__(RT) k_sd_dots(Vecs V) {
  dependent_launch_enter();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const int it = S.it;
  if (it == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { V.st->c0 = 0.0; V.st->c1 = 0.0; }
    return;
  }
  const int h = S.head, hp = (h + 2) % 3;
  const float *A1 = V.Ap + (size_t)h * V.n, *A0 = V.Ap + (size_t)hp * V.n;
  const bool two = it >= 2;
  CSum a1s, a0s;
  for (uint32_t g0 = blockIdx.x * RT * UNR + threadIdx.x; g0 < V.ngroups; g0 += gridDim.x * RT * UNR) {
    float z[UNR][4], a1[UNR][4], a0[UNR][4];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const uint32_t g = g0 + u * RT;
      if (g >= V.ngroups) continue;
      ld4(V.z + 4 * g, z[u]);
      ld4(A1 + 4 * g, a1[u]);
      if (two) ld4(A0 + 4 * g, a0[u]);
    }
    float s1 = 0.f, s0 = 0.f;
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      if (g0 + u * RT >= V.ngroups) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        s1 = fmaf(z[u][c], a1[u][c], s1);
        if (two) s0 = fmaf(z[u][c], a0[u][c], s0);
      }
    }
    a1s.add(s1);
    a0s.add(s0);
  }
  double v[2] = {a1s.get(), a0s.get()};
  double o[2];
  if (reduce_last<2>(v, V, 1, o) && threadIdx.x == 0) {
    State &W = *V.st;
    const double c1 = o[0] / W.alpha[h];
    const double c0 = two ? (o[1] - c1 * W.e_last) / W.alpha[hp] : 0.0;
    W.c1 = c1;
    W.c0 = c0;
  }
}

// The same two products from the preconditioner's level-0 epilogue (ZDots): the per-tile FP64
// partials summed by ZT_BLOCKS blocks (each thread a fixed strided share, then the blocks' fixed
// reduction and the last block's sum in block order), then c1, c0 as above.
constexpr int ZT_BLOCKS = 64;
__global__ void __launch_bounds__(RT) k_sd_dots_tiles(Vecs V) {
  dependent_launch_enter();
  dependent_launch_trigger();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const int it = S.it;
  if (it == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { V.st->c0 = 0.0; V.st->c1 = 0.0; }
    return;
  }
  const double2 *zp = reinterpret_cast<const double2 *>(V.zpart);
  const int64_t stride = (int64_t)gridDim.x * RT;
  double a1 = 0.0, a0 = 0.0;
  for (int64_t t0 = (int64_t)blockIdx.x * RT + threadIdx.x; t0 < V.ztiles; t0 += 4 * stride) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t t = t0 + u * stride;
      v[u] = t < V.ztiles ? zp[t] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a1 += v[u].x;
      a0 += v[u].y;
    }
  }
  double v[2] = {a1, a0};
  double o[2];
  if (reduce_last<2>(v, V, 1, o) && threadIdx.x == 0) {
    State &W = *V.st;
    const int h = W.head, hp = (h + 2) % 3;
    const double c1 = o[0] / W.alpha[h];
    const double c0 = it >= 2 ? (o[1] - c1 * W.e_last) / W.alpha[hp] : 0.0;
    W.c1 = c1;
    W.c0 = c0;
  }
}

// q = z - c1 p_recent - c0 p_previous into the next ring slot
__global__ void __launch_bounds__(RT) k_sd_qform(Vecs V) {
  dependent_launch_enter();
  dependent_launch_trigger();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const int h = S.head, hp = (h + 2) % 3, hn = (h + 1) % 3;
  const float c1 = (float)S.c1, c0 = (float)S.c0;
  const float *P1 = V.p + (size_t)h * V.n, *P0 = V.p + (size_t)hp * V.n;
  float *Q = V.p + (size_t)hn * V.n;
  const int it = S.it;
  for (uint32_t g0 = blockIdx.x * RT * UNR + threadIdx.x; g0 < V.ngroups; g0 += gridDim.x * RT * UNR) {
    float z[UNR][4], a[UNR][4], b[UNR][4];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const uint32_t q = 4u * (g0 + u * RT);
      if (g0 + u * RT >= V.ngroups) continue;
      ld4(V.z + q, z[u]);
      if (it >= 1) ld4(P1 + q, a[u]);
      if (it >= 2) ld4(P0 + q, b[u]);
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const uint32_t q = 4u * (g0 + u * RT);
      if (g0 + u * RT >= V.ngroups) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (it >= 1) z[u][c] = fmaf(-c1, a[u][c], z[u][c]);
        if (it >= 2) z[u][c] = fmaf(-c0, b[u][c], z[u][c]);
      }
      st4(Q + q, z[u]);
    }
  }
}

// Aq, alpha = q.Aq, q.r, e = Aq.p_recent; then beta = q.r / alpha
__global__ void __launch_bounds__(RT) k_sd_spmv(Vecs V) {
  dependent_launch_enter();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const int h = S.head, hn = (h + 1) % 3;
  const float *Q = V.p + (size_t)hn * V.n, *P1 = V.p + (size_t)h * V.n;
  float *AQ = V.Ap + (size_t)hn * V.n;
  const bool has_prev = S.it >= 1;
  CSum t0, t1, t2;
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    uint32_t q; int i, j, k0;
    group_coords(V, g, q, i, j, k0);
    float rq[4], p1[4], qc[4], aq[4];
    ld4(V.r + q, rq);
    if (has_prev) ld4(P1 + q, p1);
    lap4_code(V, q, i, j, k0, SrcF32{Q}, aq, qc);
    st4(AQ + q, aq);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      s0 = fmaf(qc[c], aq[c], s0);
      s1 = fmaf(qc[c], rq[c], s1);
      if (has_prev) s2 = fmaf(aq[c], p1[c], s2);
    }
    t0.add(s0); t1.add(s1); t2.add(s2);
  }
  double v[3] = {t0.get(), t1.get(), t2.get()};
  double o[3];
  if (reduce_last<3>(v, V, 2, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.alpha[hn] = o[0];
    W.e_last = o[2];
    W.head = hn;
    W.beta = o[1] / o[0];
    const float2 bdf = df_from_double(W.beta);
    W.beta_hi = bdf.x;
    W.beta_lo = bdf.y;
    if (!(o[0] > 0.0) || !isfinite(W.beta)) W.status = isfinite(o[0]) ? ST_BREAKDOWN : ST_NONFINITE;
  }
}

// The same step with q staged in shared memory by TMA: each CTA loops over 4 (x) x 16 (y) x 64 (z)
// output tiles; thread 0 has the tensor-memory accelerator copy the tile's q box with a one-cell
// halo (6 x 18 x 76 floats, z from z0 - 4: 16-byte aligned; zero outside the grid) while every
// thread loads its two 8-cell z-runs' codes, r and p_recent; the 7-point operator then reads the
// box (same terms, same order as lap4_code).  Thread t takes x planes 2 (t >> 7) + {0, 1} and the
// (y, z) run of lane pattern run_ty / run_tz, whose 16-byte shared loads of a row are
// conflict-free with the 76-float row pitch.  Requires N3 % 8 == 0.
constexpr int SPX = 4, SPY = 16, SPZ = 64;        // output tile
constexpr int SBX = SPX + 2, SBY = SPY + 2, SBZ = 76;  // q box
__device__ __forceinline__ int sp_tz(int t) { return (t & 3) | ((t >> 1) & 4); }
__device__ __forceinline__ int sp_ty(int t) { return ((t >> 2) & 1) | ((t >> 3) & 2) | ((t >> 5) << 2); }

__global__ void __launch_bounds__(RT, 3) k_sd_spmv_tma(Vecs V, const __grid_constant__ CUtensorMap tq0,
                                                   const __grid_constant__ CUtensorMap tq1,
                                                   const __grid_constant__ CUtensorMap tq2) {
  dependent_launch_enter();
  dependent_launch_trigger();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  __shared__ __align__(128) float T[SBX][SBY][SBZ];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t never;  // nothing arrives on it: the copy-stall test waits here
  __shared__ int copy_failed;
  const int h = S.head, hn = (h + 1) % 3;
  const CUtensorMap *tm = hn == 0 ? &tq0 : (hn == 1 ? &tq1 : &tq2);
  const float *P1 = V.p + (size_t)h * V.n;
  float *AQ = V.Ap + (size_t)hn * V.n;
  const bool has_prev = S.it >= 1;
  const int n1 = V.n1, n2 = V.n2, n3 = V.n3;
  const int tiles_z = (n3 + SPZ - 1) / SPZ, tiles_y = (n2 + SPY - 1) / SPY, tiles_x = (n1 + SPX - 1) / SPX;
  const int ntiles = tiles_z * tiles_y * tiles_x;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&mbar);
  const uint32_t nbar = (uint32_t)__cvta_generic_to_shared(&never);
  const bool stall = S.stall_copies != 0;
  if (threadIdx.x == 0) {
    copy_failed = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(nbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int tt = threadIdx.x & 127, hx = threadIdx.x >> 7;
  const int tz = sp_tz(tt), ty = sp_ty(tt);
  CSum t0, t1, t2;
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, phase ^= 1u) {
    const int bz = tile % tiles_z, rest = tile / tiles_z, by = rest % tiles_y, bx = rest / tiles_y;
    const int z0 = bz * SPZ, y0 = by * SPY, x0 = bx * SPX;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                   "r"((uint32_t)sizeof(T)) : "memory");
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
          ::"r"((uint32_t)__cvta_generic_to_shared(&T[0][0][0])), "l"(reinterpret_cast<uint64_t>(tm)), "r"(z0 - 4),
          "r"(y0 - 1), "r"(x0 - 1), "r"(bar)
          : "memory");
    }
    const int k0 = z0 + 8 * tz, j = y0 + ty;
    bool valid[2];
    uint32_t q0[2];
    uint2 cd[2];
    float rq[2][8], p1[2][8];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int i = x0 + 2 * hx + r;
      valid[r] = i < n1 && j < n2 && k0 < n3;
      q0[r] = valid[r] ? ((uint32_t)i * (uint32_t)n2 + (uint32_t)j) * (uint32_t)n3 + (uint32_t)k0 : 0u;
      cd[r] = make_uint2(0u, 0u);
      if (valid[r]) {
        cd[r] = *reinterpret_cast<const uint2 *>(V.code + q0[r]);
        ld4(V.r + q0[r], rq[r]);
        ld4(V.r + q0[r] + 4, rq[r] + 4);
        if (has_prev) {
          ld4(P1 + q0[r], p1[r]);
          ld4(P1 + q0[r] + 4, p1[r] + 4);
        }
      }
    }
    // bounded wait for the box (phase `phase`); a copy that never lands stops the solve.  With the
    // copy-stall knob the first wait polls the barrier nothing arrives on (256 tries), so it runs
    // out while the real copy completes; the second wait then lets that copy land
    uint32_t done = 0;
    const uint32_t wbar = stall ? nbar : bar, lim = stall ? 256u : (1u << 22);
    for (uint32_t it = 0; it < lim && !done; ++it)
      asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                   : "=r"(done) : "r"(wbar), "r"(stall ? 0u : phase) : "memory");
    if (!done) {
      copy_failed = 1;
      for (uint32_t it = 0; it < (1u << 22) && !done; ++it)  // let a late copy land before leaving
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done) : "r"(bar), "r"(phase) : "memory");
    }
    __syncthreads();
    if (copy_failed) break;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (!valid[r]) continue;
      const int lx = 2 * hx + r + 1;  // box plane of the run
      const float *C = &T[lx][ty + 1][8 * tz];
      float c16[16];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float4 a = reinterpret_cast<const float4 *>(C)[m];
        c16[4 * m] = a.x; c16[4 * m + 1] = a.y; c16[4 * m + 2] = a.z; c16[4 * m + 3] = a.w;
      }
      auto row8 = [&](const float *row, float v[8]) {
        const float4 a = reinterpret_cast<const float4 *>(row + 4)[0];
        const float4 b = reinterpret_cast<const float4 *>(row + 4)[1];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
      };
      float xm[8], xp[8], ym[8], yp[8];
      row8(&T[lx - 1][ty + 1][8 * tz], xm);
      row8(&T[lx + 1][ty + 1][8 * tz], xp);
      row8(&T[lx][ty][8 * tz], ym);
      row8(&T[lx][ty + 2][8 * tz], yp);
      float aq[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        float off = 0.f;
        off += xm[c];
        off += ym[c];
        off += c16[c + 3];  // z - 1
        off += c16[c + 5];  // z + 1
        off += yp[c];
        off += xp[c];
        const uint8_t k = (uint8_t)((c < 4 ? cd[r].x : cd[r].y) >> (8 * (c & 3)));
        aq[c] = (k & kNotFluid) ? 0.f : (float)k * c16[c + 4] - off;
      }
      st4(AQ + q0[r], aq);
      st4(AQ + q0[r] + 4, aq + 4);
#pragma unroll
      for (int gq = 0; gq < 2; ++gq) {
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
        for (int c = 4 * gq; c < 4 * gq + 4; ++c) {
          s0 = fmaf(c16[c + 4], aq[c], s0);
          s1 = fmaf(c16[c + 4], rq[r][c], s1);
          if (has_prev) s2 = fmaf(aq[c], p1[r][c], s2);
        }
        t0.add(s0); t1.add(s1); t2.add(s2);
      }
    }
    __syncthreads();  // every thread is done with the box before the next tile's copy
  }
  double v[3] = {t0.get(), t1.get(), t2.get()};
  double o[3];
  if (reduce_last<3>(v, V, 2, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.alpha[hn] = o[0];
    W.e_last = o[2];
    W.head = hn;
    W.beta = o[1] / o[0];
    const float2 bdf = df_from_double(W.beta);
    W.beta_hi = bdf.x;
    W.beta_lo = bdf.y;
    if (!(o[0] > 0.0) || !isfinite(W.beta)) W.status = isfinite(o[0]) ? ST_BREAKDOWN : ST_NONFINITE;
  }
  if (copy_failed && threadIdx.x == 0) V.st->status = ST_COPYFAIL;
}

// ---------------------------------------------------------------------------
// NPCG
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_cg_rz(Vecs V) {
  dependent_launch_enter();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  CSum t;
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    float r[4], z[4];
    ld4(V.r + 4 * g, r);
    ld4(V.z + 4 * g, z);
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) s = fmaf(r[c], z[c], s);
    t.add(s);
  }
  double v[1] = {t.get()};
  double o[1];
  if (reduce_last<1>(v, V, 1, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.rz = o[0];
    W.c1 = (W.it == 0) ? 0.0 : o[0] / W.rz_old;  // beta of the p update
    W.rz_old = o[0];
  }
}

// r . z from the preconditioner's level-0 epilogue (ZDots, single product): the per-tile FP64
// partials summed like k_sd_dots_tiles, then the same state update as k_cg_rz
__global__ void __launch_bounds__(RT) k_cg_rz_tiles(Vecs V) {
  dependent_launch_enter();
  dependent_launch_trigger();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const double2 *zp = reinterpret_cast<const double2 *>(V.zpart);
  const int64_t stride = (int64_t)gridDim.x * RT;
  double a = 0.0;
  for (int64_t t0 = (int64_t)blockIdx.x * RT + threadIdx.x; t0 < V.ztiles; t0 += 4 * stride) {
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t t = t0 + u * stride;
      v[u] = t < V.ztiles ? zp[t] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) a += v[u].x;
  }
  double v[1] = {a};
  double o[1];
  if (reduce_last<1>(v, V, 1, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.rz = o[0];
    W.c1 = (W.it == 0) ? 0.0 : o[0] / W.rz_old;  // beta of the p update
    W.rz_old = o[0];
  }
}

// p_new = z + beta p_old (ping-pong buffers), w = A p_new, pw = p_new . w, alpha = rz / pw
__global__ void __launch_bounds__(RT) k_cg_pspmv(Vecs V) {
  dependent_launch_enter();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const int cur = S.pp, nxt = cur ^ 1;
  float *Pn = V.p + (size_t)nxt * V.n;
  const SrcAxpy src{V.z, V.p + (size_t)cur * V.n, (float)S.c1, S.it == 0};
  CSum t;
  for (uint32_t g = gtid(); g < V.ngroups; g += gstride()) {
    uint32_t q; int i, j, k0;
    group_coords(V, g, q, i, j, k0);
    float w[4], pc[4];
    lap4_code(V, q, i, j, k0, src, w, pc);
    st4(Pn + q, pc);
    st4(V.Ap + q, w);
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) s = fmaf(pc[c], w[c], s);
    t.add(s);
  }
  double v[1] = {t.get()};
  double o[1];
  if (reduce_last<1>(v, V, 2, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.pp = nxt;
    W.beta = W.rz / o[0];  // the step length alpha of cg_tests.py:81
    const float2 bdf = df_from_double(W.beta);
    W.beta_hi = bdf.x;
    W.beta_lo = bdf.y;
    if (!isfinite(W.beta) || o[0] == 0.0) W.status = isfinite(o[0]) ? ST_BREAKDOWN : ST_NONFINITE;
  }
}

// ---------------------------------------------------------------------------
// shared: x += beta d (double-float); r -= beta A d; rr = r.r; decide whether a true residual is due
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_update(Vecs V) {
  dependent_launch_enter();
  dependent_launch_trigger();
  const State &S = *V.st;
  if (S.status != ST_RUNNING) return;
  const float *D, *AD;
  if (S.method == M_NPSD) {
    D = V.p + (size_t)S.head * V.n;
    AD = V.Ap + (size_t)S.head * V.n;
  } else {
    D = V.p + (size_t)S.pp * V.n;
    AD = V.Ap;
  }
  const float2 bd = make_float2(S.beta_hi, S.beta_lo);
  const float bf = (float)S.beta;
  // every other iteration x += beta_prev d_prev + beta d in one pass; in between only r moves
  const bool commit = S.pend != 0;
  const float *DP = V.p + (size_t)S.pend_buf * V.n;
  const float2 bp = make_float2(S.pend_hi, S.pend_lo);
  CSum t;
  for (uint32_t g0 = blockIdx.x * RT * UNR + threadIdx.x; g0 < V.ngroups; g0 += gridDim.x * RT * UNR) {
    float d[UNR][4], dp[UNR][4], ad[UNR][4], r[UNR][4];
    float2 x[UNR][4];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const uint32_t q = 4u * (g0 + u * RT);
      if (g0 + u * RT >= V.ngroups) continue;
      ld4(AD + q, ad[u]);
      ld4(V.r + q, r[u]);
      if (commit) {
        ld4(D + q, d[u]);
        ld4(DP + q, dp[u]);
        ld4(V.xd + q, x[u]);
      }
    }
    float s = 0.f;
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const uint32_t q = 4u * (g0 + u * RT);
      if (g0 + u * RT >= V.ngroups) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (commit) x[u][c] = df_add(df_add(x[u][c], df_mul_f(bp, dp[u][c])), df_mul_f(bd, d[u][c]));
        r[u][c] = fmaf(-bf, ad[u][c], r[u][c]);
        s = fmaf(r[u][c], r[u][c], s);
      }
      if (commit) st4(V.xd + q, x[u]);
      st4(V.r + q, r[u]);
    }
    t.add(s);
  }
  double v[1] = {t.get()};
  double o[1];
  if (reduce_last<1>(v, V, 3, o) && threadIdx.x == 0) {
    State &W = *V.st;
    W.rr = o[0];
    // every block has read the pending state before the ticket: safe to move it on
    if (commit) {
      W.pend = 0;
    } else {
      W.pend = 1;
      W.pend_buf = W.method == M_NPSD ? W.head : W.pp;
      W.pend_hi = W.beta_hi;
      W.pend_lo = W.beta_lo;
    }
    const int itn = W.it + 1;
    const double rel = sqrt(o[0] / W.bb);
    W.rel = rel;
    W.need_true = (rel < W.tol) || (W.true_every > 0 && itn % W.true_every == 0) || (itn >= W.max_it) ||
                  !isfinite(rel);
  }
}

// one thread: iteration bookkeeping, convergence, loop condition
__device__ __forceinline__ void control_step(const Vecs &V, cudaGraphConditionalHandle handle, int use_handle) {
  State &S = *V.st;
  if (S.status == ST_RUNNING) {
    const int itn = S.it + 1;
    S.it = itn;
    double rel = S.rel;
    if (S.need_true) {
      rel = sqrt(S.rr_true / S.bb);
      S.rr = S.rr_true;
      S.rel = rel;
      S.need_true = 0;
      if (rel < S.tol) S.status = ST_CONVERGED;
    }
    if (!isfinite(rel)) S.status = ST_NONFINITE;
    V.hist[itn] = rel;
    if (S.status == ST_RUNNING && itn >= S.max_it) S.status = ST_MAXIT;
    S.rscale = (S.rr > 0.0) ? (float)(1.0 / sqrt((double)(float)S.rr)) : 1.f;
  }
  // a preconditioner tile copy that did not complete left z invalid: that, not the breakdown or
  // non-finite value it may have caused, ends the solve (a converged or max_it result stands, its
  // residual being the true one)
  if (V.perr && *V.perr && S.status != ST_CONVERGED && S.status != ST_MAXIT) S.status = ST_COPYFAIL;
  if (use_handle) cudaGraphSetConditional(handle, S.status == ST_RUNNING ? 1u : 0u);
}

// The end of an iteration: r = b - A x (double-float) when due, then the control step -- by the
// last block of that reduction, or by block 0 when no true residual is due (the other blocks then
// return at once, whatever order they read the state in).
__global__ void __launch_bounds__(RT) k_true_residual_control(Vecs V, cudaGraphConditionalHandle handle,
                                                              int use_handle) {
  dependent_launch_enter();
  const State &S = *V.st;
  if (S.status != ST_RUNNING || !S.need_true) {
    if (blockIdx.x == 0 && threadIdx.x == 0) control_step(V, handle, use_handle);
    return;
  }
  CSum bb, rr;
  residual_pass<false>(V, bb, rr);
  double v[2] = {0.0, rr.get()};
  double o[2];
  if (reduce_last<2>(v, V, 0, o) && threadIdx.x == 0) {
    V.st->rr_true = o[1];
    control_step(V, handle, use_handle);
  }
}

// Batched solves: one loop for many systems.  Each system's control step
// updates its own state; this one keeps the loop running while any runs.
constexpr int kMaxBatch = 64;
struct BatchStates {
  State *st[kMaxBatch];
  int count;
};
__global__ void k_batch_control(BatchStates B, cudaGraphConditionalHandle handle) {
  dependent_launch_enter();
  const int t = threadIdx.x;
  const int running = (t < B.count && B.st[t]->status == ST_RUNNING) ? 1 : 0;
  const int any = __syncthreads_or(running);
  if (t == 0) cudaGraphSetConditional(handle, any ? 1u : 0u);
}

}  // namespace mlpcg

using namespace mlpcg;

struct mlpcg_solver {
  int n1, n2, n3, method, max_it, true_every;
  double tol;
  const mlpcg_precond *plan = nullptr;
  Vecs V{};
  size_t bytes = 0;
  bool bound = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture_stream = nullptr;  // graphs are captured here, launched on the caller's stream
  int sched_blocks = 0;                    // blocks of the solver's grid-stride kernels (0: automatic)
  int stall_copies = 0;                    // copy-stall test knob (mlpcg_solver_set_copy_stall)
  CUtensorMap qmap[3];                     // the three search-direction buffers, for the TMA SpMV
  bool qmap_ok = false;
  bool dependent_launch = true;            // programmatic edges in the captured loop body
  bool fused_dots = true;                  // NPSD: z . Ap in the preconditioner's level-0 epilogue
  int64_t zcap = 0;                        // tiles of V.zpart
  int dependent_edges = 0;                 // edges converted in the current graph
};

struct mlpcg_batch {
  std::vector<mlpcg_solver *> solvers;
  std::vector<cudaStream_t> streams;   // one per system: the graph's parallel branches
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static size_t al256s(size_t b) { return (b + 255) / 256 * 256; }

// CTAs of the once-per-solve kernels (prepare, initial and true residual, finalize): the full
// reduction grid whatever the schedule of the iteration kernels, so that these single passes
// keep enough loads in flight
static unsigned full_grid(const Vecs &V) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(RB_MAX, ((int64_t)V.ngroups + RT - 1) / RT));
}

static FastDiv make_fastdiv(uint32_t d) {
  int l = 0;
  while ((1ull << l) < d) ++l;  // ceil(log2 d)
  const uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
  FastDiv f;
  f.m = (uint32_t)m;
  f.s1 = l < 1 ? (uint32_t)l : 1u;
  f.s2 = l > 1 ? (uint32_t)(l - 1) : 0u;
  return f;
}

static size_t solver_layout(mlpcg_solver &s, char *base) {
  size_t off = 0;
  auto take = [&](size_t b) -> void * {
    void *p = base ? base + off : nullptr;
    off += al256s(b);
    return p;
  };
  const int64_t n = cells(s.n1, s.n2, s.n3);
  const int nslots = s.method == M_NPSD ? 3 : 2;
  const int naps = s.method == M_NPSD ? 3 : 1;
  s.V.code = (uint8_t *)take(n);
  s.V.xd = (float2 *)take(n * 8);
  s.V.bd = (float2 *)take(n * 8);
  s.V.r = (float *)take(n * 4);
  s.V.z = (float *)take(n * 4);
  s.V.p = (float *)take(nslots * n * 4);
  s.V.Ap = (float *)take(naps * n * 4);
  s.V.part = (double *)take(NRED * RB_MAX * 8);
  s.V.zpart = s.zcap > 0 ? (double *)take(2 * s.zcap * 8) : nullptr;
  s.V.hist = (double *)take((s.max_it + 1) * 8);
  s.V.st = (State *)take(sizeof(State));
  return off;
}

static void destroy_graph(mlpcg_solver *s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->exec = nullptr;
  s->graph = nullptr;
}

// Turns the captured loop body's kernel-to-kernel edges into programmatic ones:
// the downstream kernel's blocks may be scheduled as the upstream kernel's
// blocks exit, and they wait in dependent_launch_enter() for the upstream
// grid's completion and writes -- the launch of each kernel of an iteration
// overlaps its predecessor's tail, the order of every memory access is
// unchanged.  Only edges into a
// kernel with a single incoming edge are converted (the batch's join keeps its
// ordinary edges).  Returns the number of converted edges, or -1 when the graph
// API refused (the edges already converted stay, the refused one is restored).
static int make_dependent_edges(cudaGraph_t body) {
  size_t ne = 0;
  if (cudaGraphGetEdges(body, nullptr, nullptr, nullptr, &ne) != cudaSuccess) return -1;
  std::vector<cudaGraphNode_t> from(ne), to(ne);
  std::vector<cudaGraphEdgeData> data(ne);
  if (ne && cudaGraphGetEdges(body, from.data(), to.data(), data.data(), &ne) != cudaSuccess) return -1;
  int converted = 0;
  for (size_t e = 0; e < ne; ++e) {
    size_t indeg = 0;
    for (size_t f = 0; f < ne; ++f) indeg += to[f] == to[e];
    cudaGraphNodeType a, b;
    if (cudaGraphNodeGetType(from[e], &a) != cudaSuccess || cudaGraphNodeGetType(to[e], &b) != cudaSuccess)
      return -1;
    if (a != cudaGraphNodeTypeKernel || b != cudaGraphNodeTypeKernel || indeg != 1 ||
        data[e].type != cudaGraphDependencyTypeDefault || data[e].from_port != cudaGraphKernelNodePortDefault)
      continue;
    cudaGraphEdgeData pe{};
    pe.from_port = cudaGraphKernelNodePortProgrammatic;
    pe.type = cudaGraphDependencyTypeProgrammatic;
    if (cudaGraphRemoveDependencies(body, &from[e], &to[e], &data[e], 1) != cudaSuccess) return -1;
    if (cudaGraphAddDependencies(body, &from[e], &to[e], &pe, 1) != cudaSuccess) {
      cudaGraphAddDependencies(body, &from[e], &to[e], &data[e], 1);
      return -1;
    }
    ++converted;
  }
  return converted;
}

// state reset, operator codes, b and x0 as pairs, the initial residual
static int start_solve(mlpcg_solver *s, cudaStream_t st) {
  Vecs &V = s->V;
  V.perr = precond_copy_flag(s->plan);
  k_reset<<<1, 32, 0, st>>>(V.st, s->max_it, s->true_every, s->method, s->tol, s->stall_copies);
  k_prepare<<<full_grid(V), RT, 0, st>>>(V);
  k_init<<<full_grid(V), RT, 0, st>>>(V);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

// a plan whose level-0 post-block computes the solver's products (npsd z . Ap, npcg r . z;
// precond_zdots_tiles)
static bool uses_fused_dots(const mlpcg_solver *s) {
  return s->fused_dots && s->V.zpart && s->zcap > 0 && precond_zdots_tiles(s->plan) == s->zcap;
}

static int enqueue_body(mlpcg_solver *s, cudaStream_t st, cudaGraphConditionalHandle h, int use_handle) {
  Vecs &V = s->V;
  const unsigned nb = (unsigned)V.nblk;
  State *S = V.st;
  // z = M (r / ||r||): the scale is read from the device state; the kernels
  // return at once once this system has stopped (its status word is nonzero)
  const bool zdots = uses_fused_dots(s);
  const ZDots zd = s->method == M_NPSD ? ZDots{V.Ap, &S->head, &S->it, V.zpart, V.n, 0}
                                        : ZDots{V.r, &S->head, &S->it, V.zpart, V.n, 1};
  int rc = precond_apply_gated(s->plan, V.r, &S->rscale, V.z, &S->status, st, zdots ? &zd : nullptr);
  if (rc) return rc;
  if (s->method == M_NPSD) {
    if (zdots) k_sd_dots_tiles<<<ZT_BLOCKS, RT, 0, st>>>(V);
    else k_sd_dots<<<nb, RT, 0, st>>>(V);
    k_sd_qform<<<nb, RT, 0, st>>>(V);
    if (s->qmap_ok) k_sd_spmv_tma<<<nb, RT, 0, st>>>(V, s->qmap[0], s->qmap[1], s->qmap[2]);
    else k_sd_spmv<<<nb, RT, 0, st>>>(V);
  } else {
    if (zdots) k_cg_rz_tiles<<<ZT_BLOCKS, RT, 0, st>>>(V);
    else k_cg_rz<<<nb, RT, 0, st>>>(V);
    k_cg_pspmv<<<nb, RT, 0, st>>>(V);
  }
  k_update<<<nb, RT, 0, st>>>(V);
  k_true_residual_control<<<full_grid(V), RT, 0, st>>>(V, h, use_handle);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

extern "C" {

int mlpcg_solver_create(int N1, int N2, int N3, const mlpcg_precond *plan, int method, int max_it, double tol,
                        int true_every, mlpcg_solver **out) {
  clear_error();
  MLPCG_REQUIRE(out && plan, MLPCG_ERR_ARG, "solver_create: NULL argument");
  MLPCG_REQUIRE(method == M_NPSD || method == M_NPCG, MLPCG_ERR_ARG, "solver_create: method must be 0 (npsd) or 1 (npcg)");
  MLPCG_REQUIRE(max_it >= 1 && max_it <= 1000000, MLPCG_ERR_ARG, "solver_create: max_it out of range");
  MLPCG_REQUIRE(tol > 0.0, MLPCG_ERR_ARG, "solver_create: tol must be > 0");
  MLPCG_REQUIRE(N1 >= 1 && N2 >= 1 && N3 >= 1, MLPCG_ERR_SHAPE, "solver_create: bad grid");
  MLPCG_REQUIRE(N3 % 4 == 0, MLPCG_ERR_SHAPE, "solver_create: N3 (%d) must be a multiple of 4", N3);
  MLPCG_REQUIRE(cells(N1, N2, N3) < ((int64_t)1 << 31), MLPCG_ERR_SHAPE, "solver_create: grid must have < 2^31 cells");
  int p1 = 0, p2 = 0, p3 = 0, pf = 0;
  if (int rc = mlpcg_precond_level_info(plan, 0, &p1, &p2, &p3, &pf)) return rc;
  MLPCG_REQUIRE(p1 == N1 && p2 == N2 && p3 == N3, MLPCG_ERR_SHAPE,
                "solver_create: the plan's grid %dx%dx%d is not the solver's %dx%dx%d", p1, p2, p3, N1, N2, N3);
  auto *s = new mlpcg_solver();
  s->n1 = N1; s->n2 = N2; s->n3 = N3;
  s->method = method; s->max_it = max_it; s->tol = tol; s->true_every = true_every;
  s->plan = plan;
  s->zcap = precond_level0_tiles(plan);
  s->bytes = solver_layout(*s, nullptr);
  *out = s;
  return MLPCG_OK;
}

size_t mlpcg_solver_workspace(const mlpcg_solver *s) { return s ? s->bytes : 0; }

void mlpcg_solver_destroy(mlpcg_solver *s) {
  if (!s) return;
  destroy_graph(s);
  if (s->capture_stream) cudaStreamDestroy(s->capture_stream);
  delete s;
}

int mlpcg_solver_bind(mlpcg_solver *s, void *workspace, size_t workspace_bytes, const uint8_t *flags,
                      const double *b, double *x) {
  clear_error();
  MLPCG_REQUIRE(s && workspace && flags && b && x, MLPCG_ERR_ARG, "solver_bind: NULL argument");
  MLPCG_REQUIRE(workspace_bytes >= s->bytes, MLPCG_ERR_WORKSPACE, "solver workspace too small: %zu < %zu",
                workspace_bytes, s->bytes);
  MLPCG_REQUIRE(((uintptr_t)workspace & 255) == 0, MLPCG_ERR_ALIGN, "solver workspace must be 256-byte aligned");
  // the kernels read flags 4 cells and b, x 2 doubles at a time
  MLPCG_REQUIRE(((uintptr_t)flags & 3) == 0 && ((uintptr_t)b & 15) == 0 && ((uintptr_t)x & 15) == 0, MLPCG_ERR_ALIGN,
                "solver_bind: flags must be 4-byte and b, x 16-byte aligned");
  destroy_graph(s);
  solver_layout(*s, (char *)workspace);
  Vecs &V = s->V;
  V.flags = flags; V.b = b; V.x = x;
  V.n1 = s->n1; V.n2 = s->n2; V.n3 = s->n3;
  V.n = cells(s->n1, s->n2, s->n3);
  V.ngroups = (uint32_t)(V.n / 4);
  V.ztiles = s->zcap;
  V.fd3 = make_fastdiv((uint32_t)s->n3);
  V.fd2 = make_fastdiv((uint32_t)s->n2);
  int64_t nb = ((int64_t)V.ngroups + RT * UNR - 1) / (RT * UNR);
  if (s->sched_blocks > 0) nb = std::min<int64_t>(nb, s->sched_blocks);
  V.nblk = (int)(nb < 1 ? 1 : (nb > RB_MAX ? RB_MAX : nb));
  // tensor maps of the three search-direction buffers for the TMA-tiled npsd SpMV
  s->qmap_ok = V.n3 % 8 == 0;
  for (int k = 0; k < 3 && s->qmap_ok; ++k)
    s->qmap_ok = encode_grid_map(&s->qmap[k], V.p + (size_t)k * V.n, V.n1, V.n2, V.n3, SBZ, SBY, SBX);
  s->bound = true;
  return MLPCG_OK;
}

// Resets the state and x's residual, then runs the loop: as one CUDA graph
// (use_graph = 1; built on the first call and reused) or as plain launches
// with one host check per iteration (use_graph = 0).  Asynchronous for the
// graph; mlpcg_solver_result() synchronises.
static int solve_impl(mlpcg_solver *s, int use_graph, int zero_guess, cudaStream_t st) {
  Vecs &V = s->V;
  V.zero_guess = zero_guess;  // read by k_prepare and k_finalize, which run outside the graph
  if (int rc0 = start_solve(s, st)) return rc0;
  if (!use_graph) {
    for (int it = 0; it < s->max_it; ++it) {
      int status = 0;
      MLPCG_CUDA_CHECK(cudaMemcpyAsync(&status, &V.st->status, sizeof(int), cudaMemcpyDeviceToHost, st));
      MLPCG_CUDA_CHECK(cudaStreamSynchronize(st));
      if (status != ST_RUNNING) break;
      int rc = enqueue_body(s, st, 0, 0);
      if (rc) return rc;
    }
    k_finalize<<<full_grid(V), RT, 0, st>>>(V);
    MLPCG_LAUNCH_CHECK();
    return MLPCG_OK;
  }
  // capture with programmatic edges when enabled; a graph the runtime will not
  // instantiate with them is captured again with ordinary edges
  for (int dep = s->dependent_launch ? 1 : 0; !s->exec && dep >= 0; --dep) {
    if (!s->capture_stream)
      MLPCG_CUDA_CHECK(cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking));
    MLPCG_CUDA_CHECK(cudaGraphCreate(&s->graph, 0));
    cudaGraphConditionalHandle h;
    MLPCG_CUDA_CHECK(cudaGraphConditionalHandleCreate(&h, s->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MLPCG_CUDA_CHECK(cudaGraphAddNode(&node, s->graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs = s->capture_stream;
    MLPCG_CUDA_CHECK(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_body(s, cs, h, 1);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &captured);
    if (rc) { destroy_graph(s); return rc; }
    if (e != cudaSuccess) { destroy_graph(s); MLPCG_CUDA_CHECK(e); }
    s->dependent_edges = dep ? make_dependent_edges(body) : 0;
    const cudaError_t ei = s->dependent_edges < 0 ? cudaErrorNotSupported
                                                  : cudaGraphInstantiate(&s->exec, s->graph, 0);
    if (ei != cudaSuccess) {
      s->exec = nullptr;
      destroy_graph(s);
      s->dependent_edges = 0;
      cudaGetLastError();
      if (!dep) MLPCG_CUDA_CHECK(ei);
    }
  }
  // the loop only starts when the initial residual is not already converged:
  // the body's first kernels see status != RUNNING and the control step
  // ends the loop after one pass.
  MLPCG_CUDA_CHECK(cudaGraphLaunch(s->exec, st));
  k_finalize<<<full_grid(V), RT, 0, st>>>(V);
  MLPCG_LAUNCH_CHECK();
  return MLPCG_OK;
}

int mlpcg_solver_solve(mlpcg_solver *s, int use_graph, void *stream) {
  clear_error();
  MLPCG_REQUIRE(s && s->bound, MLPCG_ERR_ARG, "solver_solve: solver not bound");
  return solve_impl(s, use_graph, 0, as_stream(stream));
}

int mlpcg_solver_solve_zero_guess(mlpcg_solver *s, int use_graph, void *stream) {
  clear_error();
  MLPCG_REQUIRE(s && s->bound, MLPCG_ERR_ARG, "solver_solve_zero_guess: solver not bound");
  return solve_impl(s, use_graph, 1, as_stream(stream));
}

int mlpcg_solver_result(const mlpcg_solver *s, int *iters, int *status, double *rel_res, double *history,
                        void *stream) {
  clear_error();
  MLPCG_REQUIRE(s && s->bound, MLPCG_ERR_ARG, "solver_result: solver not bound");
  cudaStream_t st = as_stream(stream);
  State S;
  MLPCG_CUDA_CHECK(cudaMemcpyAsync(&S, s->V.st, sizeof(State), cudaMemcpyDeviceToHost, st));
  if (history)
    MLPCG_CUDA_CHECK(cudaMemcpyAsync(history, s->V.hist, (s->max_it + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
  MLPCG_CUDA_CHECK(cudaStreamSynchronize(st));
  if (iters) *iters = S.it;
  if (status) *status = S.status;
  if (rel_res) *rel_res = S.rel;
  return MLPCG_OK;
}

int mlpcg_solver_set_schedule(mlpcg_solver *s, int blocks) {
  clear_error();
  MLPCG_REQUIRE(s, MLPCG_ERR_ARG, "solver_set_schedule: NULL solver");
  MLPCG_REQUIRE(blocks >= 0 && blocks <= RB_MAX, MLPCG_ERR_ARG, "solver_set_schedule: blocks %d out of [0, %d]",
                blocks, RB_MAX);
  s->sched_blocks = blocks;
  if (s->bound) {
    Vecs &V = s->V;
    int64_t nb = ((int64_t)V.ngroups + RT * UNR - 1) / (RT * UNR);
    if (blocks > 0) nb = std::min<int64_t>(nb, blocks);
    V.nblk = (int)(nb < 1 ? 1 : (nb > RB_MAX ? RB_MAX : nb));
    destroy_graph(s);  // recaptured with the new grid on the next solve
  }
  return MLPCG_OK;
}

int mlpcg_solver_set_copy_stall(mlpcg_solver *s, int on) {
  clear_error();
  MLPCG_REQUIRE(s, MLPCG_ERR_ARG, "solver_set_copy_stall: NULL solver");
  s->stall_copies = on ? 1 : 0;
  return MLPCG_OK;
}

int mlpcg_solver_set_dependent_launch(mlpcg_solver *s, int on) {
  clear_error();
  MLPCG_REQUIRE(s, MLPCG_ERR_ARG, "solver_set_dependent_launch: NULL solver");
  if (s->dependent_launch != (on != 0)) destroy_graph(s);  // recaptured on the next solve
  s->dependent_launch = on != 0;
  return MLPCG_OK;
}

int mlpcg_solver_set_fused_dots(mlpcg_solver *s, int on) {
  clear_error();
  MLPCG_REQUIRE(s, MLPCG_ERR_ARG, "solver_set_fused_dots: NULL solver");
  if (s->fused_dots != (on != 0)) destroy_graph(s);  // recaptured on the next solve
  s->fused_dots = on != 0;
  return MLPCG_OK;
}

int mlpcg_solver_fused_dots(const mlpcg_solver *s, int *active) {
  clear_error();
  MLPCG_REQUIRE(s && active, MLPCG_ERR_ARG, "solver_fused_dots: NULL argument");
  *active = s->bound && uses_fused_dots(s) ? 1 : 0;
  return MLPCG_OK;
}

int mlpcg_solver_dependent_edges(const mlpcg_solver *s, int *edges) {
  clear_error();
  MLPCG_REQUIRE(s && edges, MLPCG_ERR_ARG, "solver_dependent_edges: NULL argument");
  *edges = s->exec ? s->dependent_edges : 0;
  return MLPCG_OK;
}

int mlpcg_solver_get_schedule(const mlpcg_solver *s, int *blocks_in_use) {
  clear_error();
  MLPCG_REQUIRE(s && blocks_in_use, MLPCG_ERR_ARG, "solver_get_schedule: NULL argument");
  *blocks_in_use = s->bound ? s->V.nblk : s->sched_blocks;
  return MLPCG_OK;
}

int mlpcg_batch_create(mlpcg_solver *const *solvers, int count, mlpcg_batch **out) {
  clear_error();
  MLPCG_REQUIRE(out && solvers, MLPCG_ERR_ARG, "batch_create: NULL argument");
  *out = nullptr;
  MLPCG_REQUIRE(count >= 1 && count <= kMaxBatch, MLPCG_ERR_ARG, "batch_create: count %d out of [1, %d]", count,
                kMaxBatch);
  for (int i = 0; i < count; ++i) {
    MLPCG_REQUIRE(solvers[i] && solvers[i]->bound, MLPCG_ERR_ARG, "batch_create: solver %d is NULL or not bound", i);
    for (int j = 0; j < i; ++j)
      MLPCG_REQUIRE(solvers[j] != solvers[i], MLPCG_ERR_ARG, "batch_create: solver %d appears twice", i);
  }
  auto *b = new mlpcg_batch();
  b->solvers.assign(solvers, solvers + count);
  *out = b;
  return MLPCG_OK;
}

static void destroy_batch_graph(mlpcg_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

void mlpcg_batch_destroy(mlpcg_batch *b) {
  if (!b) return;
  destroy_batch_graph(b);
  for (auto st : b->streams) cudaStreamDestroy(st);
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  delete b;
}

int mlpcg_batch_solve(mlpcg_batch *b, void *stream) {
  clear_error();
  MLPCG_REQUIRE(b, MLPCG_ERR_ARG, "batch_solve: NULL batch");
  cudaStream_t st = as_stream(stream);
  const int K = (int)b->solvers.size();
  for (auto *s : b->solvers) {
    MLPCG_REQUIRE(s->bound, MLPCG_ERR_ARG, "batch_solve: a solver is no longer bound");
    s->V.zero_guess = 0;  // batches start from each solver's x
    if (int rc = start_solve(s, st)) return rc;
  }
  // ordinary edges: with the systems' chains running side by side, programmatic edges were
  // measured slower for the batch (16 systems of 64^3-192^3: 14.54 vs 14.42 ms)
  if (!b->exec) {
    if (!b->capture_stream) {
      MLPCG_CUDA_CHECK(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
      MLPCG_CUDA_CHECK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
      b->streams.resize(K, nullptr);
      b->joins.resize(K, nullptr);
      for (int i = 0; i < K; ++i) {
        MLPCG_CUDA_CHECK(cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking));
        MLPCG_CUDA_CHECK(cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming));
      }
    }
    MLPCG_CUDA_CHECK(cudaGraphCreate(&b->graph, 0));
    cudaGraphConditionalHandle h;
    MLPCG_CUDA_CHECK(cudaGraphConditionalHandleCreate(&h, b->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MLPCG_CUDA_CHECK(cudaGraphAddNode(&node, b->graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs = b->capture_stream;
    MLPCG_CUDA_CHECK(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    // one branch per system: each waits on the fork, runs its iteration, joins
    int rc = 0;
    cudaError_t e = cudaEventRecord(b->fork, cs);
    BatchStates B{};
    B.count = K;
    for (int i = 0; i < K && !rc && e == cudaSuccess; ++i) {
      B.st[i] = b->solvers[i]->V.st;
      e = cudaStreamWaitEvent(b->streams[i], b->fork, 0);
      if (e == cudaSuccess) rc = enqueue_body(b->solvers[i], b->streams[i], h, 0);
      if (!rc && e == cudaSuccess) e = cudaEventRecord(b->joins[i], b->streams[i]);
      if (!rc && e == cudaSuccess) e = cudaStreamWaitEvent(cs, b->joins[i], 0);
    }
    if (!rc && e == cudaSuccess) {
      k_batch_control<<<1, kMaxBatch, 0, cs>>>(B, h);
      e = cudaGetLastError();
    }
    cudaGraph_t captured = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &captured);
    if (rc) { destroy_batch_graph(b); return rc; }
    if (e != cudaSuccess) { destroy_batch_graph(b); MLPCG_CUDA_CHECK(e); }
    if (e2 != cudaSuccess) { destroy_batch_graph(b); MLPCG_CUDA_CHECK(e2); }
    const cudaError_t ei = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (ei != cudaSuccess) {
      b->exec = nullptr;
      destroy_batch_graph(b);
      MLPCG_CUDA_CHECK(ei);
    }
  }
  MLPCG_CUDA_CHECK(cudaGraphLaunch(b->exec, st));
  for (auto *s : b->solvers) {
    k_finalize<<<full_grid(s->V), RT, 0, st>>>(s->V);
    MLPCG_LAUNCH_CHECK();
  }
  return MLPCG_OK;
}

}  // extern "C"
