// CPU comparator of the oracle package -- TEST AND BASELINE INFRASTRUCTURE ONLY.
//
// The reference sets its network-preconditioned solves beside an AMGCL solve on
// the host (cxx_src/lib/AMGCLSolver.h:58-128, bound as pyamgcl.solve in
// cxx_src/pyamgcl.cpp:9-16 and called by cg_tests.py:343-346): algebraic
// multigrid with smoothed-aggregation coarsening and SPAI-0 relaxation as the
// preconditioner of an FP64 conjugate-gradient solve, x0 = 0, stopping at
// |r| / |b| < max(tol, atol / |b|).  AMGCL itself is an un-vendored submodule
// (no source, no pinned commit), so this file restates the published methods
// with parameters of its own, and its iteration counts are not pinned to
// AMGCL's:
//
//  * coarsening: smoothed aggregation (Vanek, Mandel, Brezina, Computing 56,
//    1996).  Strong couplings a_ij^2 > eps^2 |a_ii a_jj|, eps = 0.08 on the
//    finest level, halved on each coarser one; greedy aggregation in two
//    passes (a node whose strong neighbours are all free starts an aggregate
//    with them; every other node joins a neighbouring aggregate); tentative
//    prolongation = aggregate indicator; smoothed prolongation
//    P = (I - w D_F^-1 A_F) P_tent with the filtered matrix A_F (weak
//    couplings added to the diagonal) and w = (4/3) / rho, rho bounded by the
//    Gershgorin bound of D_F^-1 A_F; restriction R = P^T; Galerkin coarse
//    operator R A P; coarsening stops at 1,000 unknowns or 20 levels, where a
//    dense Cholesky factorisation solves exactly (a singular direction --
//    a pivot at round-off level -- is left at zero);
//  * relaxation: SPAI-0 (Broker, Grote, 2002), the diagonal approximate
//    inverse m_i = a_ii / sum_j a_ij^2, one sweep before and one after the
//    coarse correction, so the V-cycle is a symmetric operator and plain CG
//    applies;
//  * CG: FP64, OpenMP-parallel products; reductions in a fixed order, so a
//    solve repeats bit for bit with the same thread count.
//
// C entry points (ctypes, oracle/amg.py): amg_cg_solve and amg_apply.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct Csr {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> ptr;
  std::vector<int32_t> col;
  std::vector<double> val;
  int64_t nnz() const { return (int64_t)col.size(); }
};

// y = A x
void spmv(const Csr &A, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.rows; ++i) {
    double s = 0.0;
    for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
    y[i] = s;
  }
}

// r = b - A x
void residual(const Csr &A, const double *x, const double *b, double *r) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.rows; ++i) {
    double s = b[i];
    for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s -= A.val[k] * x[A.col[k]];
    r[i] = s;
  }
}

// y += A x
void spmv_add(const Csr &A, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.rows; ++i) {
    double s = 0.0;
    for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
    y[i] += s;
  }
}

// x . y from per-thread partial sums over fixed ranges, added in thread order:
// the same bits on every run with the same thread count
double dot(const double *x, const double *y, int64_t n) {
  std::vector<double> part(omp_get_max_threads(), 0.0);
  int used = 1;
#pragma omp parallel num_threads((int)part.size())
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    double s = 0.0;
    for (int64_t i = lo; i < hi; ++i) s += x[i] * y[i];
    part[t] = s;
    if (t == 0) used = nt;
  }
  double s = 0.0;
  for (int t = 0; t < used; ++t) s += part[t];
  return s;
}

std::vector<int64_t> row_bounds(int64_t rows, int parts) {
  std::vector<int64_t> b(parts + 1);
  for (int t = 0; t <= parts; ++t) b[t] = rows * t / parts;
  return b;
}

// A^T, in parallel over row blocks: each block counts its entries per column,
// and a column's entries are placed block after block, rows in order -- the
// same arrays as a sequential transpose
Csr transpose(const Csr &A) {
  const int parts = omp_get_max_threads();
  const std::vector<int64_t> bounds = row_bounds(A.rows, parts);
  Csr T;
  T.rows = A.cols;
  T.cols = A.rows;
  T.ptr.assign(T.rows + 1, 0);
  T.col.resize(A.nnz());
  T.val.resize(A.nnz());
  std::vector<int64_t> pos((size_t)parts * A.cols, 0);
#pragma omp parallel num_threads(parts)
  {
    const int t = omp_get_thread_num();
    int64_t *cnt = pos.data() + (size_t)t * A.cols;
    for (int64_t i = bounds[t]; i < bounds[t + 1]; ++i)
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) ++cnt[A.col[k]];
#pragma omp barrier
#pragma omp single
    {
      int64_t run = 0;
      for (int64_t c = 0; c < A.cols; ++c) {
        T.ptr[c] = run;
        for (int u = 0; u < parts; ++u) {
          const int64_t v = pos[(size_t)u * A.cols + c];
          pos[(size_t)u * A.cols + c] = run;
          run += v;
        }
      }
      T.ptr[A.cols] = run;
    }
    for (int64_t i = bounds[t]; i < bounds[t + 1]; ++i)
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        const int64_t p = cnt[A.col[k]]++;
        T.col[p] = (int32_t)i;
        T.val[p] = A.val[k];
      }
  }
  return T;
}

// rows [lo, hi) of a product built by one thread: entries appended per row,
// merged through a marker array over the columns
struct RowBlock {
  std::vector<int64_t> len;
  std::vector<int32_t> col;
  std::vector<double> val;
};

// assembles per-thread row blocks (thread t owns rows [bounds[t], bounds[t+1]))
Csr gather_blocks(std::vector<RowBlock> &blk, const std::vector<int64_t> &bounds, int64_t rows, int64_t cols) {
  Csr C;
  C.rows = rows;
  C.cols = cols;
  C.ptr.assign(rows + 1, 0);
  for (size_t t = 0; t < blk.size(); ++t)
    for (int64_t i = bounds[t]; i < bounds[t + 1]; ++i) C.ptr[i + 1] = blk[t].len[i - bounds[t]];
  for (int64_t i = 0; i < rows; ++i) C.ptr[i + 1] += C.ptr[i];
  C.col.resize(C.ptr[rows]);
  C.val.resize(C.ptr[rows]);
#pragma omp parallel for schedule(static, 1)
  for (int t = 0; t < (int)blk.size(); ++t) {
    const int64_t off = C.ptr[bounds[t]];
    std::copy(blk[t].col.begin(), blk[t].col.end(), C.col.begin() + off);
    std::copy(blk[t].val.begin(), blk[t].val.end(), C.val.begin() + off);
    blk[t] = RowBlock();
  }
  return C;
}

// Galerkin product R A P, one coarse row at a time: sum over the fine rows i of
// R's row I, over A's row i, over P's row j
Csr galerkin(const Csr &R, const Csr &A, const Csr &P) {
  const int parts = omp_get_max_threads();
  const std::vector<int64_t> bounds = row_bounds(R.rows, parts);
  std::vector<RowBlock> blk(parts);
#pragma omp parallel num_threads(parts)
  {
    const int t = omp_get_thread_num();
    RowBlock &out = blk[t];
    out.len.reserve(bounds[t + 1] - bounds[t]);
    out.col.reserve((bounds[t + 1] - bounds[t]) * 27);
    out.val.reserve((bounds[t + 1] - bounds[t]) * 27);
    std::vector<int64_t> marker(P.cols, -1);
    for (int64_t I = bounds[t]; I < bounds[t + 1]; ++I) {
      const int64_t start = (int64_t)out.col.size();
      for (int64_t a = R.ptr[I]; a < R.ptr[I + 1]; ++a) {
        const int64_t i = R.col[a];
        const double ri = R.val[a];
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
          const int64_t j = A.col[k];
          const double rik = ri * A.val[k];
          for (int64_t q = P.ptr[j]; q < P.ptr[j + 1]; ++q) {
            const int32_t K = P.col[q];
            if (marker[K] < start) {
              marker[K] = (int64_t)out.col.size();
              out.col.push_back(K);
              out.val.push_back(rik * P.val[q]);
            } else {
              out.val[marker[K]] += rik * P.val[q];
            }
          }
        }
      }
      out.len.push_back((int64_t)out.col.size() - start);
    }
  }
  return gather_blocks(blk, bounds, R.rows, P.cols);
}

struct Level {
  Csr A, P, R;
  std::vector<double> m;        // SPAI-0 weights
  std::vector<double> b, x, r;  // V-cycle vectors of this level
};

struct Hierarchy {
  std::vector<Level> lv;
  std::vector<double> chol;   // dense lower factor of the coarsest operator (row-major)
  std::vector<char> singular;  // coarsest directions left at zero
  int64_t nc = 0;
  double op_complexity = 0.0;

  static constexpr int64_t kCoarseEnough = 1000;
  static constexpr int kMaxLevels = 20;

  void build(Csr A0) {
    lv.clear();
    lv.emplace_back();
    lv[0].A = std::move(A0);
    double eps = 0.08;
    while ((int)lv.size() < kMaxLevels && lv.back().A.rows > kCoarseEnough) {
      Level &L = lv.back();
      Csr Ac;
      if (!coarsen(L, eps, Ac)) break;
      lv.emplace_back();
      lv.back().A = std::move(Ac);
      eps *= 0.5;
    }
    int64_t nnz_all = 0;
    for (Level &L : lv) {
      nnz_all += L.A.nnz();
      const int64_t n = L.A.rows;
      L.m.assign(n, 0.0);
      L.b.assign(n, 0.0);
      L.x.assign(n, 0.0);
      L.r.assign(n, 0.0);
      const Csr &A = L.A;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        double d = 0.0, s = 0.0;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
          s += A.val[k] * A.val[k];
          if (A.col[k] == i) d = A.val[k];
        }
        L.m[i] = s > 0.0 ? d / s : 0.0;
      }
    }
    op_complexity = (double)nnz_all / (double)std::max<int64_t>(1, lv[0].A.nnz());
    factor_coarsest();
  }

  // one level of smoothed aggregation; false when no coarser level can be formed
  bool coarsen(Level &L, double eps, Csr &Ac) {
    const Csr &A = L.A;
    const int64_t n = A.rows;
    std::vector<double> d(n, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
        if (A.col[k] == i) d[i] = A.val[k];
    std::vector<char> strong(A.nnz(), 0);
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        const int64_t j = A.col[k];
        strong[k] = j != i && A.val[k] * A.val[k] > eps2 * std::fabs(d[i] * d[j]);
      }
    // aggregation: -1 free, -2 no strong coupling (left out of every aggregate)
    std::vector<int32_t> agg(n, -1);
    for (int64_t i = 0; i < n; ++i) {
      bool any = false;
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1] && !any; ++k) any = strong[k];
      if (!any) agg[i] = -2;
    }
    int32_t count = 0;
    for (int64_t i = 0; i < n; ++i) {
      if (agg[i] != -1) continue;
      bool free_nb = true;
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1] && free_nb; ++k)
        if (strong[k] && agg[A.col[k]] != -1) free_nb = false;
      if (!free_nb) continue;
      const int32_t c = count++;
      agg[i] = c;
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
        if (strong[k]) agg[A.col[k]] = c;
    }
    const std::vector<int32_t> first(agg);
    for (int64_t i = 0; i < n; ++i) {
      if (agg[i] != -1) continue;
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
        if (strong[k] && first[A.col[k]] >= 0) {
          agg[i] = first[A.col[k]];
          break;
        }
      if (agg[i] == -1) {
        const int32_t c = count++;
        agg[i] = c;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
          if (strong[k] && agg[A.col[k]] == -1) agg[A.col[k]] = c;
      }
    }
    if (count == 0 || count >= n) return false;
    // filtered diagonal and the Gershgorin bound of D_F^-1 A_F
    std::vector<double> dF(n, 0.0);
    double rho = 0.0;
#pragma omp parallel for schedule(static) reduction(max : rho)
    for (int64_t i = 0; i < n; ++i) {
      double di = d[i], off = 0.0;
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
        if (A.col[k] != i) {
          if (strong[k]) off += std::fabs(A.val[k]);
          else di += A.val[k];
        }
      dF[i] = di;
      if (di != 0.0) rho = std::max(rho, (std::fabs(di) + off) / std::fabs(di));
    }
    const double w = rho > 0.0 ? (4.0 / 3.0) / rho : 0.0;
    // smoothed prolongation, row i: e_agg(i) - (w / dF_i) sum_j aF_ij e_agg(j)
    const int parts = omp_get_max_threads();
    const std::vector<int64_t> bounds = row_bounds(n, parts);
    std::vector<RowBlock> blk(parts);
#pragma omp parallel num_threads(parts)
    {
      const int t = omp_get_thread_num();
      RowBlock &out = blk[t];
      // at most one entry per coupling of the row, plus its own aggregate
      const int64_t cap = A.ptr[bounds[t + 1]] - A.ptr[bounds[t]] + (bounds[t + 1] - bounds[t]);
      out.len.reserve(bounds[t + 1] - bounds[t]);
      out.col.reserve(cap);
      out.val.reserve(cap);
      for (int64_t i = bounds[t]; i < bounds[t + 1]; ++i) {
        const size_t start = out.col.size();
        auto add = [&](int32_t K, double v) {
          for (size_t q = start; q < out.col.size(); ++q)
            if (out.col[q] == K) {
              out.val[q] += v;
              return;
            }
          out.col.push_back(K);
          out.val.push_back(v);
        };
        if (agg[i] >= 0) add(agg[i], 1.0);
        if (dF[i] != 0.0) {
          const double s = w / dF[i];
          for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int64_t j = A.col[k];
            const double a = j == i ? dF[i] : (strong[k] ? A.val[k] : 0.0);
            if (a != 0.0 && agg[j] >= 0) add(agg[j], -s * a);
          }
        }
        out.len.push_back((int64_t)(out.col.size() - start));
      }
    }
    L.P = gather_blocks(blk, bounds, n, count);
    L.R = transpose(L.P);
    Ac = galerkin(L.R, A, L.P);
    return true;
  }

  void factor_coarsest() {
    const Csr &A = lv.back().A;
    nc = A.rows;
    chol.assign((size_t)nc * nc, 0.0);
    singular.assign(nc, 0);
    double dmax = 0.0;
    for (int64_t i = 0; i < nc; ++i)
      for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        chol[(size_t)i * nc + A.col[k]] += A.val[k];
        if (A.col[k] == i) dmax = std::max(dmax, std::fabs(A.val[k]));
      }
    const double floor = 1e-12 * std::max(dmax, 1e-300);
    for (int64_t j = 0; j < nc; ++j) {
      double *Lj = &chol[(size_t)j * nc];
      double s = Lj[j];
      for (int64_t k = 0; k < j; ++k) s -= Lj[k] * Lj[k];
      if (s <= floor) {
        singular[j] = 1;
        for (int64_t i = j; i < nc; ++i) chol[(size_t)i * nc + j] = 0.0;
        continue;
      }
      const double ljj = std::sqrt(s);
      Lj[j] = ljj;
#pragma omp parallel for schedule(static) if (nc - j > 256)
      for (int64_t i = j + 1; i < nc; ++i) {
        double *Li = &chol[(size_t)i * nc];
        double v = Li[j];
        for (int64_t k = 0; k < j; ++k) v -= Li[k] * Lj[k];
        Li[j] = v / ljj;
      }
    }
  }

  void solve_coarsest(const double *b, double *x) const {
    std::vector<double> y(nc, 0.0);
    for (int64_t i = 0; i < nc; ++i) {
      if (singular[i]) continue;
      const double *Li = &chol[(size_t)i * nc];
      double s = b[i];
      for (int64_t k = 0; k < i; ++k) s -= Li[k] * y[k];
      y[i] = s / Li[i];
    }
    for (int64_t i = nc - 1; i >= 0; --i) {
      if (singular[i]) {
        x[i] = 0.0;
        continue;
      }
      double s = y[i];
      for (int64_t k = i + 1; k < nc; ++k) s -= chol[(size_t)k * nc + i] * x[k];
      x[i] = s / chol[(size_t)i * nc + i];
    }
  }

  // x_l = B_l b_l (the V-cycle from a zero guess)
  void vcycle(size_t l) {
    Level &L = lv[l];
    const int64_t n = L.A.rows;
    if (l + 1 == lv.size()) {
      solve_coarsest(L.b.data(), L.x.data());
      return;
    }
    double *x = L.x.data(), *r = L.r.data();
    const double *b = L.b.data(), *m = L.m.data();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] = m[i] * b[i];
    residual(L.A, x, b, r);
    spmv(L.R, r, lv[l + 1].b.data());
    vcycle(l + 1);
    spmv_add(L.P, lv[l + 1].x.data(), x);
    residual(L.A, x, b, r);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] += m[i] * r[i];
  }

  void apply(const double *r, double *z) {
    Level &L = lv[0];
    std::copy(r, r + L.A.rows, L.b.begin());
    vcycle(0);
    std::copy(L.x.begin(), L.x.end(), z);
  }
};

Csr from_arrays(int64_t n, const int64_t *ptr, const int32_t *col, const double *val) {
  Csr A;
  A.rows = A.cols = n;
  A.ptr.assign(ptr, ptr + n + 1);
  A.col.assign(col, col + ptr[n]);
  A.val.assign(val, val + ptr[n]);
  return A;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

// Solves A x = b (x0 = 0) by CG with the smoothed-aggregation V-cycle as the
// preconditioner.  stats[0..7] = iterations, setup s, solve s, true relative
// residual |b - A x| / |b|, levels, operator complexity, coarsest unknowns,
// threads.  Returns 0, or -1 for bad arguments.
int amg_cg_solve(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *b, double *x,
                 double tol, double atol, int maxiter, int threads, double *stats) {
  if (n < 1 || !ptr || !col || !val || !b || !x || !stats || maxiter < 0) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  const auto t0 = std::chrono::steady_clock::now();
  Hierarchy H;
  H.build(from_arrays(n, ptr, col, val));
  const double setup_s = seconds_since(t0);
  const Csr &A = H.lv[0].A;
  const auto t1 = std::chrono::steady_clock::now();
  std::vector<double> r(b, b + n), z(n), p(n), q(n);
  std::fill(x, x + n, 0.0);
  const double bn = std::sqrt(dot(b, b, n));
  int it = 0;
  if (bn > 0.0) {
    const double eps = std::max(tol, atol / bn);
    H.apply(r.data(), z.data());
    std::copy(z.begin(), z.end(), p.begin());
    double rz = dot(r.data(), z.data(), n);
    while (it < maxiter) {
      spmv(A, p.data(), q.data());
      const double alpha = rz / dot(p.data(), q.data(), n);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        x[i] += alpha * p[i];
        r[i] -= alpha * q[i];
      }
      ++it;
      if (std::sqrt(dot(r.data(), r.data(), n)) < eps * bn) break;
      H.apply(r.data(), z.data());
      const double rz_new = dot(r.data(), z.data(), n);
      const double beta = rz_new / rz;
      rz = rz_new;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  }
  const double solve_s = seconds_since(t1);
  residual(A, x, b, r.data());
  stats[0] = it;
  stats[1] = setup_s;
  stats[2] = solve_s;
  stats[3] = bn > 0.0 ? std::sqrt(dot(r.data(), r.data(), n)) / bn : 0.0;
  stats[4] = (double)H.lv.size();
  stats[5] = H.op_complexity;
  stats[6] = (double)H.nc;
  stats[7] = omp_get_max_threads();
  return 0;
}

// The FP64 7-point matrix over the fluid cells of a flag grid (z fastest; the
// matrix of lib/discrete_laplacian.py:122-160 compressed to the fluid cells as
// lib/read_data.py:164-165 does): diagonal = number of fluid or air face
// neighbours, -1 between fluid face neighbours; cells outside the grid count as
// solid.  Entries of a row in the order -x, -y, -z, self, +z, +y, +x, which is
// increasing column order.  With fluid == nullptr only *nf and *nnz are
// returned (the sizes of the arrays of the second call).
int amg_fluid_matrix(int64_t n1, int64_t n2, int64_t n3, const uint8_t *flags, int64_t *nf, int64_t *nnz,
                     int64_t *fluid, int64_t *ptr, int32_t *col, double *val) {
  constexpr uint8_t kFluid = 2, kAir = 3;
  if (n1 < 1 || n2 < 1 || n3 < 1 || !flags || !nf || !nnz) return -1;
  const int64_t n = n1 * n2 * n3, s1 = n2 * n3, s2 = n3;
  auto neighbour = [&](int64_t c, int d, int64_t &nb) {
    const int64_t i = c / s1, j = (c / s2) % n2, k = c % n3;
    switch (d) {
      case 0: if (i == 0) return false; nb = c - s1; return true;
      case 1: if (j == 0) return false; nb = c - s2; return true;
      case 2: if (k == 0) return false; nb = c - 1; return true;
      case 3: if (k == n3 - 1) return false; nb = c + 1; return true;
      case 4: if (j == n2 - 1) return false; nb = c + s2; return true;
      default: if (i == n1 - 1) return false; nb = c + s1; return true;
    }
  };
  if (!fluid) {
    int64_t f = 0, e = 0;
    for (int64_t c = 0; c < n; ++c) {
      if (flags[c] != kFluid) continue;
      ++f;
      ++e;
      for (int d = 0; d < 6; ++d) {
        int64_t nb;
        if (neighbour(c, d, nb) && flags[nb] == kFluid) ++e;
      }
    }
    *nf = f;
    *nnz = e;
    return 0;
  }
  if (!ptr || !col || !val) return -1;
  std::vector<int32_t> index(n, -1);
  int64_t f = 0;
  for (int64_t c = 0; c < n; ++c)
    if (flags[c] == kFluid) {
      fluid[f] = c;
      index[c] = (int32_t)f++;
    }
  if (f != *nf) return -1;
  ptr[0] = 0;
  for (int64_t r = 0; r < f; ++r) {
    const int64_t c = fluid[r];
    int64_t e = 1;
    for (int d = 0; d < 6; ++d) {
      int64_t nb;
      if (neighbour(c, d, nb) && flags[nb] == kFluid) ++e;
    }
    ptr[r + 1] = ptr[r] + e;
  }
  if (ptr[f] != *nnz) return -1;
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < f; ++r) {
    const int64_t c = fluid[r];
    int64_t p = ptr[r];
    double diag = 0.0;
    int64_t nbs[6];
    bool in[6];
    for (int d = 0; d < 6; ++d) {
      in[d] = neighbour(c, d, nbs[d]);
      if (in[d] && (flags[nbs[d]] == kFluid || flags[nbs[d]] == kAir)) diag += 1.0;
    }
    for (int d = 0; d < 6; ++d) {
      if (d == 3) {
        col[p] = (int32_t)r;
        val[p++] = diag;
      }
      if (in[d] && flags[nbs[d]] == kFluid) {
        col[p] = index[nbs[d]];
        val[p++] = -1.0;
      }
    }
  }
  return 0;
}

// z = B r, one V-cycle of the hierarchy built from A; levels[0] = its depth.
int amg_apply(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *r, double *z,
              int *levels) {
  if (n < 1 || !ptr || !col || !val || !r || !z) return -1;
  Hierarchy H;
  H.build(from_arrays(n, ptr, col, val));
  H.apply(r, z);
  if (levels) *levels = (int)H.lv.size();
  return 0;
}

}  // extern "C"
