// ORACLE -- test infrastructure only.
//
// CPU restatement of the reference's batched ILU(0) / ParILU(0) / ISAI /
// BiCGSTAB arithmetic (aggarwal2000/Merging-ILU0, paths relative to
// Batched-ILU0-merged/ILU0_ISAI_bicgstab/).  Every floating-point operation is
// written out in the order the reference's CUDA kernels perform it, with the
// fused multiply-adds that nvcc contracts `a += b*c` / `a - b*c` into made
// explicit (std::fma); the file is compiled with -ffp-contract=off so the host
// compiler adds no contraction of its own.  The reference kernels themselves
// are compiled from source and run on the GPU by oracle/ref_launch.cpp, which
// is what pins this restatement (tests/test_ref_pin.py).
//
// Only tests, the smoke check and bench.py's CPU-baseline leg may call this
// library; the product path (libbilu) never links or loads it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace {

// ---------------------------------------------------------------------------
// reductions in the reference's order
// ---------------------------------------------------------------------------

// inner_product(n, v1, v2, result) (Bicgstab_common.hpp:97-128): warp 0 only,
// lane l accumulates idx = l, l+32, ... with `temp += v1*v2` (fma), then a
// __shfl_down_sync tree with offsets 16, 8, 4, 2, 1; lane 0 holds the result.
inline double dot_warp0(int n, const double* a, const double* b) {
  double p[32];
  for (int l = 0; l < 32; ++l) {
    double t = 0.0;
    for (int i = l; i < n; i += 32) t = std::fma(a[i], b[i], t);
    p[l] = t;
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int l = 0; l < off; ++l) p[l] = p[l] + p[l + off];
  return p[0];
}

// inner_product(n, v1, v2) (Bicgstab_common.hpp:82-95): serial loop, every
// thread computes the same value; used by the ISAI solver kernels.
inline double dot_serial(int n, const double* a, const double* b) {
  double t = 0.0;
  for (int i = 0; i < n; ++i) t = std::fma(a[i], b[i], t);
  return t;
}

// One row of SpMV / ComputeResidualVec (Bicgstab_common.hpp:5-40, 254-290):
// warp per row, lane l accumulates entries beg+l, beg+l+32, ... with
// `temp += val*vec[col]` (fma), then the 16..1 shfl_down tree.
inline double row_tree(const double* vals, const int* ci, int beg, int end, const double* x) {
  double p[32];
  for (int l = 0; l < 32; ++l) {
    double t = 0.0;
    for (int k = beg + l; k < end; k += 32) t = std::fma(vals[k], x[ci[k]], t);
    p[l] = t;
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int l = 0; l < off; ++l) p[l] = p[l] + p[l + off];
  return p[0];
}

inline void spmv_tree(int n, const int* rp, const int* ci, const double* vals, const double* x, double* y) {
  for (int i = 0; i < n; ++i) y[i] = row_tree(vals, ci, rp[i], rp[i + 1], x);
}

// FP32-stored ISAI applied in FP32 (the library's BILU_FP32 mode; no
// reference counterpart): input rounded to float, each row a sequential fmaf
// sum in CSR order, result widened to double.
inline void spmv_f32(int n, const int* rp, const int* ci, const float* vals, const float* x, float* y) {
  for (int i = 0; i < n; ++i) {
    float acc = 0.0f;
    for (int k = rp[i]; k < rp[i + 1]; ++k) acc = std::fmaf(vals[k], x[ci[k]], acc);
    y[i] = acc;
  }
}

// ---------------------------------------------------------------------------
// triangular solves on in-place factors (L strictly lower with unit diagonal,
// U upper), PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:22-143 and the
// split L/U form PrecondBiCGSTAB_ilu_gpu.cu:22-150 (same arithmetic: the L
// diagonal there is an explicit 1.0 and x/1.0 == x).
// lower: sum over the row's entries left of the diagonal in ascending order
//        (fma), y_i = (v_i - sum)/1
// upper: sum over the entries right of the diagonal in DESCENDING order (fma),
//        z_i = (y_i - sum)/u_ii
// ---------------------------------------------------------------------------
inline void trsv_lu(int n, const int* rp, const int* ci, const int* diag, const double* lu, const double* v,
                    double* y, double* z) {
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int k = rp[i]; k < diag[i]; ++k) s = std::fma(lu[k], y[ci[k]], s);
    y[i] = v[i] - s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = 0.0;
    for (int k = rp[i + 1] - 1; k > diag[i]; --k) s = std::fma(lu[k], z[ci[k]], s);
    z[i] = (y[i] - s) / lu[diag[i]];
  }
}

// FP32-stored factors, applied in FP32 (the library's BILU_FP32 mode; no
// reference counterpart): the right-hand side is rounded to float, every
// product-sum is an fmaf in the same order as above, the diagonal division is
// a multiplication by the float reciprocal rounded from the double
// reciprocal, and the result is widened back to double.
inline void trsv_lu_f32(int n, const int* rp, const int* ci, const int* diag, const float* lu, const float* rinv,
                        const double* v, float* y, double* z_out) {
  for (int i = 0; i < n; ++i) {
    float s = 0.0f;
    for (int k = rp[i]; k < diag[i]; ++k) s = std::fmaf(lu[k], y[ci[k]], s);
    y[i] = (float)v[i] - s;
  }
  for (int i = n - 1; i >= 0; --i) {
    float s = 0.0f;
    for (int k = rp[i + 1] - 1; k > diag[i]; --k) s = std::fmaf(lu[k], y[ci[k]], s);
    y[i] = (y[i] - s) * rinv[i];
  }
  for (int i = 0; i < n; ++i) z_out[i] = (double)y[i];
}

}  // namespace

// ===========================================================================
// pattern utilities (factorization.cu)
// ===========================================================================

// Count_Missing_Diagonal_Elements (factorization.cu:399-421).
ORC_API int orc_count_missing_diag(int n, const int* rp, const int* ci) {
  int missing = 0;
  for (int i = 0; i < n; ++i) {
    bool has = false;
    for (int k = rp[i]; k < rp[i + 1]; ++k) has |= (ci[k] == i);
    missing += has ? 0 : 1;
  }
  return missing;
}

// Add_Missing_Diagonal_Elements (factorization.cu:425-467): the new pattern
// has (i,i) inserted in column order; src[k_new] = old index or -1 (value 0).
ORC_API void orc_add_missing_diag(int n, const int* rp, const int* ci, int* new_rp, int* new_ci, int* src) {
  int pos = 0;
  new_rp[0] = 0;
  for (int i = 0; i < n; ++i) {
    bool has = false;
    for (int k = rp[i]; k < rp[i + 1]; ++k) has |= (ci[k] == i);
    bool placed = has;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      if (!placed && ci[k] > i) {
        new_ci[pos] = i;
        src[pos] = -1;
        ++pos;
        placed = true;
      }
      new_ci[pos] = ci[k];
      src[pos] = k;
      ++pos;
    }
    if (!placed) {
      new_ci[pos] = i;
      src[pos] = -1;
      ++pos;
    }
    new_rp[i + 1] = pos;
  }
}

// Find_locations_of_diagonal_elements (factorization.cu:472-480).
ORC_API void orc_find_diag(int n, const int* rp, const int* ci, int* diag) {
  for (int i = 0; i < n; ++i) {
    diag[i] = -1;
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (ci[k] == i) diag[i] = k;
  }
}

// L/U split (factorization.cu:216-344): L row = strictly-lower entries then
// an explicit unit diagonal; U row = diagonal then the strictly-upper entries.
// Pattern pass: l_rp/l_ci/u_rp/u_ci; value pass (nsys pages) gathers from the
// in-place factors.
ORC_API void orc_split_pattern(int n, const int* rp, const int* ci, const int* diag, int* l_rp, int* l_ci, int* u_rp,
                               int* u_ci) {
  l_rp[0] = u_rp[0] = 0;
  for (int i = 0; i < n; ++i) {
    int lp = l_rp[i], up = u_rp[i];
    for (int k = rp[i]; k < diag[i]; ++k) l_ci[lp++] = ci[k];
    l_ci[lp++] = i;
    for (int k = diag[i]; k < rp[i + 1]; ++k) u_ci[up++] = ci[k];
    l_rp[i + 1] = lp;
    u_rp[i + 1] = up;
  }
}

ORC_API void orc_split_values(int n, int nnz, const int* rp, const int* diag, int nsys, const double* lu, int nnz_l,
                              double* l, int nnz_u, double* u) {
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    const double* a = lu + (size_t)s * nnz;
    double* L = l + (size_t)s * nnz_l;
    double* U = u + (size_t)s * nnz_u;
    int lp = 0, up = 0;
    for (int i = 0; i < n; ++i) {
      for (int k = rp[i]; k < diag[i]; ++k) L[lp++] = a[k];
      L[lp++] = 1.0;
      for (int k = diag[i]; k < rp[i + 1]; ++k) U[up++] = a[k];
    }
  }
}

// ===========================================================================
// ILU(0)
// ===========================================================================
//
// approach 1 (ILU_0_gpu.cu:26-171; the merged solver's inlined copy
// PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:145-246): right-looking, for
// pivot row k = 0..n-1 and every row i > k: l_ik = a_ik / u_kk, then
// a_ij = fma(-l_ik, u_kj, a_ij) for j > k (rows without a_ik and columns
// without u_kj receive an exact zero update).  Written here in the same
// per-entry order: every entry receives its updates in ascending k.
// approach 4 (ILU_0_gpu.cu:947-1229): the same updates per entry in
// ascending k (`values[loc] -= values[loc_1] * row_ele`), same bits.
// approach 3 (ILU_0_gpu.cu:693-935): sum = sum of l_ik*u_kj (fma) over k in
// ascending order starting from 0, then a_ij = (a_ij - sum)/d with d = u_jj
// below the diagonal and d = 1 elsewhere.
// approach 2 (ILU_0_gpu.cu:376-685): as approach 3 but the dependency list
// is a linked list built by head insertion, so k runs DESCENDING.
ORC_API void orc_ilu0(int n, int nnz, const int* rp, const int* ci, int nsys, const double* vals, double* lu,
                      int approach) {
  std::vector<int> diag(n);
  orc_find_diag(n, rp, ci, diag.data());
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    double* a = lu + (size_t)s * nnz;
    std::memcpy(a, vals + (size_t)s * nnz, sizeof(double) * nnz);
    std::vector<int> colpos(n, -1);
    std::vector<int> ks;
    std::vector<std::pair<int, int>> pairs;  // (pos_ik, pos_kj)
    for (int i = 0; i < n; ++i) {
      for (int k = rp[i]; k < rp[i + 1]; ++k) colpos[ci[k]] = k;
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const int j = ci[e];
        const int kmax = std::min(i, j);  // k < min(i, j)
        pairs.clear();
        for (int lk = rp[i]; lk < rp[i + 1] && ci[lk] < kmax; ++lk) {
          const int k = ci[lk];
          for (int uk = diag[k] + 1; uk < rp[k + 1]; ++uk)
            if (ci[uk] == j) pairs.emplace_back(lk, uk);
        }
        if (approach == 1 || approach == 4) {
          double v = a[e];
          for (auto& p : pairs) v = std::fma(-a[p.first], a[p.second], v);
          if (j < i) v = v / a[diag[j]];
          a[e] = v;
        } else {
          double sum = 0.0;
          if (approach == 3) {
            for (auto& p : pairs) sum = std::fma(a[p.first], a[p.second], sum);
          } else {
            for (auto it = pairs.rbegin(); it != pairs.rend(); ++it) sum = std::fma(a[it->first], a[it->second], sum);
          }
          double v = a[e] - sum;
          if (j < i) v = v / a[diag[j]];
          a[e] = v;
        }
      }
      for (int k = rp[i]; k < rp[i + 1]; ++k) colpos[ci[k]] = -1;
    }
  }
}

// ParILU(0) sweep (parILU_0_gpu.cu:18-57) with the dependency list of
// create_dependency_graph_parilu (parILU_0_gpu.cu:118-220): for entry (i,j),
// sum = sum over k < min(i,j) ascending of l_ik*u_kj (fma from 0), then
// (a_ij - sum)/u_jj below the diagonal and (a_ij - sum)/1 on and above it.
// The reference updates in place without a barrier inside a sweep (its
// result depends on thread timing when nnz > blockDim); this restatement
// uses the documented deterministic schedule of the library: Jacobi sweeps
// (every entry of sweep t+1 reads the values of sweep t).  Initial guess
// (Fill_L_and_U, factorization.cu:288-344): L = strict-lower(A) + I,
// U = upper(A), i.e. the in-place factors start equal to A; `init` overrides.
// fast = 1: the library's BILU_REDUCE_FAST sweep (k_parilu0<true>): lower
// entries are multiplied by the reciprocals 1 / u_jj of the current diagonal,
// formed once per sweep, instead of divided.
ORC_API void orc_parilu0_ex(int n, int nnz, const int* rp, const int* ci, int nsys, const double* vals,
                            const double* init, int sweeps, double* lu, int fast) {
  std::vector<int> diag(n);
  orc_find_diag(n, rp, ci, diag.data());
  // dependency lists (pattern only)
  std::vector<int> dptr(nnz + 1, 0), dl, du;
  for (int i = 0; i < n; ++i)
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int j = ci[e];
      const int kmax = std::min(i, j);
      for (int lk = rp[i]; lk < rp[i + 1] && ci[lk] < kmax; ++lk) {
        const int k = ci[lk];
        for (int uk = diag[k] + 1; uk < rp[k + 1]; ++uk)
          if (ci[uk] == j) {
            dl.push_back(lk);
            du.push_back(uk);
          }
      }
      dptr[e + 1] = (int)dl.size();
    }
  std::vector<int> rowof(nnz);
  for (int i = 0; i < n; ++i)
    for (int e = rp[i]; e < rp[i + 1]; ++e) rowof[e] = i;
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    const double* A = vals + (size_t)s * nnz;
    double* cur = lu + (size_t)s * nnz;
    std::memcpy(cur, init ? init + (size_t)s * nnz : A, sizeof(double) * nnz);
    std::vector<double> nxt(nnz), rinv(n);
    for (int t = 0; t < sweeps; ++t) {
      if (fast)
        for (int r = 0; r < n; ++r) rinv[r] = 1.0 / cur[diag[r]];
      for (int e = 0; e < nnz; ++e) {
        double sum = 0.0;
        for (int q = dptr[e]; q < dptr[e + 1]; ++q) sum = std::fma(cur[dl[q]], cur[du[q]], sum);
        double v = A[e] - sum;
        const int i = rowof[e], j = ci[e];
        if (j < i) v = fast ? v * rinv[j] : v / cur[diag[j]];
        nxt[e] = v;
      }
      std::memcpy(cur, nxt.data(), sizeof(double) * nnz);
    }
  }
}

ORC_API void orc_parilu0(int n, int nnz, const int* rp, const int* ci, int nsys, const double* vals,
                         const double* init, int sweeps, double* lu) {
  orc_parilu0_ex(n, nnz, rp, ci, nsys, vals, init, sweeps, lu, 0);
}

// ||(A - L U)|_S||_F / ||A||_F on the factor pattern S (the ILU residual that
// judges a ParILU warm start; no reference counterpart).  Products summed in
// ascending k with fma, in double.
ORC_API void orc_ilu_residual(int n, int nnz, const int* rp, const int* ci, int nsys, const double* vals,
                              const double* lu, double* out) {
  std::vector<int> diag(n);
  orc_find_diag(n, rp, ci, diag.data());
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    const double* A = vals + (size_t)s * nnz;
    const double* F = lu + (size_t)s * nnz;
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; ++i)
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const int j = ci[e];
        // (LU)_ij = sum_{k <= min(i,j)} l_ik u_kj, l_ii = 1
        double acc = 0.0;
        for (int lk = rp[i]; lk < rp[i + 1] && ci[lk] <= std::min(i, j); ++lk) {
          const int k = ci[lk];
          const double l = (k == i) ? 1.0 : F[lk];
          if (k == j && k < i) {  // u_jj with j < i
            acc = std::fma(l, F[diag[j]], acc);
            continue;
          }
          for (int uk = diag[k]; uk < rp[k + 1]; ++uk)
            if (ci[uk] == j) acc = std::fma(l, F[uk], acc);
        }
        const double d = A[e] - acc;
        num = std::fma(d, d, num);
        den = std::fma(A[e], A[e], den);
      }
    out[s] = std::sqrt(num) / std::sqrt(den);
  }
}

// ===========================================================================
// ISAI (isai_gpu.cu)
// ===========================================================================

// Pattern of |T|^power (isai_gpu.cu:40-179).  The reference forms the powers
// densely from page 0's numeric values, so an entry is in the pattern when
// the computed value is nonzero; with vals0 == NULL the structural pattern is
// returned instead (identical unless an entry cancels to exactly 0).
// Returns nnz; ai_rp / ai_ci may be NULL for a size query.
ORC_API int orc_isai_pattern(int n, const int* rp, const int* ci, int power, const double* vals0, int* ai_rp,
                             int* ai_ci) {
  // dense column-major n x n, same summation order as the reference
  std::vector<double> cur((size_t)n * n, 0.0), nxt;
  for (int r = 0; r < n; ++r)
    for (int k = rp[r]; k < rp[r + 1]; ++k) cur[(size_t)ci[k] * n + r] = vals0 ? vals0[k] : 1.0;
  std::vector<double> base = cur;
  for (int p = 2; p <= power; ++p) {
    nxt.assign((size_t)n * n, 0.0);
    for (int col = 0; col < n; ++col)
      for (int r = 0; r < n; ++r) {
        double sum = 0.0;
        for (int k = rp[r]; k < rp[r + 1]; ++k) {
          const double v = vals0 ? vals0[k] : 1.0;
          // host code, x86 without FMA contraction: separate multiply and add
          sum = sum + v * cur[(size_t)col * n + ci[k]];
        }
        nxt[(size_t)col * n + r] = sum;
      }
    cur.swap(nxt);
  }
  int nz = 0;
  if (ai_rp) ai_rp[0] = 0;
  for (int r = 0; r < n; ++r) {
    for (int col = 0; col < n; ++col)
      if (cur[(size_t)col * n + r] != 0.0) {
        if (ai_ci) ai_ci[nz] = col;
        ++nz;
      }
    if (ai_rp) ai_rp[r + 1] = nz;
  }
  return nz;
}

// ISAI values (isai_gpu.cu:209-287 extraction, 325-389 and 559-626 solves).
// For row i of M with pattern J (sorted, |J| <= 32): the reference loads
// lane t with row t of T(J,J)^T and solves
//   lower T (tri = 0): upper-triangular back substitution, rhs e_{|J|-1}
//     (solve_upper_tri_dense): for col = |J|-1 .. 0: lane col divides by its
//     diagonal, then lanes t < col do sol_t = fma(-sol_col, T(J_col,J_t), sol_t)
//   upper T (tri = 1): forward substitution, rhs e_0 (solve_lower_tri_dense):
//     for col = 0 .. |J|-1, lanes t > col update.
// Missing entries of T(J,J) are zeros (they give exact zero updates).
//   general T (tri = 2): Gauss-Jordan with partial pivoting, rhs e_pos(i).
// T is given in the reference's separate CSR form (t_rp/t_ci/t_vals; for L
// the explicit unit diagonal is part of the pattern).
// fast = 1: the library's BILU_REDUCE_FAST ISAI of an upper triangle (k_isai
// with FAST): each division by a diagonal entry is a multiplication by its
// correctly rounded reciprocal 1.0 / u.
ORC_API int orc_isai_values_ex(int n, const int* t_rp, const int* t_ci, int t_nnz, int nsys, const double* t_vals,
                               int tri, const int* ai_rp, const int* ai_ci, int ai_nnz, double* ai_vals, int fast) {
  for (int i = 0; i < n; ++i)
    if (ai_rp[i + 1] - ai_rp[i] > 32) return -1;
  if (fast == 2 && tri != 2) {
    // the library's FAST ISAI stored in FP32 (k_isai_f32): T rounded to float,
    // float fmas in the same order, aiU scaled by 1.0f / u (float); L's unit
    // diagonal is exact.  Values returned widened to double.
#pragma omp parallel for schedule(static)
    for (int s = 0; s < nsys; ++s) {
      const double* T = t_vals + (size_t)s * t_nnz;
      double* M = ai_vals + (size_t)s * ai_nnz;
      float loc[32][32];
      for (int i = 0; i < n; ++i) {
        const int beg = ai_rp[i], sz = ai_rp[i + 1] - ai_rp[i];
        const int* J = ai_ci + beg;
        for (int t = 0; t < sz; ++t)
          for (int c = 0; c < sz; ++c) {
            float v = 0.0f;
            for (int k = t_rp[J[c]]; k < t_rp[J[c] + 1]; ++k)
              if (t_ci[k] == J[t]) v = (float)T[k];
            loc[t][c] = v;
          }
        float sol[32];
        if (tri == 0) {
          for (int t = 0; t < sz; ++t) sol[t] = (t == sz - 1) ? 1.0f : 0.0f;
          for (int col = sz - 1; col >= 0; --col) {
            const float bot = sol[col];  // unit diagonal
            for (int t = 0; t < col; ++t) sol[t] = std::fma(-bot, loc[t][col], sol[t]);
          }
        } else {
          for (int t = 0; t < sz; ++t) sol[t] = (t == 0) ? 1.0f : 0.0f;
          for (int col = 0; col < sz; ++col) {
            sol[col] = sol[col] * (1.0f / loc[col][col]);
            const float top = sol[col];
            for (int t = col + 1; t < sz; ++t) sol[t] = std::fma(-top, loc[t][col], sol[t]);
          }
        }
        for (int t = 0; t < sz; ++t) M[beg + t] = (double)sol[t];
      }
    }
    return 0;
  }
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    const double* T = t_vals + (size_t)s * t_nnz;
    double* M = ai_vals + (size_t)s * ai_nnz;
    double loc[32][32];  // loc[t][c] = T(J_c, J_t)
    for (int i = 0; i < n; ++i) {
      const int beg = ai_rp[i], sz = ai_rp[i + 1] - ai_rp[i];
      const int* J = ai_ci + beg;
      for (int t = 0; t < sz; ++t)
        for (int c = 0; c < sz; ++c) {
          double v = 0.0;
          for (int k = t_rp[J[c]]; k < t_rp[J[c] + 1]; ++k)
            if (t_ci[k] == J[t]) v = T[k];
          loc[t][c] = v;
        }
      double sol[32];
      if (tri == 0) {
        for (int t = 0; t < sz; ++t) sol[t] = (t == sz - 1) ? 1.0 : 0.0;
        for (int col = sz - 1; col >= 0; --col) {
          sol[col] = sol[col] / loc[col][col];
          const double bot = sol[col];
          for (int t = 0; t < col; ++t) sol[t] = std::fma(-bot, loc[t][col], sol[t]);
        }
      } else if (tri == 1) {
        for (int t = 0; t < sz; ++t) sol[t] = (t == 0) ? 1.0 : 0.0;
        for (int col = 0; col < sz; ++col) {
          sol[col] = fast ? sol[col] * (1.0 / loc[col][col]) : sol[col] / loc[col][col];
          const double top = sol[col];
          for (int t = col + 1; t < sz; ++t) sol[t] = std::fma(-top, loc[t][col], sol[t]);
        }
      } else {
        // general (solve_general_dense, isai_gpu.cu:392-554): Gauss-Jordan on the
        // rows of T(J,J)^T (one lane each in the reference) with partial pivoting.
        // choose_pivot_row_1's shfl_down tree with strict > keeps the lower lane on
        // ties, and lanes outside [dp, sz) carry row dp's value: the pivot is the
        // first row with the largest |a_r[dp]|.
        int pos = 0;
        for (int t = 0; t < sz; ++t)
          if (J[t] == i) pos = t;
        for (int t = 0; t < sz; ++t) sol[t] = (t == pos) ? 1.0 : 0.0;
        for (int dp = 0; dp < sz; ++dp) {
          int piv = dp;
          double best = std::fabs(loc[dp][dp]);
          for (int r = dp + 1; r < sz; ++r)
            if (std::fabs(loc[r][dp]) > best) {
              best = std::fabs(loc[r][dp]);
              piv = r;
            }
          if (piv != dp) {
            for (int c = 0; c < sz; ++c) std::swap(loc[dp][c], loc[piv][c]);
            std::swap(sol[dp], sol[piv]);
          }
          const double d = loc[dp][dp];
          for (int r = 0; r < sz; ++r) {
            if (r == dp) continue;
            const double mult = loc[r][dp] / d;
            for (int c = 0; c < sz; ++c) loc[r][c] = std::fma(-mult, loc[dp][c], loc[r][c]);
            sol[r] = std::fma(-mult, sol[dp], sol[r]);
          }
        }
        for (int t = 0; t < sz; ++t) sol[t] = sol[t] / loc[t][t];
      }
      for (int t = 0; t < sz; ++t) M[beg + t] = sol[t];
    }
  }
  return 0;
}

// ===========================================================================
// BiCGSTAB (KernelBatchedPreconditionedBiCGSTAB_ILU in
// PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:249-538 and
// PrecondBiCGSTAB_ilu_gpu.cu:155-438; KernelBatchedPreconditionedBiCGSTAB_ILU_ISAI
// in PrecondBiCGSTAB_ilu_isai_gpu.cu:49-262)
// ===========================================================================
//
// prec: 0 = in-place LU factors (lu on the factor pattern f_rp/f_ci = A's
//           pattern with inserted diagonals; NULL = A's), triangular solves;
//       1 = ISAI: z = aiU * (aiL * v), both with the SpMV tree order;
//       2 = identity;
//       3 = in-place LU stored as float (lu_f32), applied in FP32 (library mode);
//       4 = ISAI stored as float (ail_f/aiu_f), applied in FP32;
//       5 = general ISAI of A: z = aiA * v (PrecondBiCGSTAB_general_isai_gpu.cu:23-30);
//       6 = the same stored and applied in FP32.
// dot: 0 = warp-0 tree inner products (ILU solver kernels),
//      1 = serial inner products (ISAI solver kernel).
// tol_mode: 0 = absolute (||r|| < tol, the reference's ATOL), 1 = relative to ||b||.
// Outputs per system: x, iteration count (0.5 steps), conv flag (1/-1),
// recursive residual norm and a detailed status (BILU_SYS_* values).
ORC_API int orc_isai_values(int n, const int* t_rp, const int* t_ci, int t_nnz, int nsys, const double* t_vals,
                            int tri, const int* ai_rp, const int* ai_ci, int ai_nnz, double* ai_vals) {
  return orc_isai_values_ex(n, t_rp, t_ci, t_nnz, nsys, t_vals, tri, ai_rp, ai_ci, ai_nnz, ai_vals, 0);
}

ORC_API void orc_bicgstab(int n, int nnz, const int* rp, const int* ci, int nsys, const double* A, const double* b,
                          int f_nnz, const int* f_rp, const int* f_ci, int prec, const double* lu,
                          const float* lu_f32, int ail_nnz, const int* ail_rp,
                          const int* ail_ci, const double* ail, const float* ail_f, int aiu_nnz, const int* aiu_rp,
                          const int* aiu_ci, const double* aiu, const float* aiu_f, int dot, int tol_mode,
                          double tol, int max_iter, double* x_out, float* iters_out, int* conv_out,
                          double* res_out, int* status_out) {
  // factor pattern (A's pattern with inserted diagonals); defaults to A's
  if (!f_rp) {
    f_rp = rp;
    f_ci = ci;
    f_nnz = nnz;
  }
  std::vector<int> diag(n);
  orc_find_diag(n, f_rp, f_ci, diag.data());
#pragma omp parallel for schedule(dynamic, 4)
  for (int s = 0; s < nsys; ++s) {
    const double* As = A + (size_t)s * nnz;
    const double* bs = b + (size_t)s * n;
    const double* LU = lu ? lu + (size_t)s * f_nnz : nullptr;
    const float* LUf = lu_f32 ? lu_f32 + (size_t)s * f_nnz : nullptr;
    const double* AIL = ail ? ail + (size_t)s * ail_nnz : nullptr;
    const double* AIU = aiu ? aiu + (size_t)s * aiu_nnz : nullptr;
    const float* AILf = ail_f ? ail_f + (size_t)s * ail_nnz : nullptr;
    const float* AIUf = aiu_f ? aiu_f + (size_t)s * aiu_nnz : nullptr;
    std::vector<double> x(n, 0.0), r(n), rh(n), p(n, 0.0), v(n, 0.0), sv(n), t(n), ph(n), sh(n), tmp(n);
    std::vector<float> yf(n), rinvf(n), fin(n), fmid(n);
    if (prec == 3)
      for (int i = 0; i < n; ++i) rinvf[i] = (float)(1.0 / (double)LUf[diag[i]]);
    auto dotf = [&](const double* a1, const double* a2) {
      return dot == 0 ? dot_warp0(n, a1, a2) : dot_serial(n, a1, a2);
    };
    auto apply = [&](const double* in, double* out) {
      if (prec == 0) {
        trsv_lu(n, f_rp, f_ci, diag.data(), LU, in, tmp.data(), out);
      } else if (prec == 1) {
        spmv_tree(n, ail_rp, ail_ci, AIL, in, tmp.data());
        spmv_tree(n, aiu_rp, aiu_ci, AIU, tmp.data(), out);
      } else if (prec == 3) {
        trsv_lu_f32(n, f_rp, f_ci, diag.data(), LUf, rinvf.data(), in, yf.data(), out);
      } else if (prec == 5) {
        spmv_tree(n, ail_rp, ail_ci, AIL, in, out);
      } else if (prec == 6) {
        for (int i = 0; i < n; ++i) fin[i] = (float)in[i];
        spmv_f32(n, ail_rp, ail_ci, AILf, fin.data(), fmid.data());
        for (int i = 0; i < n; ++i) out[i] = (double)fmid[i];
      } else if (prec == 4) {
        for (int i = 0; i < n; ++i) fin[i] = (float)in[i];
        spmv_f32(n, ail_rp, ail_ci, AILf, fin.data(), fmid.data());
        spmv_f32(n, aiu_rp, aiu_ci, AIUf, fmid.data(), fin.data());
        for (int i = 0; i < n; ++i) out[i] = (double)fin[i];
      } else {
        for (int i = 0; i < n; ++i) out[i] = in[i];
      }
    };
    // initialization (Bicgstab_common.hpp:151-192): x = 0, r = b - A*0 = b, r_hat = r
    for (int i = 0; i < n; ++i) r[i] = bs[i];
    rh = r;
    const double res_initial = std::sqrt(dotf(r.data(), r.data()));
    const double b_norm = std::sqrt(dotf(bs, bs));
    const double thr = (tol_mode == 0) ? tol : tol * b_norm;
    double rho_old = 1, rho_new = 1, omega_old = 1, omega_new = 1, alpha = 1, beta = 1;
    double res = res_initial;
    float iter = 0;
    int conv = -1, status = -1;
    if (b_norm == 0) {
      std::fill(x.begin(), x.end(), 0.0);
      iter = 0;
      conv = 1;
      res = 0;
      status = 2;
    } else if (res_initial < thr) {
      iter = 0;
      conv = 1;
      status = 3;
    } else {
      while (iter < (float)max_iter) {
        rho_new = dotf(r.data(), rh.data());
        if (rho_new == 0) {
          status = -2;
          break;
        }
        beta = (rho_new / rho_old) * (alpha / omega_old);
        for (int i = 0; i < n; ++i) p[i] = std::fma(beta, std::fma(-omega_old, v[i], p[i]), r[i]);
        apply(p.data(), ph.data());
        spmv_tree(n, rp, ci, As, ph.data(), v.data());
        const double rv = dotf(rh.data(), v.data());
        alpha = rho_new / rv;
        for (int i = 0; i < n; ++i) sv[i] = std::fma(-alpha, v[i], r[i]);
        res = std::sqrt(dotf(sv.data(), sv.data()));
        iter = iter + 0.5f;
        if (res < thr) {
          for (int i = 0; i < n; ++i) x[i] = std::fma(alpha, ph[i], x[i]);
          conv = 1;
          status = 1;
          break;
        }
        apply(sv.data(), sh.data());
        spmv_tree(n, rp, ci, As, sh.data(), t.data());
        const double ts = dotf(t.data(), sv.data());
        const double tt = dotf(t.data(), t.data());
        omega_new = ts / tt;
        for (int i = 0; i < n; ++i) x[i] = std::fma(omega_new, sh[i], std::fma(alpha, ph[i], x[i]));
        iter = iter + 0.5f;
        for (int i = 0; i < n; ++i) r[i] = std::fma(-omega_new, t[i], sv[i]);
        res = std::sqrt(dotf(r.data(), r.data()));
        rho_old = rho_new;
        omega_old = omega_new;
        if (res < thr) {
          conv = 1;
          status = 1;
          break;
        }
      }
      if (status == -1 && !(std::isfinite(res))) status = -3;
    }
    std::memcpy(x_out + (size_t)s * n, x.data(), sizeof(double) * n);
    if (iters_out) iters_out[s] = iter;
    if (conv_out) conv_out[s] = conv;
    if (res_out) res_out[s] = res;
    if (status_out) status_out[s] = status;
  }
}

// KernelFillTrueResNorms (Bicgstab_common.hpp:294-342): r = b - A x with the
// SpMV tree order, norm = sqrt of the SERIAL inner product.
// BILU_REDUCE_FAST BiCGSTAB of the register-resident kernel (k_solve_rr.cu)
// with `nt` threads per system, thread t owning rows t + k*nt: the same
// recurrences, exits and iteration counting as orc_bicgstab, in this order --
//   thread partial   d_t = fma over thread t's rows in k order, from 0.0
//   no ILU factors   lane l: s_l = d_l + d_(l+32) + d_(l+64) + ... in order, then
//                    xor butterfly s_l = s_l + s_(l^off), off = 16..1; lane 0
//   ILU factors      xor butterfly per warp (lane 0: w_j), then w_0 + w_1 + ...
//   rows             A*x and the ISAI rows: fma over the row, from 0.0; ISAI in
//                    float when fp32 (input rounded, output widened)
//   LU solve         in-place factors: input rounded to FT; lower rows ascending,
//                    a = y_i, a = fma(-l_ik, y_k, a) over k ascending, y_i = a;
//                    upper rows descending, a = y_i, a = fma(-u_ik, z_k, a) over k
//                    descending, z_i = a * rinv_i, rinv_i = 1.0 / u_ii (FP64,
//                    rounded to float for FP32 factors); output widened
// pv: 0 none, 1 z = aiU (aiL v), 2 z = aiA v, 3 z = U^-1 L^-1 v (in-place LU
// factors on the factor pattern given as the `l` triangle).  No reference
// counterpart.
namespace {

// FAST LU solve (T = double, or float for FP32 factors with the input already
// rounded): the level-scheduled kernel computes each row from rows finished in
// earlier levels, so the row-sequential order below gives the same values.
template <typename T>
inline void trsv_lu_fast(int n, const int* rp, const int* ci, const int* diag, const T* lu, const T* rinv, T* y) {
  for (int i = 0; i < n; ++i) {
    T a = y[i];
    for (int k = rp[i]; k < diag[i]; ++k) a = std::fma(-lu[k], y[ci[k]], a);
    y[i] = a;
  }
  for (int i = n - 1; i >= 0; --i) {
    T a = y[i];
    for (int k = rp[i + 1] - 1; k > diag[i]; --k) a = std::fma(-lu[k], y[ci[k]], a);
    y[i] = a * rinv[i];
  }
}

double fast_block_sum(const std::vector<double>& part, int nt, bool lanes_first) {
  double v[32], nv[32];
  auto butterfly = [&]() {
    for (int off = 16; off >= 1; off >>= 1) {
      for (int l = 0; l < 32; ++l) nv[l] = v[l] + v[l ^ off];
      for (int l = 0; l < 32; ++l) v[l] = nv[l];
    }
  };
  if (lanes_first) {
    for (int l = 0; l < 32; ++l) {
      v[l] = part[l];
      for (int w = 1; w < nt / 32; ++w) v[l] = v[l] + part[32 * w + l];
    }
    butterfly();
    return v[0];
  }
  double s = 0.0;
  for (int w = 0; w < nt / 32; ++w) {
    for (int l = 0; l < 32; ++l) v[l] = part[32 * w + l];
    butterfly();
    s = w == 0 ? v[0] : s + v[0];
  }
  return s;
}

template <typename T>
T fast_row(const int* rp, const int* ci, const T* val, int i, const T* x) {
  T acc = T(0);
  for (int k = rp[i]; k < rp[i + 1]; ++k) acc = std::fma(val[k], x[ci[k]], acc);
  return acc;
}

}  // namespace

ORC_API int orc_bicgstab_fast(int n, int nnz, const int* rp, const int* ci, int nsys, const double* A,
                              const double* b, int pv, int fp32, const int* l_rp, const int* l_ci, int l_nnz,
                              const double* l_vals, const float* l_vals32, const int* u_rp, const int* u_ci, int u_nnz,
                              const double* u_vals, const float* u_vals32, int nt, int tol_mode, double tol,
                              int max_iter, double* x_out, float* iters, int* conv, double* res_out, int* status_out,
                              double* true_res) {
  if (nt <= 0 || nt % 32) return -1;
  int R = 0;
  for (int c : {1, 2, 4, 8})
    if (!R && (long long)c * nt >= n) R = c;
  if (!R) return -1;
  // bilu.h BILU_SYS_* values
  constexpr int kConverged = 1, kMaxIter = -1, kBreakdown = -2, kNonfinite = -3, kZeroRhs = 2, kInitialOk = 3;
  std::vector<int> ldiag(pv == 3 ? n : 0);
  if (pv == 3) orc_find_diag(n, l_rp, l_ci, ldiag.data());
#pragma omp parallel for schedule(dynamic, 1)
  for (int s = 0; s < nsys; ++s) {
    const double* As = A + (size_t)s * nnz;
    const double* bs = b + (size_t)s * n;
    const double* Ld = l_vals ? l_vals + (size_t)s * l_nnz : nullptr;
    const float* Lf = l_vals32 ? l_vals32 + (size_t)s * l_nnz : nullptr;
    const double* Ud = u_vals ? u_vals + (size_t)s * u_nnz : nullptr;
    const float* Uf = u_vals32 ? u_vals32 + (size_t)s * u_nnz : nullptr;
    std::vector<double> x(n, 0.0), r(bs, bs + n), p(n, 0.0), v(n, 0.0), t(n, 0.0), sph(n, 0.0), part(nt);
    std::vector<double> ind(n), midd(n), rinvd(pv == 3 ? n : 0);
    std::vector<float> inf(n), midf(n), rinvf(pv == 3 ? n : 0);
    if (pv == 3)
      for (int i = 0; i < n; ++i) {
        if (fp32)
          rinvf[i] = (float)(1.0 / (double)Lf[ldiag[i]]);
        else
          rinvd[i] = 1.0 / Ld[ldiag[i]];
      }
    // per-thread partial sums of f(i) over thread t's rows
    auto reduce = [&](auto f) {
      for (int th = 0; th < nt; ++th) {
        double d = 0.0;
        for (int k = 0; k < R; ++k) {
          const int i = th + k * nt;
          if (i < n) d = f(i, d);
        }
        part[th] = d;
      }
      return fast_block_sum(part, nt, pv != 3);
    };
    // z = M in into sph
    auto apply = [&](const std::vector<double>& in) {
      if (pv == 0) {
        sph = in;
      } else if (pv == 3) {
        if (fp32) {
          for (int i = 0; i < n; ++i) inf[i] = (float)in[i];
          trsv_lu_fast<float>(n, l_rp, l_ci, ldiag.data(), Lf, rinvf.data(), inf.data());
          for (int i = 0; i < n; ++i) sph[i] = (double)inf[i];
        } else {
          sph = in;
          trsv_lu_fast<double>(n, l_rp, l_ci, ldiag.data(), Ld, rinvd.data(), sph.data());
        }
      } else if (fp32) {
        for (int i = 0; i < n; ++i) inf[i] = (float)in[i];
        if (pv == 1) {
          for (int i = 0; i < n; ++i) midf[i] = fast_row<float>(l_rp, l_ci, Lf, i, inf.data());
          for (int i = 0; i < n; ++i) sph[i] = (double)fast_row<float>(u_rp, u_ci, Uf, i, midf.data());
        } else {
          for (int i = 0; i < n; ++i) sph[i] = (double)fast_row<float>(l_rp, l_ci, Lf, i, inf.data());
        }
      } else {
        if (pv == 1) {
          for (int i = 0; i < n; ++i) midd[i] = fast_row<double>(l_rp, l_ci, Ld, i, in.data());
          for (int i = 0; i < n; ++i) sph[i] = fast_row<double>(u_rp, u_ci, Ud, i, midd.data());
        } else {
          for (int i = 0; i < n; ++i) sph[i] = fast_row<double>(l_rp, l_ci, Ld, i, in.data());
        }
      }
    };
    const double q0 = reduce([&](int i, double d) { return std::fma(bs[i], bs[i], d); });
    const double bnorm = std::sqrt(q0);
    const double thr = tol_mode == 0 ? tol : tol * bnorm;
    double rho = q0, rho_old = 1.0, alpha = 1.0, omega_old = 1.0, res = bnorm;
    float iter = 0.0f;
    int status = kMaxIter;
    bool stop = false;
    if (bnorm == 0.0) {
      res = 0.0;
      status = kZeroRhs;
      stop = true;
    } else if (bnorm < thr) {
      status = kInitialOk;
      stop = true;
    }
    const float fmax = (float)max_iter;
    while (!stop && iter < fmax) {
      if (rho == 0.0) {
        status = kBreakdown;
        break;
      }
      const double beta = (rho / rho_old) * (alpha / omega_old);
      for (int i = 0; i < n; ++i) p[i] = std::fma(beta, std::fma(-omega_old, v[i], p[i]), r[i]);
      apply(p);
      for (int i = 0; i < n; ++i) v[i] = fast_row<double>(rp, ci, As, i, sph.data());
      const double rv = reduce([&](int i, double d) { return std::fma(bs[i], v[i], d); });
      alpha = rho / rv;
      for (int i = 0; i < n; ++i) {
        x[i] = std::fma(alpha, sph[i], x[i]);
        r[i] = std::fma(-alpha, v[i], r[i]);
      }
      const double ss = reduce([&](int i, double d) { return std::fma(r[i], r[i], d); });
      res = std::sqrt(ss);
      iter = iter + 0.5f;
      if (res < thr) {
        status = kConverged;
        break;
      }
      apply(r);
      for (int i = 0; i < n; ++i) t[i] = fast_row<double>(rp, ci, As, i, sph.data());
      const double ts = reduce([&](int i, double d) { return std::fma(t[i], r[i], d); });
      const double tt = reduce([&](int i, double d) { return std::fma(t[i], t[i], d); });
      const double omega = ts / tt;
      for (int i = 0; i < n; ++i) {
        x[i] = std::fma(omega, sph[i], x[i]);
        r[i] = std::fma(-omega, t[i], r[i]);
      }
      const double rr = reduce([&](int i, double d) { return std::fma(r[i], r[i], d); });
      const double rhr = reduce([&](int i, double d) { return std::fma(bs[i], r[i], d); });
      res = std::sqrt(rr);
      iter = iter + 0.5f;
      rho_old = rho;
      omega_old = omega;
      rho = rhr;
      if (res < thr) {
        status = kConverged;
        break;
      }
    }
    if (status == kMaxIter && !std::isfinite(res)) status = kNonfinite;
    std::memcpy(x_out + (size_t)s * n, x.data(), sizeof(double) * n);
    iters[s] = iter;
    conv[s] = (status == kConverged || status == kZeroRhs || status == kInitialOk) ? 1 : -1;
    res_out[s] = res;
    if (status_out) status_out[s] = status;
    if (true_res) {
      const double tr = reduce([&](int i, double d) {
        const double ri = bs[i] - fast_row<double>(rp, ci, As, i, x.data());
        return std::fma(ri, ri, d);
      });
      true_res[s] = std::sqrt(tr);
    }
  }
  return 0;
}

ORC_API void orc_true_residual(int n, int nnz, const int* rp, const int* ci, int nsys, const double* A,
                               const double* b, const double* x, double* out) {
#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    const double* As = A + (size_t)s * nnz;
    const double* bs = b + (size_t)s * n;
    const double* xs = x + (size_t)s * n;
    std::vector<double> r(n);
    for (int i = 0; i < n; ++i) r[i] = bs[i] - row_tree(As, ci, rp[i], rp[i + 1], xs);
    out[s] = std::sqrt(dot_serial(n, r.data(), r.data()));
  }
}

// ===========================================================================
// FP64 dense LU with partial pivoting (forward-error oracle; no reference
// counterpart).  Solves each system densely; returns x.  Pivot = first row
// of largest |a_ik|; multipliers f = a_ik / a_kk; updates fma(-f, a_kj, a_ij)
// (rhs alike); column-oriented back substitution.  The library's GPU dense
// solve (bilu_forward_error) performs the same operations.
// ===========================================================================
ORC_API void orc_dense_solve(int n, int nnz, const int* rp, const int* ci, int nsys, const int* sys_ids,
                             const double* A, const double* b, double* x_out) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < nsys; ++q) {
    const int s = sys_ids ? sys_ids[q] : q;
    std::vector<double> M((size_t)n * n, 0.0), y(b + (size_t)s * n, b + (size_t)s * n + n);
    const double* As = A + (size_t)s * nnz;
    for (int i = 0; i < n; ++i)
      for (int k = rp[i]; k < rp[i + 1]; ++k) M[(size_t)i * n + ci[k]] = As[k];
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
      int pr = k;
      double best = std::fabs(M[(size_t)k * n + k]);
      for (int i = k + 1; i < n; ++i) {
        const double v = std::fabs(M[(size_t)i * n + k]);
        if (v > best) {
          best = v;
          pr = i;
        }
      }
      if (pr != k) {
        for (int j = 0; j < n; ++j) std::swap(M[(size_t)k * n + j], M[(size_t)pr * n + j]);
        std::swap(y[k], y[pr]);
      }
      const double d = M[(size_t)k * n + k];
      for (int i = k + 1; i < n; ++i) {
        const double f = M[(size_t)i * n + k] / d;
        if (f == 0.0) continue;
        M[(size_t)i * n + k] = f;
        for (int j = k + 1; j < n; ++j) M[(size_t)i * n + j] = std::fma(-f, M[(size_t)k * n + j], M[(size_t)i * n + j]);
        y[i] = std::fma(-f, y[k], y[i]);
      }
    }
    // column-oriented back substitution: x_j = y_j / u_jj, then y_i -= u_ij x_j for i < j
    double* xs = x_out + (size_t)q * n;
    for (int j = n - 1; j >= 0; --j) {
      xs[j] = y[j] / M[(size_t)j * n + j];
      for (int i = 0; i < j; ++i) y[i] = std::fma(-M[(size_t)i * n + j], xs[j], y[i]);
    }
  }
}

ORC_API int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

ORC_API void orc_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

// ===========================================================================
// learned ParILU warm start (no reference counterpart): the library's
// features (computed the same way, so bit-identical) and an FP64 forward /
// backward of the 9-64-64-1 GELU network over BF16-rounded weights, for
// checking the GPU training kernels.
// ===========================================================================
namespace {

// round-to-nearest-even of an FP32 value to BF16 precision (IEEE rounding rule)
inline float bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  std::memcpy(&x, &u, 4);
  return x;
}

constexpr int MF = 9, MH = 64;
constexpr int MOW1 = 0, MOB1 = MH * MF, MOW2 = MOB1 + MH, MOB2 = MOW2 + MH * MH, MOW3 = MOB2 + MH, MOB3 = MOW3 + MH;
constexpr int MNP = MOB3 + 1;

// GELU, tanh form: 0.5 x (1 + tanh(k (x + c x^3))), k = sqrt(2/pi), c = 0.044715
constexpr double kGk = 0.7978845608028654, kGc = 0.044715;
inline double gelu_d(double x) { return 0.5 * x * (1.0 + std::tanh(kGk * (x + kGc * x * x * x))); }
inline double gelu_dd(double x) {
  const double t = std::tanh(kGk * (x + kGc * x * x * x));
  return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * kGk * (1.0 + 3.0 * kGc * x * x);
}

}  // namespace

ORC_API int orc_mlp_param_count(void) { return MNP; }

// features of entries idx[q] = s*nnz + e (factor pattern with every diagonal)
ORC_API void orc_mlp_features(int n, int nnz, const int* rp, const int* ci, int nsys, const double* vals, int nsample,
                              const int* idx, float* feat, double* base) {
  std::vector<int> diag(n), rowof(nnz), tpos(nnz, -1), lev(n, 0);
  orc_find_diag(n, rp, ci, diag.data());
  int nlev = 0;
  for (int i = 0; i < n; ++i) {
    int l = 0;
    for (int k = rp[i]; k < diag[i]; ++k) l = std::max(l, lev[ci[k]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      rowof[k] = i;
      const int j = ci[k];
      for (int t = rp[j]; t < rp[j + 1]; ++t)
        if (ci[t] == i) tpos[k] = t;
    }
  }
  for (int q = 0; q < nsample; ++q) {
    const long long g = idx[q];
    const int s = (int)(g / nnz), e = (int)(g % nnz);
    const double* As = vals + (size_t)s * nnz;
    auto stats = [&](int r, float& rn, float& cn, float& cr) {  // FP32, as k_rowstats
      float a = 0.0f, b = 0.0f, c = 0.0f;
      for (int k = rp[r]; k < rp[r + 1]; ++k) {
        const float ak = (float)As[k];
        a = std::fma(ak, ak, a);
        const int t = tpos[k];
        if (t >= 0) {
          const float at = (float)As[t];
          b = std::fma(at, at, b);
          if (k < diag[r]) c = std::fma(ak, at / (float)As[diag[ci[k]]], c);
        }
      }
      rn = std::sqrt(a);
      cn = std::sqrt(b);
      cr = c;
    };
    const int i = rowof[e], j = ci[e];
    float rni, cni, cri, rnj, cnj, crj;
    stats(i, rni, cni, cri);
    stats(j, rnj, cnj, crj);
    const float fij = (float)As[e], fii = (float)As[diag[i]], fjj = (float)As[diag[j]];
    const float inv = 1.0f / (fii != 0.0f ? std::fabs(fii) : 1.0f);
    float* f = feat + (size_t)q * MF;
    f[0] = fij * inv;
    f[1] = fii * inv;
    f[2] = fjj * inv;
    f[3] = rni * inv;
    f[4] = cnj * inv;
    f[5] = nlev > 1 ? (float)lev[i] / (float)(nlev - 1) : 0.0f;
    f[6] = j < i ? -1.0f : (j > i ? 1.0f : 0.0f);
    f[7] = cri * inv;
    f[8] = crj * inv;
    float bs = 1.0f;
    if (j < i) {
      const float den = fjj - crj;
      bs = den != 0.0f ? 1.0f / den : (fjj != 0.0f ? 1.0f / fjj : 1.0f);
    } else if (j == i) {
      bs = fii != 0.0f ? (fii - cri) / fii : 1.0f;
    }
    base[q] = (double)bs;
  }
}

// mean squared error over the samples and its gradient (FP64 arithmetic,
// weights rounded to BF16 as the GPU computes with them); returns the loss;
// out (optional) receives the network outputs
ORC_API double orc_mlp_loss_grad(const float* params, int nsample, const float* feat, const float* y, double* grad,
                                 double* out) {
  std::vector<double> w(MNP);
  for (int k = 0; k < MNP; ++k) w[k] = (double)bf16_round(params[k]);
  std::fill(grad, grad + MNP, 0.0);
  double loss = 0.0;
  for (int q = 0; q < nsample; ++q) {
    const float* x = feat + (size_t)q * MF;
    double p1[MH], h1[MH], p2[MH], h2[MH];
    for (int u = 0; u < MH; ++u) {
      double a = w[MOB1 + u];
      for (int k = 0; k < MF; ++k) a += w[MOW1 + u * MF + k] * (double)x[k];
      p1[u] = a;
      h1[u] = gelu_d(a);
    }
    double o = w[MOB3];
    for (int u = 0; u < MH; ++u) {
      double a = w[MOB2 + u];
      for (int v = 0; v < MH; ++v) a += w[MOW2 + u * MH + v] * h1[v];
      p2[u] = a;
      h2[u] = gelu_d(a);
      o += w[MOW3 + u] * h2[u];
    }
    if (out) out[q] = o;
    const double diff = o - (double)y[q];
    loss += diff * diff / nsample;
    const double dout = 2.0 * diff / nsample;
    grad[MOB3] += dout;
    double dp2[MH];
    for (int u = 0; u < MH; ++u) {
      grad[MOW3 + u] += dout * h2[u];
      dp2[u] = dout * w[MOW3 + u] * gelu_dd(p2[u]);
      grad[MOB2 + u] += dp2[u];
      for (int v = 0; v < MH; ++v) grad[MOW2 + u * MH + v] += dp2[u] * h1[v];
    }
    for (int v = 0; v < MH; ++v) {
      double dh = 0.0;
      for (int u = 0; u < MH; ++u) dh += w[MOW2 + u * MH + v] * dp2[u];
      const double dp1 = dh * gelu_dd(p1[v]);
      grad[MOB1 + v] += dp1;
      for (int k = 0; k < MF; ++k) grad[MOW1 + v * MF + k] += dp1 * (double)x[k];
    }
  }
  return loss;
}
