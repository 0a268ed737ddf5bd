// Seeded synthetic batches of the benchmark workloads (host only).
//
// The reference reads Matrix Market directories (ReadWriteData.cpp:258-490)
// that are not shipped with it; these generators stand in for them with the
// shapes and value distributions of the benchmark configurations.  Random
// numbers: splitmix64 (Steele, Lea, Flood 2014 / Vigna) seeded per system, so
// any system of any batch can be regenerated independently and in parallel.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "bilu.h"
#include "bilu_internal.h"

namespace bilu {

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed, uint64_t stream) {
    s = seed ^ (0xD1B54A32D192ED03ull * (stream + 1));
    next();
  }
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double sym() { return 2.0 * u01() - 1.0; }                                      // [-1,1)
  double normal() {  // Box-Muller, one of the pair
    double u1 = 1.0 - u01();
    double u2 = u01();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// Pattern of a 2D 5-point (gz == 1) or 3D 7-point stencil in natural ordering,
// columns ascending within each row.
static void stencil_pattern(int gx, int gy, int gz, std::vector<int>& rp, std::vector<int>& ci) {
  const int n = gx * gy * gz;
  rp.assign(n + 1, 0);
  ci.clear();
  for (int z = 0; z < gz; ++z)
    for (int y = 0; y < gy; ++y)
      for (int x = 0; x < gx; ++x) {
        const int i = (z * gy + y) * gx + x;
        if (z > 0) ci.push_back(i - gx * gy);
        if (y > 0) ci.push_back(i - gx);
        if (x > 0) ci.push_back(i - 1);
        ci.push_back(i);
        if (x < gx - 1) ci.push_back(i + 1);
        if (y < gy - 1) ci.push_back(i + gx);
        if (z < gz - 1) ci.push_back(i + gx * gy);
        rp[i + 1] = (int)ci.size();
      }
}

}  // namespace bilu

using namespace bilu;

// systems first .. first+nsys-1 of the seeded stream (system s draws from Rng(seed, s))
static bilu_status gen_stencil(int kind, int gx, int gy, int gz, long long first, int nsys, uint64_t seed,
                               int* n_out, int* nnz_out, int* h_row_ptrs, int* h_col_idxs, double* h_values,
                               double* h_b) {
  if (gx <= 0 || gy <= 0 || gz <= 0 || nsys < 0 || first < 0)
    return set_error(BILU_ERR_INVALID, "bilu_gen_stencil: bad sizes");
  if (!(kind == 1 || kind == 2 || kind == 4 || kind == 5))
    return set_error(BILU_ERR_INVALID, "bilu_gen_stencil: kind must be 1, 2, 4 or 5");
  std::vector<int> rp, ci;
  stencil_pattern(gx, gy, gz, rp, ci);
  const int n = gx * gy * gz;
  const int nnz = (int)ci.size();
  if (n_out) *n_out = n;
  if (nnz_out) *nnz_out = nnz;
  if (h_row_ptrs) std::memcpy(h_row_ptrs, rp.data(), sizeof(int) * (n + 1));
  if (h_col_idxs) std::memcpy(h_col_idxs, ci.data(), sizeof(int) * nnz);
  if (!h_values && !h_b) return BILU_OK;

#pragma omp parallel for schedule(static)
  for (int s = 0; s < nsys; ++s) {
    Rng rng(seed, (uint64_t)(first + s));
    double peclet = 0.0;
    if (kind == 2) peclet = 0.5 * rng.u01();
    if (kind == 4) peclet = 2.0 * rng.u01();
    double* v = h_values ? h_values + (size_t)s * nnz : nullptr;
    for (int i = 0; i < n; ++i) {
      const int beg = rp[i], end = rp[i + 1];
      // per-row draws happen in a fixed order whether or not values are wanted
      double skew = 0.0;
      if (kind == 1) skew = 0.3 * rng.u01();
      for (int k = beg; k < end; ++k) {
        const int j = ci[k];
        double a;
        if (kind == 1) {
          if (j == i) a = 4.0 + rng.u01();
          else {
            a = -(1.0 + 0.2 * rng.sym());
            if (j == i + 1) a += skew;       // east
            else if (j == i - 1) a -= skew;  // west
          }
        } else if (kind == 2) {
          if (j == i) a = 6.0 + rng.u01();
          else {
            a = -(1.0 + 0.25 * rng.sym());
            if (j == i + 1) a += 0.5 * peclet;
            else if (j == i - 1) a -= 0.5 * peclet;
          }
        } else if (kind == 4) {
          // -Laplace(u) + Pe * du/dx, unit mesh, first-order upwind for the x-convection
          if (j == i) a = 4.0 + peclet;
          else if (j == i - 1) a = -1.0 - peclet;
          else a = -1.0;
        } else {  // kind 5
          if (j == i) a = 6.0 + rng.u01();
          else a = -(1.0 + 0.3 * rng.sym());
        }
        if (v) v[k] = a;
      }
    }
    if (h_b) {
      double* bb = h_b + (size_t)s * n;
      for (int i = 0; i < n; ++i) bb[i] = rng.sym();
    }
  }
  return BILU_OK;
}

extern "C" bilu_status bilu_gen_stencil(int kind, int gx, int gy, int gz, int nsys, uint64_t seed, int* n_out,
                                        int* nnz_out, int* h_row_ptrs, int* h_col_idxs, double* h_values,
                                        double* h_b) {
  return gen_stencil(kind, gx, gy, gz, 0, nsys, seed, n_out, nnz_out, h_row_ptrs, h_col_idxs, h_values, h_b);
}

extern "C" bilu_status bilu_gen_stencil_range(int kind, int gx, int gy, int gz, long long first, int nsys,
                                              uint64_t seed, int* n_out, int* nnz_out, int* h_row_ptrs,
                                              int* h_col_idxs, double* h_values, double* h_b) {
  return gen_stencil(kind, gx, gy, gz, first, nsys, seed, n_out, nnz_out, h_row_ptrs, h_col_idxs, h_values, h_b);
}

// Uneven batch: per-system sizes n_s = floor(exp(U(ln nmin, ln nmax))), per row
// k ~ U{kmin..kmax} distinct off-diagonal columns plus the diagonal (sorted),
// off-diagonals ~ N(0,1), a_ii = 1.2 * sum_j |a_ij| * sign, sign ~ U{+-1}.
// Two passes: with h_row_ptrs == NULL only sys_n / sys_nnz are filled.
// Layout of the outputs: systems back to back; sys_row_off / sys_nnz_off
// (nsys+1 entries each, exclusive prefix sums) locate each system; row
// pointers are per system and local (start at 0).
extern "C" bilu_status bilu_gen_uneven(int nsys, uint64_t seed, int nmin, int nmax, int kmin, int kmax,
                                       int* sys_n, int* sys_nnz, int* h_row_ptrs, int* h_col_idxs,
                                       double* h_values, double* h_b) {
  if (nsys < 0 || nmin < 2 || nmax < nmin || kmin < 0 || kmax < kmin || kmax >= nmin)
    return set_error(BILU_ERR_INVALID, "bilu_gen_uneven: bad sizes");
  if (!sys_n || !sys_nnz) return set_error(BILU_ERR_INVALID, "bilu_gen_uneven: sys_n/sys_nnz required");
  const double lmin = std::log((double)nmin), lmax = std::log((double)nmax);
  // pass 1: sizes (cheap, serial so that offsets can be formed)
  for (int s = 0; s < nsys; ++s) {
    Rng rng(seed, (uint64_t)s);
    int n = (int)std::floor(std::exp(lmin + (lmax - lmin) * rng.u01()));
    n = std::min(std::max(n, nmin), nmax);
    long long nnz = n;  // diagonals
    for (int i = 0; i < n; ++i) nnz += kmin + (int)(rng.next() % (uint64_t)(kmax - kmin + 1));
    sys_n[s] = n;
    sys_nnz[s] = (int)nnz;
  }
  if (!h_row_ptrs) return BILU_OK;
  std::vector<long long> roff(nsys + 1, 0), zoff(nsys + 1, 0);
  for (int s = 0; s < nsys; ++s) {
    roff[s + 1] = roff[s] + sys_n[s];
    zoff[s + 1] = zoff[s] + sys_nnz[s];
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int s = 0; s < nsys; ++s) {
    Rng rng(seed, (uint64_t)s);
    const int n = sys_n[s];
    rng.u01();  // the size draw
    std::vector<int> rowk(n);
    for (int i = 0; i < n; ++i) rowk[i] = kmin + (int)(rng.next() % (uint64_t)(kmax - kmin + 1));
    int* rp = h_row_ptrs + roff[s] + s;  // n+1 entries per system
    int* ci = h_col_idxs + zoff[s];
    double* va = h_values ? h_values + zoff[s] : nullptr;
    double* bb = h_b ? h_b + roff[s] : nullptr;
    std::vector<int> cols;
    std::vector<double> vals;
    int pos = 0;
    rp[0] = 0;
    for (int i = 0; i < n; ++i) {
      cols.clear();
      // distinct off-diagonal columns by rejection
      while ((int)cols.size() < rowk[i]) {
        int j = (int)(rng.next() % (uint64_t)n);
        if (j == i) continue;
        if (std::find(cols.begin(), cols.end(), j) != cols.end()) continue;
        cols.push_back(j);
      }
      std::sort(cols.begin(), cols.end());
      double rowsum = 0.0;
      vals.assign(cols.size(), 0.0);
      for (size_t q = 0; q < cols.size(); ++q) {
        vals[q] = rng.normal();
        rowsum += std::fabs(vals[q]);
      }
      const double sign = (rng.next() & 1ull) ? 1.0 : -1.0;
      double diag = 1.2 * rowsum * sign;
      if (diag == 0.0) diag = 1.0;  // an empty row (kmin = 0) still gets a nonzero pivot
      bool placed = false;
      for (size_t q = 0; q <= cols.size(); ++q) {
        if (!placed && (q == cols.size() || cols[q] > i)) {
          ci[pos] = i;
          if (va) va[pos] = diag;
          ++pos;
          placed = true;
        }
        if (q < cols.size()) {
          ci[pos] = cols[q];
          if (va) va[pos] = vals[q];
          ++pos;
        }
      }
      rp[i + 1] = pos;
    }
    if (bb)
      for (int i = 0; i < n; ++i) bb[i] = rng.sym();
  }
  return BILU_OK;
}
