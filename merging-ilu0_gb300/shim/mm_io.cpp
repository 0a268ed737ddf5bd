// Drop-in Matrix Market batch I/O: FillSubdir, ReadData, Print_ans and
// PrintSolverResults with the behaviour of ReadWriteData.cpp of
// Batched-ILU0-merged/ILU0_ISAI_bicgstab, on this project's own Matrix Market
// parser (no mmio).
//
//   FillSubdir        readdir order, "." and ".." skipped, paths main_dir + name
//                     (ReadWriteData.cpp:89-113)
//   ReadData          Problem_Size * #subdir pages; page p is read from
//                     subdir[p % #subdir]; A.mtx / b.mtx, or A_scaled.mtx /
//                     b_scaled.mtx when is_scaled; every page must repeat page 0's
//                     pattern (ReadWriteData.cpp:258-490)
//   COO -> CSR        counting sort by row, then columns ascending within a row;
//                     symmetric files are expanded to both triangles
//                     (ReadWriteData.cpp:117-255)
//   Print_ans         "%%MatrixMarket matrix array real general", "M 1", one
//                     "%0.17lg" value per line, for the first #subdir pages
//                     (ReadWriteData.cpp:16-54)
//   PrintSolverResults "%d   %f  " per subdirectory: conv flag, iteration count
//                     (ReadWriteData.cpp:57-86)
//
// Errors in the input files print a message and end the process with the
// original's exit codes (1, or 0 for a differing nonzero count, an empty or
// unreadable directory), because the original drivers rely on them.
#include <dirent.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <utility>
#include <vector>

#include "ReadWriteData.h"
#include "SolverResults.h"
#include "matrix.h"

namespace {

struct Banner {
  std::string object, format, field, symmetry;
};

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// reads the banner line; false if the file does not start with one
bool read_banner(FILE* f, Banner* b) {
  char line[1025];
  if (!std::fgets(line, sizeof(line), f)) return false;
  char t0[128] = "", t1[128] = "", t2[128] = "", t3[128] = "", t4[128] = "";
  if (std::sscanf(line, "%127s %127s %127s %127s %127s", t0, t1, t2, t3, t4) != 5) return false;
  if (std::strcmp(t0, "%%MatrixMarket") != 0) return false;
  b->object = lower(t1);
  b->format = lower(t2);
  b->field = lower(t3);
  b->symmetry = lower(t4);
  return true;
}

// skips comment and blank lines, then parses `count` integers of the size line
bool read_size(FILE* f, int* v, int count) {
  char line[1025];
  while (std::fgets(line, sizeof(line), f)) {
    if (line[0] == '%') continue;
    const char* p = line;
    while (*p && std::isspace((unsigned char)*p)) ++p;
    if (!*p) continue;
    if (count == 3) return std::sscanf(line, "%d %d %d", v, v + 1, v + 2) == 3;
    return std::sscanf(line, "%d %d", v, v + 1) == 2;
  }
  return false;
}

[[noreturn]] void stop(const std::string& msg, int code) {
  std::cout << msg << std::endl;
  std::exit(code);
}

void coo_to_csr(int m, const std::vector<int>& ri, const std::vector<int>& cj, const std::vector<double>& v, int* rp,
                int* ci, double* vals) {
  const int nz = (int)ri.size();
  std::fill(rp, rp + m + 1, 0);
  for (int k = 0; k < nz; ++k) ++rp[ri[k] + 1];
  for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
  std::vector<int> next(rp, rp + m);
  for (int k = 0; k < nz; ++k) {
    const int d = next[ri[k]]++;
    ci[d] = cj[k];
    vals[d] = v[k];
  }
  std::vector<std::pair<int, double>> row;
  for (int i = 0; i < m; ++i) {
    row.clear();
    for (int k = rp[i]; k < rp[i + 1]; ++k) row.emplace_back(ci[k], vals[k]);
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      ci[k] = row[k - rp[i]].first;
      vals[k] = row[k - rp[i]].second;
    }
  }
}

void read_A_and_b(int problem_id, const std::string& dir, PagedCSRMatrices& A, PagedVectors& b, bool is_scaled) {
  const std::string fa = dir + (is_scaled ? "/A_scaled.mtx" : "/A.mtx");
  const std::string fb = dir + (is_scaled ? "/b_scaled.mtx" : "/b.mtx");
  FILE* f = std::fopen(fa.c_str(), "r");
  if (!f) stop("cannot open " + fa, 1);
  Banner ba;
  if (!read_banner(f, &ba)) stop("no Matrix Market banner in " + fa, 1);
  if (ba.object != "matrix" || ba.format != "coordinate")
    stop(fa + ": A must be a 'matrix coordinate' file, not '" + ba.object + " " + ba.format + "'", 1);
  int sz[3];
  if (!read_size(f, sz, 3)) stop(fa + ": no size line", 1);
  const int M = sz[0], N = sz[1], nz_file = sz[2];
  if (M != N) stop(fa + ": A is not square", 1);
  const bool symmetric = ba.symmetry == "symmetric";
  if (ba.symmetry != "general" && !symmetric) stop(fa + ": unsupported symmetry " + ba.symmetry, 1);
  if (ba.field != "real" && ba.field != "integer") stop(fa + ": unsupported field " + ba.field, 1);
  std::vector<int> ri, cj;
  std::vector<double> v;
  ri.reserve(symmetric ? 2 * nz_file : nz_file);
  for (int k = 0; k < nz_file; ++k) {
    int I, J;
    double val;
    if (std::fscanf(f, "%d %d %lg", &I, &J, &val) != 3) stop("premature end of " + fa, 1);
    --I;
    --J;
    if (I < 0 || I >= M || J < 0 || J >= N) stop("entry out of range in " + fa, 1);
    ri.push_back(I);
    cj.push_back(J);
    v.push_back(val);
    if (symmetric && I != J) {
      ri.push_back(J);
      cj.push_back(I);
      v.push_back(val);
    }
  }
  std::fclose(f);
  const int true_nz = (int)ri.size();

  FILE* g = std::fopen(fb.c_str(), "r");
  if (!g) stop("cannot open " + fb, 1);
  Banner bb;
  if (!read_banner(g, &bb)) stop("no Matrix Market banner in " + fb, 1);
  if (bb.object != "matrix" || bb.format != "array")
    stop(fb + ": b must be a 'matrix array' file, not '" + bb.object + " " + bb.format + "'", 1);
  int bs[2];
  if (!read_size(g, bs, 2)) stop(fb + ": no size line", 1);
  if (bs[1] != 1 || bs[0] != M) stop(fb + ": b is not one column of " + std::to_string(M) + " rows", 1);
  if (bb.field != "real" && bb.field != "integer") stop(fb + ": unsupported field " + bb.field, 1);

  if (problem_id == 0) {
    A.SetNumRows(M);
    A.SetNumCols(N);
    A.SetNumNz(true_nz);
    A.AllocateMemory(LOCATION::CPU);
    coo_to_csr(M, ri, cj, v, A.GetPtrToCpuRowPtrs(), A.GetPtrToCpuColInd(), A.GetPtrToCpuValues());
  } else {
    if (M != A.GetNumRows() || N != A.GetNumCols()) stop(fa + ": size differs from the first system's", 1);
    if (true_nz != A.GetNumNz()) stop(fa + ": nonzero count differs from the first system's", 0);
    std::vector<int> rp(M + 1), ci(true_nz);
    std::vector<double> vals(true_nz);
    coo_to_csr(M, ri, cj, v, rp.data(), ci.data(), vals.data());
    if (!std::equal(ci.begin(), ci.end(), A.GetPtrToCpuColInd()) ||
        !std::equal(rp.begin(), rp.begin() + M, A.GetPtrToCpuRowPtrs()))
      stop(fa + ": sparsity pattern differs from the first system's", 1);
    std::copy(vals.begin(), vals.end(), A.GetPtrToCpuValues() + (size_t)problem_id * true_nz);
  }

  if (problem_id == 0) {
    b.SetNumElements(bs[0]);
    b.AllocateMemory(LOCATION::CPU);
  }
  double* bv = b.GetPtrToCpuValues() + (size_t)problem_id * M;
  for (int i = 0; i < M; ++i)
    if (std::fscanf(g, "%lg", bv + i) != 1) stop("premature end of " + fb, 1);
  std::fclose(g);
}

}  // namespace

void FillSubdir(const std::string& main_dir, std::vector<std::string>& subdir) {
  DIR* dr = opendir(main_dir.c_str());
  if (!dr) {
    std::cout << "cannot open directory " << main_dir << std::endl;
    std::exit(0);
  }
  while (dirent* de = readdir(dr)) {
    if (std::strcmp(de->d_name, ".") == 0 || std::strcmp(de->d_name, "..") == 0) continue;
    subdir.push_back(main_dir + std::string(de->d_name));
  }
  closedir(dr);
}

void ReadData(const int Problem_Size, const std::vector<std::string>& subdir, PagedCSRMatrices& A_pages,
              PagedVectors& b_pages, const bool is_scaled) {
  const int num_pages = Problem_Size * (int)subdir.size();
  A_pages.SetNumPages(num_pages);
  b_pages.SetNumPages(num_pages);
  if (num_pages == 0) {
    std::cout << "no systems to read (empty directory or Problem_Size 0)" << std::endl;
    std::exit(0);
  }
  for (int p = 0; p < num_pages; ++p) read_A_and_b(p, subdir[p % subdir.size()], A_pages, b_pages, is_scaled);
  std::cout << "read " << num_pages << " systems from " << subdir.size() << " directories" << std::endl;
}

void Print_ans(const std::vector<std::string>& subdir, const PagedVectors& Ans_pages, const std::string& ans_name) {
  if (!Ans_pages.ExistsCPU()) {
    std::cerr << "Print_ans: the solution is not on the CPU" << std::endl;
    std::abort();
  }
  const int M = Ans_pages.GetNumElements();
  for (size_t p = 0; p < subdir.size(); ++p) {
    const std::string path = subdir[p] + "/" + ans_name;
    FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) {
      std::fprintf(stderr, "Print_ans: cannot write %s\n", path.c_str());
      continue;
    }
    std::fprintf(fp, "%%%%MatrixMarket matrix array real general\n%d %d\n", M, 1);
    const double* x = Ans_pages.GetPtrToCpuValues() + p * (size_t)M;
    for (int i = 0; i < M; ++i) std::fprintf(fp, "%0.17lg\n", x[i]);
    std::fclose(fp);
  }
}

void PrintSolverResults(const std::vector<std::string>& subdir, const SolverResults& solver_results,
                        const std::string& f_name) {
  if (!solver_results.ExistsCPU()) {
    std::cerr << "PrintSolverResults: the results are not on the CPU" << std::endl;
    std::abort();
  }
  FILE* fp = std::fopen(f_name.c_str(), "w");
  if (!fp) {
    std::fprintf(stderr, "PrintSolverResults: cannot write %s\n", f_name.c_str());
    return;
  }
  for (size_t i = 0; i < subdir.size(); ++i)
    std::fprintf(fp, "%d   %f  \n", solver_results.GetPtrToCpuConvFlag()[i], solver_results.GetPtrToCpuIterCount()[i]);
  std::fclose(fp);
}
