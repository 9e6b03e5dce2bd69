// MatrixMarket files -> CSR (host code, no GPU). The same reading as the
// reference's CooMatrix::InitMarket and CsrMatrix::Init
// (conjugateGradient/matrix/sparse_matrix.h:217-380, 633-730):
//   * banner flags by substring: "symmetric", "skew", "array";
//   * coordinate entries "row col [value]" (1-based; a missing value reads as
//     1.0, the reference's default), array entries column-major;
//   * symmetric files: every off-diagonal entry is mirrored (negated for
//     skew-symmetric);
//   * entries stably sorted by (row, column); duplicates are kept, not summed.
// Errors come back as status codes with a message, never exit().
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "runtime.cuh"

namespace perks {
namespace {

struct Entry {
  int row, col;
  double val;
};

int read_market(const char* path, int* rows_out, int* cols_out, std::vector<Entry>* out) {
  if (!path) return fail(PERKS_ERR_INVALID_ARG, "path is NULL");
  std::ifstream in(path);
  if (!in.good()) return fail(PERKS_ERR_INVALID_ARG, std::string("cannot open ") + path);
  bool array = false, symmetric = false, skew = false, have_size = false;
  long long rows = 0, cols = 0, declared = 0, seen = 0;
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line[0] == '%') {
      if (line.size() > 1 && line[1] == '%') {
        symmetric = line.find("symmetric") != std::string::npos;
        skew = line.find("skew") != std::string::npos;
        array = line.find("array") != std::string::npos;
      }
      continue;
    }
    if (line.find_first_not_of(" \t\r") == std::string::npos) continue;  // blank line
    if (!have_size) {
      long long a = 0, b = 0, c = 0;
      const int n = std::sscanf(line.c_str(), "%lld %lld %lld", &a, &b, &c);
      if (!array && n == 3) {
        declared = c;
      } else if (array && n >= 2) {
        declared = a * b;
      } else {
        return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: invalid size line: " + line);
      }
      if (a <= 0 || b <= 0 || a > 0x7fffffff || b > 0x7fffffff || declared < 0)
        return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: bad dimensions: " + line);
      rows = a;
      cols = b;
      have_size = true;
      out->reserve(size_t(symmetric ? 2 * declared : declared));
      continue;
    }
    if (seen >= declared) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: more entries than declared");
    Entry e{};
    if (array) {
      char* t = nullptr;
      e.val = std::strtod(line.c_str(), &t);
      if (t == line.c_str()) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: bad array entry: " + line);
      e.col = int(seen / rows);
      e.row = int(seen - rows * e.col);
    } else {
      const char* l = line.c_str();
      char* t = nullptr;
      const long r = std::strtol(l, &t, 0);
      if (t == l) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: bad row: " + line);
      l = t;
      const long c = std::strtol(l, &t, 0);
      if (t == l) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: bad column: " + line);
      l = t;
      e.val = std::strtod(l, &t);
      if (t == l) e.val = 1.0;  // pattern entry
      if (r < 1 || r > rows || c < 1 || c > cols) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: index out of range: " + line);
      e.row = int(r - 1);
      e.col = int(c - 1);
    }
    out->push_back(e);
    seen++;
    if (symmetric && e.row != e.col) out->push_back(Entry{e.col, e.row, skew ? -e.val : e.val});
  }
  if (!have_size) return fail(PERKS_ERR_INVALID_ARG, "MatrixMarket: no size line");
  std::stable_sort(out->begin(), out->end(),
                   [](const Entry& a, const Entry& b) { return a.row != b.row ? a.row < b.row : a.col < b.col; });
  *rows_out = int(rows);
  *cols_out = int(cols);
  return PERKS_OK;
}

}  // namespace
}  // namespace perks

using namespace perks;

extern "C" {

int perks_mtx_size(const char* path, int* rows, int* cols, long long* nnz) {
  if (!rows || !cols || !nnz) return fail(PERKS_ERR_INVALID_ARG, "NULL output");
  std::vector<Entry> e;
  const int rc = read_market(path, rows, cols, &e);
  if (rc != PERKS_OK) return rc;
  *nnz = (long long)e.size();
  return PERKS_OK;
}

int perks_mtx_read_csr(const char* path, int rows, long long nnz_cap, int* row_ptr, int* col, double* val,
                       long long* nnz) {
  if (!row_ptr || !col || !val || !nnz) return fail(PERKS_ERR_INVALID_ARG, "NULL output");
  std::vector<Entry> e;
  int r = 0, c = 0;
  const int rc = read_market(path, &r, &c, &e);
  if (rc != PERKS_OK) return rc;
  if (r != rows) return fail(PERKS_ERR_INVALID_ARG, "row count differs from perks_mtx_size");
  if ((long long)e.size() > nnz_cap) return fail(PERKS_ERR_INVALID_ARG, "more entries than nnz_cap");
  if (e.size() > 0x7fffffffull) return fail(PERKS_ERR_UNSUPPORTED, "more than 2^31-1 entries");
  // row_ptr[i] = first entry of row i (entries are sorted by row)
  long long j = 0;
  for (int i = 0; i < rows; i++) {
    row_ptr[i] = int(j);
    while (j < (long long)e.size() && e[j].row == i) j++;
  }
  row_ptr[rows] = int(e.size());
  for (size_t k = 0; k < e.size(); k++) {
    col[k] = e[k].col;
    val[k] = e[k].val;
  }
  *nnz = (long long)e.size();
  return PERKS_OK;
}

}  // extern "C"
