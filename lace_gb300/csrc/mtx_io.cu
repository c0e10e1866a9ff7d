// Matrix Market files for LACE's data_d_matrix, on host threads:
// read_z_csr_from_mtx / data_z_csr_mtx (control/magma_zmio.cpp:92-351,
// 941-955) and data_zwrite_csr_mtx (:587-774).
//
// LACE reads one entry per fscanf call and writes one per fprintf call, which
// makes the generate_iLU -> solver file exchange (factors written, read back)
// take seconds for a million-row system.  Here the file is read whole, split
// into line-aligned chunks that host threads parse with correctly rounded
// conversions (std::from_chars, as scanf's %lf rounds), and written from
// per-thread buffers formatted like %.16g (std::to_chars with precision 16 is
// specified as printf's %g).  The results are LACE's: the same entries in the
// same order (symmetric files expanded entry by entry; rows filled in file
// order, then each row sorted by column with the same std::sort), and the
// same bytes on output.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include <chrono>

#include "../../include/lace_gb300.h"
#include "hostpar.h"

namespace {

using lace::par_for;

// LACE_GB300_VERBOSE: the reader's phases
struct IoClock {
  bool on = getenv("LACE_GB300_VERBOSE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char *what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    printf("%% mtx %-24s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

// LACE_CALLOC's allocation (include/dense_types.h:430-449): posix_memalign(64)
// and zeroed, so that data_zmfree releases it
template <typename T>
T *calloc64(size_t count) {
  void *p = nullptr;
  const size_t padded = (count * sizeof(T) / 64 + 1) * 64;
  if (posix_memalign(&p, 64, padded) != 0) return nullptr;
  memset(p, 0, padded);
  return (T *)p;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// one token of [p, e) after whitespace; false at the end
bool next_token(const char *&p, const char *e, const char *&t0, const char *&t1) {
  while (p < e && is_space(*p)) ++p;
  if (p >= e) return false;
  t0 = p;
  while (p < e && !is_space(*p)) ++p;
  t1 = p;
  return true;
}

// %d: optional sign, decimal digits
bool parse_int(const char *t0, const char *t1, int &v) {
  if (t0 < t1 && *t0 == '+') ++t0;
  auto r = std::from_chars(t0, t1, v);
  return r.ec == std::errc() && r.ptr == t1;
}

// %lf: from_chars where it reads the whole token (decimal, inf, nan), else
// strtod (hexadecimal floats, a leading '+')
bool parse_double(const char *t0, const char *t1, double &v) {
  auto r = std::from_chars(t0, t1, v);
  if (r.ec == std::errc() && r.ptr == t1) return true;
  std::string s(t0, t1);
  char *end = nullptr;
  v = strtod(s.c_str(), &end);
  return end == s.c_str() + s.size() && !s.empty();
}

struct Banner {
  bool ok = false, coordinate = false, real = false, integer = false, pattern = false, complex = false;
  bool symmetric = false, hermitian = false, skew = false;
};

// mm_read_banner + mm_is_valid (control/mmio.cpp:100-210): five tokens, the
// banner prefix, fields compared in lower case
Banner read_banner(const char *line, const char *e) {
  Banner b;
  const char *p = line, *t0, *t1;
  std::string tok[5];
  for (int k = 0; k < 5; ++k) {
    if (!next_token(p, e, t0, t1)) return b;
    tok[k].assign(t0, t1);
    if (k > 0)
      for (auto &c : tok[k]) c = (char)tolower((unsigned char)c);
  }
  if (tok[0].compare(0, 14, "%%MatrixMarket") != 0 || tok[1] != "matrix") return b;
  if (tok[2] == "coordinate") b.coordinate = true;
  else if (tok[2] != "array") return b;
  if (tok[3] == "real") b.real = true;
  else if (tok[3] == "integer") b.integer = true;
  else if (tok[3] == "pattern") b.pattern = true;
  else if (tok[3] == "complex") b.complex = true;
  else return b;
  if (tok[4] == "symmetric") b.symmetric = true;
  else if (tok[4] == "hermitian") b.hermitian = true;
  else if (tok[4] == "skew-symmetric") b.skew = true;
  else if (tok[4] != "general") return b;
  if (!b.coordinate && b.pattern) return b;  // mm_is_valid
  if (b.real && b.hermitian) return b;
  if (b.pattern && (b.hermitian || b.skew)) return b;
  b.ok = true;
  return b;
}

// one line of [q, le): 1 and the entry when it holds exactly `fields`
// numbers, 0 when it is blank, -1 otherwise
int parse_line(const char *q, const char *le, int fields, bool pattern, int &row, int &col, double &val) {
  const char *t0, *t1;
  if (!next_token(q, le, t0, t1)) return 0;
  if (!parse_int(t0, t1, row)) return -1;
  if (!next_token(q, le, t0, t1) || !parse_int(t0, t1, col)) return -1;
  val = 1.0;
  if (!pattern) {
    if (!next_token(q, le, t0, t1) || !parse_double(t0, t1, val)) return -1;
    for (int f = 3; f < fields; ++f)  // the imaginary part of a complex entry: read, dropped
      if (!next_token(q, le, t0, t1)) return -1;
  }
  return next_token(q, le, t0, t1) ? -1 : 1;
}

// the data entries of [p, e) as LACE's loop reads them: `fields` numbers per
// entry separated by any whitespace (fscanf), nnz entries.  In one parallel
// pass over line-aligned chunks when every line holds one whole entry (each
// chunk into its own arrays, then concatenated in chunk order); else token by
// token.
bool parse_entries(const char *p, const char *e, int nnz, int fields, bool pattern, std::vector<int> &r,
                   std::vector<int> &c, std::vector<double> &v) {
  const size_t bytes = (size_t)(e - p);
  const int nt = std::max(1, std::min(64, (int)(bytes / (1 << 20))));
  std::vector<const char *> cut(nt + 1);
  cut[0] = p;
  cut[nt] = e;
  for (int t = 1; t < nt; ++t) {
    const char *q = p + bytes * t / nt;
    while (q < e && *q != '\n') ++q;
    cut[t] = q < e ? q + 1 : e;
  }
  struct Part {
    std::vector<int> r, c;
    std::vector<double> v;
    bool regular = true;
  };
  std::vector<Part> part(nt);
  par_for((size_t)nt, 1, [&](size_t b0, size_t b1) {
    for (size_t t = b0; t < b1; ++t) {
      Part &P = part[t];
      const size_t guess = (size_t)(cut[t + 1] - cut[t]) / 16 + 16;
      P.r.reserve(guess);
      P.c.reserve(guess);
      P.v.reserve(guess);
      const char *q = cut[t], *end = cut[t + 1];
      while (q < end) {
        const char *le = (const char *)memchr(q, '\n', (size_t)(end - q));
        if (!le) le = end;
        int row, col;
        double val;
        const int got = parse_line(q, le, fields, pattern, row, col, val);
        if (got < 0) {
          P.regular = false;
          break;
        }
        if (got > 0) {
          P.r.push_back(row - 1);
          P.c.push_back(col - 1);
          P.v.push_back(val);
        }
        q = le + 1;
      }
    }
  });
  long long total = 0;
  bool reg = true;
  std::vector<long long> first(nt, 0);
  for (int t = 0; t < nt; ++t) {
    first[t] = total;
    total += (long long)part[t].r.size();
    reg = reg && part[t].regular;
  }
  r.assign(nnz, 0);
  c.assign(nnz, 0);
  v.assign(nnz, pattern ? 1.0 : 0.0);
  if (reg && total >= nnz) {
    par_for((size_t)nt, 1, [&](size_t b0, size_t b1) {
      for (size_t t = b0; t < b1; ++t) {
        const long long k0 = first[t];
        const long long cnt = std::min<long long>((long long)part[t].r.size(), (long long)nnz - k0);
        if (cnt <= 0) continue;
        memcpy(r.data() + k0, part[t].r.data(), 4 * (size_t)cnt);
        memcpy(c.data() + k0, part[t].c.data(), 4 * (size_t)cnt);
        memcpy(v.data() + k0, part[t].v.data(), 8 * (size_t)cnt);
      }
    });
    return true;
  }
  // irregular layout: one token stream, as fscanf reads it
  const char *q = p, *t0, *t1;
  for (int k = 0; k < nnz; ++k) {
    int row, col;
    double val = 1.0;
    if (!next_token(q, e, t0, t1) || !parse_int(t0, t1, row)) return false;
    if (!next_token(q, e, t0, t1) || !parse_int(t0, t1, col)) return false;
    if (!pattern) {
      if (!next_token(q, e, t0, t1) || !parse_double(t0, t1, val)) return false;
      for (int f = 3; f < fields; ++f)
        if (!next_token(q, e, t0, t1)) return false;
    }
    r[k] = row - 1;
    c[k] = col - 1;
    v[k] = val;
  }
  return true;
}

// the file's entries in file order, symmetric and hermitian files expanded
// entry by entry (the part both of LACE's readers share)
int read_coo(const char *filename, int &M, int &N, std::vector<int> &cr, std::vector<int> &cc,
             std::vector<double> &cv, IoClock &clk) {
  FILE *f = fopen(filename, "rb");
  if (!f) return DEV_ERR_NOT_FOUND;
  std::vector<char> buf;
  if (fseek(f, 0, SEEK_END) == 0) {
    const long size = ftell(f);
    if (size > 0) {
      buf.resize((size_t)size);
      fseek(f, 0, SEEK_SET);
      if (fread(buf.data(), 1, buf.size(), f) != buf.size()) buf.clear();
    }
  }
  fclose(f);
  clk.mark("file read");
  const char *p = buf.data(), *e = buf.data() + buf.size();
  // the banner line (at most 1024 characters, as mmio's fgets reads it)
  const char *le = (const char *)memchr(p, '\n', buf.size());
  if (!le) le = e;
  const Banner b = read_banner(p, std::min(le, p + 1024));
  if (!b.ok || !b.coordinate || !(b.real || b.integer || b.pattern || b.complex)) return DEV_ERR_NOT_SUPPORTED;
  p = le < e ? le + 1 : e;
  // comment lines, then the size line (mm_read_mtx_crd_size, mmio.cpp:219-258)
  while (p < e && *p == '%') {
    le = (const char *)memchr(p, '\n', (size_t)(e - p));
    p = le ? le + 1 : e;
  }
  int NZ = 0;
  M = N = 0;
  {
    const char *t0, *t1;
    if (!next_token(p, e, t0, t1) || !parse_int(t0, t1, M) || !next_token(p, e, t0, t1) || !parse_int(t0, t1, N) ||
        !next_token(p, e, t0, t1) || !parse_int(t0, t1, NZ) || M < 0 || N < 0 || NZ < 0)
      return DEV_ERR_UNKNOWN;
  }
  const int fields = b.pattern ? 2 : (b.complex ? 4 : 3);
  if (!parse_entries(p, e, NZ, fields, b.pattern, cr, cc, cv)) return DEV_ERR_UNKNOWN;
  clk.mark("entries parsed");
  for (int k = 0; k < NZ; ++k)
    if (cr[k] < 0 || cr[k] >= M || cc[k] < 0 || cc[k] >= N) return DEV_ERR_ILLEGAL_VALUE;
  // symmetric and hermitian files: each off-diagonal entry followed by its
  // mirror (:215-269); skew-symmetric ones are read as they are
  long long total = NZ;
  if (b.symmetric || b.hermitian) {
    std::vector<int> off(NZ + 1, 0);
    for (int k = 0; k < NZ; ++k) off[k + 1] = off[k] + (cr[k] != cc[k] ? 2 : 1);
    total = off[NZ];
    if (total > 0x7fffffff) return DEV_ERR_NOT_SUPPORTED;
    std::vector<int> nr((size_t)total), nc((size_t)total);
    std::vector<double> nv((size_t)total);
    par_for((size_t)NZ, 1 << 16, [&](size_t b0, size_t b1) {
      for (size_t k = b0; k < b1; ++k) {
        const int o = off[k];
        nr[o] = cr[k];
        nc[o] = cc[k];
        nv[o] = cv[k];
        if (cr[k] != cc[k]) {
          nr[o + 1] = cc[k];
          nc[o + 1] = cr[k];
          nv[o + 1] = cv[k];
        }
      }
    });
    cr.swap(nr);
    cc.swap(nc);
    cv.swap(nv);
  }
  clk.mark("checked, expanded");
  return DEV_SUCCESS;
}

}  // namespace

extern "C" int read_z_csr_from_mtx(data_storage_t *type, int *n_row, int *n_col, int *nnz, dataType **val,
                                   int **row, int **col, const char *filename) {
  if (!type || !n_row || !n_col || !nnz || !val || !row || !col || !filename) return DEV_ERR_INVALID_PTR;
  IoClock clk;
  int M = 0, N = 0;
  std::vector<int> cr, cc;
  std::vector<double> cv;
  const int rc = read_coo(filename, M, N, cr, cc, cv, clk);
  if (rc) return rc;
  const int nz = (int)cr.size();
  // CSR: rows in file order (the stable scatter of :276-313), then each row
  // sorted by column with std::sort on (column, value) pairs (:315-329)
  int *R = calloc64<int>((size_t)M + 1);
  int *C = calloc64<int>((size_t)nz);
  double *V = calloc64<double>((size_t)nz);
  if (!R || !C || !V) {
    free(R);
    free(C);
    free(V);
    return DEV_ERR_HOST_ALLOC;
  }
  for (int k = 0; k < nz; ++k) ++R[cr[k] + 1];
  for (int i = 0; i < M; ++i) R[i + 1] += R[i];
  {
    std::vector<int> next(R, R + M);
    for (int k = 0; k < nz; ++k) {
      const int d = next[cr[k]]++;
      C[d] = cc[k];
      V[d] = cv[k];
    }
  }
  clk.mark("rows filled");
  par_for((size_t)M, 4096, [&](size_t i0, size_t i1) {
    std::vector<std::pair<int, double>> rv;
    for (size_t i = i0; i < i1; ++i) {
      const int kk = R[i], len = R[i + 1] - R[i];
      rv.resize(len);
      for (int q = 0; q < len; ++q) rv[q] = std::make_pair(C[kk + q], V[kk + q]);
      std::sort(rv.begin(), rv.end(),
                [](const std::pair<int, double> &a, const std::pair<int, double> &b) { return a.first < b.first; });
      for (int q = 0; q < len; ++q) {
        C[kk + q] = rv[q].first;
        V[kk + q] = rv[q].second;
      }
    }
  });
  clk.mark("rows sorted");
  *type = Magma_CSR;
  *n_row = M;
  *n_col = N;
  *nnz = nz;
  *row = R;
  *col = C;
  *val = V;
  return DEV_SUCCESS;
}

// LACE's COO reader (control/magma_zmio.cpp:353-557): the entries in file
// order.  LACE labels them Magma_CSR (:409) and, for symmetric files, hands
// back arrays it has just freed (:527-533); here the expanded arrays are
// returned, allocated like LACE_CALLOC.
extern "C" int read_z_coo_from_mtx(data_storage_t *type, int *n_row, int *n_col, int *nnz, dataType **coo_val,
                                   int **coo_row, int **coo_col, const char *filename) {
  if (!type || !n_row || !n_col || !nnz || !coo_val || !coo_row || !coo_col || !filename) return DEV_ERR_INVALID_PTR;
  IoClock clk;
  int M = 0, N = 0;
  std::vector<int> cr, cc;
  std::vector<double> cv;
  const int rc = read_coo(filename, M, N, cr, cc, cv, clk);
  if (rc) return rc;
  const size_t nz = cr.size();
  int *R = calloc64<int>(nz), *C = calloc64<int>(nz);
  double *V = calloc64<double>(nz);
  if (!R || !C || !V) {
    free(R);
    free(C);
    free(V);
    return DEV_ERR_HOST_ALLOC;
  }
  memcpy(R, cr.data(), 4 * nz);
  memcpy(C, cc.data(), 4 * nz);
  memcpy(V, cv.data(), 8 * nz);
  *type = Magma_CSR;
  *n_row = M;
  *n_col = N;
  *nnz = (int)nz;
  *coo_row = R;
  *coo_col = C;
  *coo_val = V;
  return DEV_SUCCESS;
}

extern "C" int data_z_coo_mtx(data_d_matrix *A, const char *filename) {
  if (!A) return DEV_ERR_INVALID_PTR;
  data_storage_t st = Magma_COO;
  return read_z_coo_from_mtx(&st, &A->num_rows, &A->num_cols, &A->nnz, &A->val, &A->row, &A->col, filename);
}

extern "C" int data_z_csr_mtx(data_d_matrix *A, const char *filename) {
  if (!A) return DEV_ERR_INVALID_PTR;
  data_storage_t st = Magma_CSR;
  const int rc = read_z_csr_from_mtx(&st, &A->num_rows, &A->num_cols, &A->nnz, &A->val, &A->row, &A->col, filename);
  if (rc) return rc;
  A->true_nnz = A->nnz;
  A->major = MagmaRowMajor;
  return DEV_SUCCESS;
}

namespace {

// "%d %d %.16g\n" for entries [k0, k1) of rows [i0, i1) of (R, C, V), the
// first number from rows (row-major output) or from columns (column-major)
void format_rows(const int *R, const int *C, const double *V, int i0, int i1, bool col_first, std::string &out) {
  char num[64];
  for (int i = i0; i < i1; ++i)
    for (int k = R[i]; k < R[i + 1]; ++k) {
      const int a = col_first ? C[k] + 1 : i + 1, b = col_first ? i + 1 : C[k] + 1;
      auto r = std::to_chars(num, num + sizeof num, a);
      out.append(num, r.ptr);
      out.push_back(' ');
      r = std::to_chars(num, num + sizeof num, b);
      out.append(num, r.ptr);
      out.push_back(' ');
      r = std::to_chars(num, num + sizeof num, V[k], std::chars_format::general, 16);
      out.append(num, r.ptr);
      out.push_back('\n');
    }
}

}  // namespace

extern "C" int data_zwrite_csr_mtx(data_d_matrix A, data_order_t MajorType, const char *filename) {
  if (!filename) return DEV_ERR_INVALID_PTR;
  if (A.storage_type == Magma_DENSE || A.storage_type == Magma_BCSR) return DEV_ERR_NOT_SUPPORTED;
  const int nr = A.num_rows, nc = A.num_cols, nz = A.nnz;
  if (nr < 0 || (nr > 0 && !A.row) || (nz > 0 && (!A.col || !A.val))) return DEV_ERR_INVALID_PTR;
  // column-major output of a row-major matrix: its transpose, rows of the
  // transpose in ascending order of the original rows (:597-651)
  const bool transpose = MajorType == MagmaColMajor && A.major != MagmaColMajor;
  std::vector<int> tr, tc;
  std::vector<double> tv;
  const int *R = A.row, *C = A.col;
  const double *V = A.val;
  int rows = nr;
  if (transpose) {
    tr.assign((size_t)nc + 1, 0);
    tc.resize((size_t)nz);
    tv.resize((size_t)nz);
    for (int k = 0; k < A.row[nr]; ++k) ++tr[A.col[k] + 1];
    for (int j = 0; j < nc; ++j) tr[j + 1] += tr[j];
    std::vector<int> next(tr.begin(), tr.end() - 1);
    for (int i = 0; i < nr; ++i)
      for (int k = A.row[i]; k < A.row[i + 1]; ++k) {
        const int d = next[A.col[k]]++;
        tc[d] = i;
        tv[d] = A.val[k];
      }
    R = tr.data();
    C = tc.data();
    V = tv.data();
    rows = nc;
  }
  FILE *fp = fopen(filename, "w");
  if (!fp) return -1;  // :606-610
  fprintf(fp, "%%%%MatrixMarket matrix coordinate real general\n");
  // (rows, columns) of A either way: LACE prints the transpose's (columns, rows)
  fprintf(fp, "%d %d %d\n", nr, nc, nz);
  // per-thread buffers of whole rows, written in order
  const int nt = std::max(1, std::min(16, (int)(((size_t)(R[rows] - R[0]) * 32) >> 20)));
  std::vector<std::string> part(nt);
  par_for((size_t)nt, 1, [&](size_t b0, size_t b1) {
    for (size_t t = b0; t < b1; ++t) {
      const int i0 = (int)((long long)rows * t / nt), i1 = (int)((long long)rows * (t + 1) / nt);
      part[t].reserve((size_t)(R[i1] - R[i0]) * 32);
      format_rows(R, C, V, i0, i1, transpose, part[t]);
    }
  });
  bool ok = true;
  for (auto &s : part) ok = ok && fwrite(s.data(), 1, s.size(), fp) == s.size();
  if (fclose(fp) != 0) ok = false;
  return ok ? DEV_SUCCESS : DEV_ERR_UNKNOWN;
}
