// The setup conversions a LACE caller runs before the solve, on host threads:
// data_zmconvert (control/magma_zmconverter.cpp:199-1601) for the storage
// changes the factorisation path uses and COO -> CSR, data_zmtranspose
// (control/magma_zmtranspose.cpp:85-515) and data_rowindex
// (control/magma_zmconverter.cpp:145-167).
//
// LACE walks each conversion in one serial loop; here rows are counted in
// parallel, offsets come from one prefix sum, and rows are filled in
// parallel.  The transpose counts each row range's columns into a per-thread
// histogram, so every thread knows where its entries of each column start
// and the output keeps LACE's order (each column's entries by ascending row).
// Results are LACE's field for field and array for array, including what its
// loops produce on unusual inputs:
//  * a split whose diagorder_type is none of UNITY/VALUE/ZERO/NODIAG counts
//    the diagonal in nnz but leaves it out of the rows (CSRL; the nnz tail
//    stays zero), and the transpose of such a matrix counts those tail
//    entries in column 0's pointer arithmetic, as LACE's does;
//  * one-based input to the transpose gives one-based output;
//  * BCSR -> BCSRL labels the result Magma_BCSR, and a UNITY diagonal block
//    holds ones on its diagonal only; the block transpose moves blocks
//    without transposing their contents.
// Differences kept on purpose: a transpose whose column count exceeds its row
// count gets a pointer array long enough for its columns (LACE's writes past
// its allocation); CSR -> BCSR without a block size returns
// DEV_ERR_NOT_SUPPORTED (LACE exits the process); conversions outside the
// list above return DEV_ERR_NOT_SUPPORTED and leave B untouched.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/lace_gb300.h"
#include "hostpar.h"

namespace {

using lace::par_for;

template <typename T>
T *calloc64(size_t count) {
  void *p = nullptr;
  const size_t padded = (count * sizeof(T) / 64 + 1) * 64;
  if (posix_memalign(&p, 64, padded) != 0) return nullptr;
  char *c = (char *)p;
  lace::par_ranges(padded, [c](size_t o, size_t len) { memset(c + o, 0, len); });
  return (T *)p;
}

int row_limit(const data_d_matrix &A) { return (A.pad_rows > 0 && A.pad_cols > 0) ? A.pad_rows : A.num_rows; }

void release(data_d_matrix *B) {
  free(B->val);
  free(B->col);
  free(B->row);
  free(B->rowidx);
  free(B->list);
  free(B->blockinfo);
  free(B->diag);
  B->val = B->diag = nullptr;
  B->row = B->col = B->rowidx = B->list = B->blockinfo = nullptr;
}

constexpr size_t kGrain = 1 << 14;

// exclusive prefix sum of cnt[0..n) into out[0..n], out[0] = 0
void prefix(const std::vector<int> &cnt, int *out, size_t n) {
  long long s = 0;
  out[0] = 0;
  for (size_t i = 0; i < n; ++i) {
    s += cnt[i];
    out[i + 1] = (int)s;
  }
}

// CSR -> CSR copy (:263-295)
int copy_csr(const data_d_matrix &A, data_d_matrix *B) {
  const int R = row_limit(A);
  B->storage_type = Magma_CSR;
  B->major = MagmaRowMajor;
  B->fill_mode = A.fill_mode;
  B->num_rows = A.num_rows;
  B->num_cols = A.num_cols;
  B->pad_rows = A.pad_rows;
  B->pad_cols = A.pad_cols;
  B->nnz = A.nnz;
  B->true_nnz = A.true_nnz;
  B->max_nnz_row = A.max_nnz_row;
  B->diameter = A.diameter;
  B->val = calloc64<double>((size_t)std::max(A.nnz, 0));
  B->row = calloc64<int>((size_t)R + 1);
  B->col = calloc64<int>((size_t)std::max(A.nnz, 0));
  if (!B->val || !B->row || !B->col) return DEV_ERR_HOST_ALLOC;
  const size_t nz = (size_t)std::max(A.nnz, 0);
  par_for(nz, 1 << 18, [&](size_t b, size_t e) {
    memcpy(B->val + b, A.val + b, 8 * (e - b));
    memcpy(B->col + b, A.col + b, 4 * (e - b));
  });
  memcpy(B->row, A.row, 4 * ((size_t)R + 1));
  return DEV_SUCCESS;
}

// the row index of every entry of rows [0, R) (:143-167, :505-540)
void fill_rowidx(const data_d_matrix &A, int R, int *out) {
  par_for((size_t)R, kGrain, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i)
      for (int j = A.row[i]; j < A.row[i + 1]; ++j) out[j] = (int)i;
  });
}

// CSR -> CSRL (lower) or CSRU (upper) (:304-461); `bs` > 0 splits a BCSR
// matrix by blocks (:1249-1437)
int split(const data_d_matrix &A, data_d_matrix *B, bool lower, int bs) {
  const int R = row_limit(A);
  const data_diagorder_t d = B->diagorder_type;
  const int ld = bs > 0 ? A.ldblock : 1;
  std::vector<int> kept((size_t)R), counted((size_t)R);
  par_for((size_t)R, kGrain, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      int k = 0, c = 0;
      for (int j = A.row[i]; j < A.row[i + 1]; ++j) {
        const int col = A.col[j];
        if (lower ? col < (int)i : col > (int)i) {
          ++k;
          ++c;
        } else if (col == (int)i && d != Magma_NODIAG) {
          ++c;
          // CSRL/BCSRL keep the diagonal only for UNITY, VALUE and ZERO; the
          // upper splits also keep it by default
          if (d == Magma_UNITY || d == Magma_VALUE || d == Magma_ZERO || !lower) ++k;
        }
      }
      kept[i] = k;
      counted[i] = c;
    }
  });
  long long total = 0;
  for (int i = 0; i < R; ++i) total += counted[i];
  B->major = MagmaRowMajor;
  B->fill_mode = lower ? MagmaLower : MagmaUpper;
  B->num_rows = A.num_rows;
  B->num_cols = A.num_cols;
  B->pad_rows = A.pad_rows;
  B->pad_cols = A.pad_cols;
  B->diameter = A.diameter;
  if (bs > 0) {
    B->storage_type = lower ? Magma_BCSR : Magma_BCSRU;
    B->blocksize = A.blocksize;
    B->ldblock = A.ldblock;
    B->numblocks = (int)total;
    B->nnz = (int)total * B->ldblock;
  } else {
    B->storage_type = lower ? Magma_CSRL : Magma_CSRU;
    B->nnz = (int)total;
    B->true_nnz = (int)total;
  }
  B->val = calloc64<double>((size_t)total * ld);
  B->row = calloc64<int>((size_t)R + 1);
  B->col = calloc64<int>((size_t)total);
  if (!B->val || !B->row || !B->col) return DEV_ERR_HOST_ALLOC;
  prefix(kept, B->row, (size_t)R);
  par_for((size_t)R, kGrain, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      int o = B->row[i];
      for (int j = A.row[i]; j < A.row[i + 1]; ++j) {
        const int col = A.col[j];
        const bool off = lower ? col < (int)i : col > (int)i;
        if (!off && col != (int)i) continue;
        double *dst = B->val + (size_t)o * ld;
        const double *src = A.val + (size_t)j * ld;
        if (off || d == Magma_VALUE || (!lower && d != Magma_UNITY && d != Magma_ZERO && d != Magma_NODIAG)) {
          memcpy(dst, src, 8 * (size_t)ld);
        } else if (d == Magma_UNITY) {
          if (bs > 0)
            for (int q = 0; q < bs; ++q) dst[q * bs + q] = 1.0;
          else
            dst[0] = 1.0;
        } else if (d == Magma_ZERO) {
          // the zeroed allocation already holds it
        } else {
          continue;  // NODIAG, or a lower split's diagonal by default
        }
        B->col[o++] = col;
      }
    }
  });
  return DEV_SUCCESS;
}

// the transpose of z_transpose_csr / z_transpose_bcsr
// (control/magma_zmtranspose.cpp:85-185, 237-343), `ld` values per entry;
// L + 1 pointers (L = the row count, or the column count where larger)
void transpose_core(const data_d_matrix &A, data_d_matrix *B, int nidx, int ld, int L, int base) {
  const int R = row_limit(A);
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::max<size_t>(
      1, std::min<size_t>({(size_t)16, hw, (size_t)R / kGrain, ((size_t)64 << 20) / (4 * ((size_t)L + 1))}));
  const size_t per = ((size_t)R + nt - 1) / nt;
  const size_t cols = (size_t)L + 1;
  // per-thread column counts of the entries in its rows (zeroed by the
  // thread that uses them), and of the entries before the first row or
  // after the last (LACE counts every entry)
  std::vector<std::vector<int>> hist(nt);
  par_for(nt, 1, [&](size_t t0, size_t t1) {
    for (size_t t = t0; t < t1; ++t) {
      std::vector<int> &h = hist[t];
      h.assign(cols, 0);
      const size_t r0 = std::min((size_t)R, t * per), r1 = std::min((size_t)R, r0 + per);
      if (r0 >= r1) continue;
      for (int k = A.row[r0] - base; k < A.row[r1] - base; ++k) ++h[A.col[k] - base];
    }
  });
  std::vector<int> tail(cols, 0);
  const int k_lo = std::max(0, A.row[0] - base), k_hi = R > 0 ? std::min(nidx, A.row[R] - base) : 0;
  for (int k = 0; k < std::min(k_lo, nidx); ++k) ++tail[A.col[k] - base];
  for (int k = std::max(k_hi, 0); k < nidx; ++k) ++tail[A.col[k] - base];
  // P[j] = entries with a column below j; hist[t][j] becomes where thread
  // t's entries of column j go
  std::vector<int> count(cols), P(cols + 1, 0), rowcount(cols);
  par_for(cols, 1 << 16, [&](size_t b, size_t e) {
    for (size_t j = b; j < e; ++j) {
      int c = tail[j];
      for (size_t t = 0; t < nt; ++t) c += hist[t][j];
      count[j] = c;
    }
  });
  for (size_t j = 0; j < cols; ++j) P[j + 1] = P[j] + count[j];
  par_for(cols, 1 << 16, [&](size_t b, size_t e) {
    for (size_t j = b; j < e; ++j) {
      int o = P[j];
      for (size_t t = 0; t < nt; ++t) {
        const int c = hist[t][j];
        hist[t][j] = o;
        o += c;
      }
      rowcount[j] = o - P[j];
    }
  });
  par_for(nt, 1, [&](size_t t0, size_t t1) {
    for (size_t t = t0; t < t1; ++t) {
      const size_t r0 = std::min((size_t)R, t * per), r1 = std::min((size_t)R, r0 + per);
      std::vector<int> &pos = hist[t];
      for (size_t i = r0; i < r1; ++i)
        for (int k = A.row[i] - base; k < A.row[i + 1] - base; ++k) {
          const int o = pos[A.col[k] - base]++;
          B->col[o] = (int)i + base;
          memcpy(B->val + (size_t)o * ld, A.val + (size_t)k * ld, 8 * (size_t)ld);
        }
    }
  });
  // LACE's pointers after its scatter and shift: row[j] = where column j-1's
  // scatter ended; the last pointer is the count below it.  One-based input:
  // every pointer and every index slot one higher, the unfilled ones too
  B->row[0] = base;
  par_for((size_t)L, 1 << 16, [&](size_t b, size_t e) {
    for (size_t j = std::max<size_t>(b, 1); j < e; ++j) B->row[j] = P[j - 1] + rowcount[j - 1] + base;
  });
  B->row[L] = P[L] + base;
  if (base) {
    par_for((size_t)nidx, 1 << 18, [&](size_t b, size_t e) {
      for (size_t k = b; k < e; ++k)
        if (B->col[k] == 0) B->col[k] = 1;
    });
  }
}

int transpose_sparse(const data_d_matrix &A, data_d_matrix *B, bool blocks) {
  const int R = row_limit(A);
  const int nidx = blocks ? A.numblocks : A.nnz;
  const int ld = blocks ? A.ldblock : 1;
  const int base = (A.row && A.row[0] == 1) ? 1 : 0;
  // the pointer count: LACE's R + 1, or more where a column index needs it
  std::vector<int> tmax(16, 0);
  par_for((size_t)std::max(nidx, 0), 1 << 18, [&](size_t b, size_t e) {
    int m = 0;
    for (size_t k = b; k < e; ++k) m = std::max(m, A.col[k] - base + 1);
    tmax[b * 16 / std::max<size_t>(1, (size_t)nidx)] = m;
  });
  int L = R;
  for (int m : tmax) L = std::max(L, m);
  B->nnz = A.nnz;
  B->true_nnz = A.true_nnz;
  B->fill_mode = A.fill_mode;
  B->num_rows = A.num_cols;
  B->num_cols = A.num_rows;
  B->pad_rows = A.pad_cols;
  B->pad_cols = A.pad_rows;
  if (blocks) {
    B->diameter = A.diameter;
    B->blocksize = A.blocksize;
    B->ldblock = A.ldblock;
    B->numblocks = A.numblocks;
  }
  B->row = calloc64<int>((size_t)L + 1);
  B->col = calloc64<int>((size_t)std::max(A.nnz, nidx));
  B->val = calloc64<double>((size_t)std::max(A.nnz, nidx * ld));
  if (!B->row || !B->col || !B->val) return DEV_ERR_HOST_ALLOC;
  B->storage_type = A.storage_type;
  transpose_core(A, B, nidx, ld, L, base);
  return DEV_SUCCESS;
}

// z_transpose_dense (control/magma_zmtranspose.cpp:410-455)
int transpose_dense(const data_d_matrix &A, data_d_matrix *B) {
  B->storage_type = A.storage_type;
  B->fill_mode = A.fill_mode;
  B->num_rows = A.num_cols;
  B->num_cols = A.num_rows;
  B->nnz = A.nnz;
  B->true_nnz = A.true_nnz;
  B->pad_rows = A.pad_cols;
  B->pad_cols = A.pad_rows;
  free(B->val);
  int rl = B->num_rows, cl = B->num_cols;
  if (A.pad_rows > 0 && A.pad_cols > 0) {
    rl = B->pad_rows;
    cl = B->pad_cols;
  }
  B->val = calloc64<double>((size_t)rl * cl);
  if (!B->val) return DEV_ERR_HOST_ALLOC;
  if (A.major == MagmaRowMajor) {
    par_for((size_t)cl, 64, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i)
        for (int j = 0; j < rl; ++j) B->val[i + (size_t)j * cl] = A.val[i * A.ld + j];
    });
    B->major = MagmaRowMajor;
    B->ld = cl;
  } else if (A.major == MagmaColMajor) {
    par_for((size_t)cl, 64, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i)
        for (int j = 0; j < rl; ++j) B->val[i * rl + j] = A.val[i + (size_t)j * A.ld];
    });
    B->major = MagmaColMajor;
    B->ld = rl;
  }
  return DEV_SUCCESS;
}

// CSR -> BCSR with block size B->blocksize: block columns ascending in each
// block row, each block row-major (LACE's zero-based mkl_dcsrbsr call,
// :640-668)
int to_bcsr(const data_d_matrix &A, data_d_matrix *B) {
  const int bs = B->blocksize, n = A.num_rows;
  const int nbr = (n + bs - 1) / bs;
  int nbc = 0;
  for (int k = 0; k < A.row[n]; ++k) nbc = std::max(nbc, A.col[k] / bs + 1);
  std::vector<int> cnt((size_t)nbr, 0);
  auto block_columns = [&](int I, std::vector<int> &mark, std::vector<int> &cols) {
    cols.clear();
    for (int r = I * bs; r < std::min(n, (I + 1) * bs); ++r)
      for (int p = A.row[r]; p < A.row[r + 1]; ++p) {
        const int J = A.col[p] / bs;
        if (mark[J] != I) {
          mark[J] = I;
          cols.push_back(J);
        }
      }
    std::sort(cols.begin(), cols.end());
  };
  par_for((size_t)nbr, 1 << 10, [&](size_t b, size_t e) {
    std::vector<int> mark((size_t)nbc + 1, -1), cols;
    for (size_t I = b; I < e; ++I) {
      block_columns((int)I, mark, cols);
      cnt[I] = (int)cols.size();
    }
  });
  long long nb = 0;
  for (int I = 0; I < nbr; ++I) nb += cnt[I];
  const int ld = bs * bs;
  B->storage_type = Magma_BCSR;
  B->true_nnz = A.nnz;
  B->ldblock = ld;
  B->numblocks = (int)nb;
  B->num_rows = nbr;
  B->num_cols = (A.num_cols + bs - 1) / bs;
  B->nnz = (int)nb * ld;
  B->val = calloc64<double>((size_t)nb * ld);
  B->row = calloc64<int>((size_t)nbr + 1);
  B->col = calloc64<int>((size_t)nb);
  if (!B->val || !B->row || !B->col) return DEV_ERR_HOST_ALLOC;
  prefix(cnt, B->row, (size_t)nbr);
  par_for((size_t)nbr, 1 << 10, [&](size_t b, size_t e) {
    std::vector<int> mark((size_t)nbc + 1, -1), slot((size_t)nbc + 1, 0), cols;
    for (size_t I = b; I < e; ++I) {
      block_columns((int)I, mark, cols);
      const int o = B->row[I];
      for (size_t q = 0; q < cols.size(); ++q) {
        B->col[o + q] = cols[q];
        slot[cols[q]] = o + (int)q;
      }
      for (int r = (int)I * bs; r < std::min(n, ((int)I + 1) * bs); ++r)
        for (int p = A.row[r]; p < A.row[r + 1]; ++p) {
          const int c = A.col[p], J = c / bs;
          B->val[(size_t)slot[J] * ld + (size_t)(r - (int)I * bs) * bs + (c - J * bs)] = A.val[p];
        }
    }
  });
  return DEV_SUCCESS;
}

// COO -> CSR (:853-926): entries scattered to their rows in input order,
// then each row sorted by column with std::sort on (column, value) pairs
// (LACE's compare_first, the same call); storage_type and fill_mode are left
// as they were, as LACE leaves them
int coo_to_csr(const data_d_matrix &A, data_d_matrix *B) {
  const int R = row_limit(A);
  const int nz = std::max(A.nnz, 0);
  B->nnz = A.nnz;
  B->true_nnz = A.true_nnz;
  B->num_rows = A.num_rows;
  B->num_cols = A.num_cols;
  B->pad_rows = A.pad_rows;
  B->pad_cols = A.pad_cols;
  B->major = MagmaRowMajor;
  B->val = calloc64<double>((size_t)nz);
  B->row = calloc64<int>((size_t)R + 1);
  B->col = calloc64<int>((size_t)nz);
  if (!B->val || !B->row || !B->col) return DEV_ERR_HOST_ALLOC;
  std::vector<int> cnt((size_t)R, 0);
  for (int k = 0; k < nz; ++k) ++cnt[A.row[k]];
  prefix(cnt, B->row, (size_t)R);
  B->row[R] = A.nnz;
  std::vector<int> next(B->row, B->row + R);
  for (int k = 0; k < nz; ++k) {
    const int o = next[A.row[k]]++;
    B->col[o] = A.col[k];
    B->val[o] = A.val[k];
  }
  par_for((size_t)R, 1 << 12, [&](size_t b, size_t e) {
    std::vector<std::pair<int, double>> rv;
    for (size_t i = b; i < e; ++i) {
      const int k0 = B->row[i], len = B->row[i + 1] - k0;
      if (len < 2) continue;
      rv.resize((size_t)len);
      for (int q = 0; q < len; ++q) rv[q] = std::make_pair(B->col[k0 + q], B->val[k0 + q]);
      std::sort(rv.begin(), rv.end(),
                [](const std::pair<int, double> &x, const std::pair<int, double> &y) { return x.first < y.first; });
      for (int q = 0; q < len; ++q) {
        B->col[k0 + q] = rv[q].first;
        B->val[k0 + q] = rv[q].second;
      }
    }
  });
  return DEV_SUCCESS;
}

bool csr_family(data_storage_t s) {
  return s == Magma_CSR || s == Magma_CSRD || s == Magma_CSRL || s == Magma_CSRU || s == Magma_CSRCOO ||
         s == Magma_CSCD || s == Magma_CSCL || s == Magma_CSCU || s == Magma_CSCCOO;
}
bool bcsr_family(data_storage_t s) {
  return s == Magma_BCSR || s == Magma_BCSRD || s == Magma_BCSRL || s == Magma_BCSRU || s == Magma_BCSC ||
         s == Magma_BCSCD || s == Magma_BCSCL || s == Magma_BCSCU;
}

}  // namespace

extern "C" int data_rowindex(data_d_matrix *A, int **rowidx) {
  if (!A || !rowidx) return DEV_ERR_INVALID_PTR;
  free(*rowidx);
  *rowidx = calloc64<int>((size_t)std::max(A->nnz, 0));
  if (!*rowidx) return DEV_ERR_HOST_ALLOC;
  fill_rowidx(*A, row_limit(*A), *rowidx);
  return DEV_SUCCESS;
}

extern "C" int data_zmtranspose(data_d_matrix A, data_d_matrix *B) {
  if (!B) return DEV_ERR_INVALID_PTR;
  if (csr_family(A.storage_type)) return transpose_sparse(A, B, false);
  if (bcsr_family(A.storage_type)) return transpose_sparse(A, B, true);
  if (A.storage_type == Magma_DENSE || A.storage_type == Magma_DENSEL || A.storage_type == Magma_DENSEU)
    return transpose_dense(A, B);
  return DEV_SUCCESS;  // LACE does nothing for other storages
}

extern "C" int data_zmconvert(data_d_matrix A, data_d_matrix *B, data_storage_t old_format,
                              data_storage_t new_format) {
  if (!B) return DEV_ERR_INVALID_PTR;
  const bool from_csr = old_format == Magma_CSR || old_format == Magma_CSRL || old_format == Magma_CSRU;
  const bool csr_target = new_format == Magma_CSR || new_format == Magma_CUCSR || new_format == Magma_CSRL ||
                          new_format == Magma_CSRU || new_format == Magma_COO || new_format == Magma_CSRCOO ||
                          new_format == Magma_CSC || new_format == Magma_CSCL || new_format == Magma_CSCU ||
                          new_format == Magma_CSCCOO || new_format == Magma_BCSR;
  const bool from_bcsr = old_format == Magma_BCSR && (new_format == Magma_BCSRL || new_format == Magma_BCSRU ||
                                                      new_format == Magma_BCSCU);
  const bool from_coo = old_format == Magma_COO && new_format == Magma_CSR;
  if (!(from_csr && csr_target) && !from_bcsr && !from_coo) return DEV_ERR_NOT_SUPPORTED;
  if (from_coo) {
    // an entry outside the rows: an error, not LACE's write out of bounds
    const int Rc = row_limit(A);
    for (int k = 0; k < A.nnz; ++k)
      if (A.row[k] < 0 || A.row[k] >= Rc) return DEV_ERR_ILLEGAL_VALUE;
    release(B);
    return coo_to_csr(A, B);
  }
  if (from_csr && new_format == Magma_BCSR && B->blocksize <= 0) return DEV_ERR_NOT_SUPPORTED;
  release(B);
  const int R = row_limit(A);
  int rc = DEV_SUCCESS;
  if (from_bcsr) {
    if (new_format == Magma_BCSCU) {
      data_d_matrix Cm;
      memset(&Cm, 0, sizeof Cm);
      Cm.storage_type = Magma_BCSR;
      rc = split(A, &Cm, false, A.blocksize);
      if (!rc) rc = data_zmtranspose(Cm, B);
      release(&Cm);
      B->storage_type = Magma_BCSCU;
      B->major = MagmaColMajor;
      return rc;
    }
    return split(A, B, new_format == Magma_BCSRL, A.blocksize);
  }
  switch (new_format) {
    case Magma_CSR:
      return copy_csr(A, B);
    case Magma_CUCSR:
      rc = copy_csr(A, B);
      B->storage_type = Magma_CUCSR;
      return rc;
    case Magma_CSRL:
    case Magma_CSRU:
      return split(A, B, new_format == Magma_CSRL, 0);
    case Magma_COO:
    case Magma_CSRCOO: {
      rc = copy_csr(A, B);
      if (rc) return rc;
      B->storage_type = new_format;
      B->major = MagmaRowMajor;
      int *idx = calloc64<int>((size_t)std::max(new_format == Magma_COO ? A.nnz : B->nnz, 0));
      if (!idx) return DEV_ERR_HOST_ALLOC;
      fill_rowidx(A, R, idx);
      if (new_format == Magma_COO) {
        free(B->row);
        B->row = idx;
      } else {
        B->rowidx = idx;
      }
      return DEV_SUCCESS;
    }
    case Magma_CSC:
      rc = data_zmtranspose(A, B);
      B->storage_type = Magma_CSC;
      B->major = MagmaColMajor;
      return rc;
    case Magma_CSCL:
    case Magma_CSCU: {
      data_d_matrix Cm;
      memset(&Cm, 0, sizeof Cm);
      Cm.storage_type = new_format == Magma_CSCL ? Magma_CSR : Magma_CSRU;
      rc = split(A, &Cm, new_format == Magma_CSCL, 0);
      if (!rc) rc = data_zmtranspose(Cm, B);
      release(&Cm);
      B->storage_type = new_format;
      B->major = MagmaColMajor;
      return rc;
    }
    case Magma_CSCCOO: {
      // the CSR copy's row indices stay; the arrays are then the transpose's
      rc = copy_csr(A, B);
      if (rc) return rc;
      int *idx = calloc64<int>((size_t)std::max(B->nnz, 0));
      if (!idx) return DEV_ERR_HOST_ALLOC;
      fill_rowidx(A, R, idx);
      free(B->val);
      free(B->row);
      free(B->col);
      B->val = nullptr;
      B->row = B->col = nullptr;
      B->rowidx = idx;
      rc = data_zmtranspose(A, B);
      B->storage_type = Magma_CSCCOO;
      B->major = MagmaColMajor;
      return rc;
    }
    case Magma_BCSR:
      return to_bcsr(A, B);
    default:
      return DEV_ERR_NOT_SUPPORTED;
  }
}
