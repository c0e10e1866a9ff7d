// Cuthill-McKee orderings and LACE's reorder dispatch, on the host:
// data_reorder_cuthill_mckee (src/cuthill_mckee.cpp:53) and
// data_sparse_reorder (src/reorder.cpp:167).
//
// The ordering is LACE's as its source states it: the seed is a node of
// maximum degree (degree = off-diagonal entries of its row, :98-113 and
// :128-139), nodes are numbered breadth first, and each node's unnumbered
// neighbours are numbered in order of decreasing degree (compare_degree,
// :31-41); nn_map[old] = new (:224-225).  Where LACE's routine is undefined
// this one is defined: ties in degree go to the lower node index (LACE's
// qsort leaves them unspecified), a new component starts at the next node of
// maximum degree (LACE reads past its queue there), each node's own
// neighbour list is used (LACE's list is shifted by one slot), and the
// reversed numbering is new' = n - 1 - new (LACE swaps array positions).
//
// data_sparse_reorder permutes A in place as LACE's reorder_csr_indices does
// (src/reorder.cpp:86-122: row i of the result is row P[i] of A, column c
// becomes Pinv[c], rows then sorted by column), with P = the new-to-old map
// of the Cuthill-McKee numbering and Pinv its inverse, so that the result is
// A in that numbering (LACE passes the old-to-new map as P and so applies
// the inverse permutation).  The AMD mode needs SuiteSparse, which LACE's
// tree does not carry: DEV_ERR_NOT_SUPPORTED.  Nothing is printed (LACE
// prints character plots of A, on the stack, n x n).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/lace_gb300.h"
#include "context.h"
#include "hostpar.h"

namespace {

using lace::par_for;

// row graph checks: pointers non-decreasing from 0, columns inside [0, n)
int check_graph(int n, const int *row, const int *col) {
  if (n < 0) return DEV_ERR_ILLEGAL_VALUE;
  if (n == 0) return 0;
  if (!row || row[0] != 0) return DEV_ERR_ILLEGAL_VALUE;
  for (int i = 0; i < n; ++i)
    if (row[i + 1] < row[i]) return DEV_ERR_ILLEGAL_VALUE;
  if (row[n] > 0 && !col) return DEV_ERR_INVALID_PTR;
  for (int p = 0; p < row[n]; ++p)
    if (col[p] < 0 || col[p] >= n) return DEV_ERR_ILLEGAL_VALUE;
  return 0;
}

// nn_map[old] = new, the Cuthill-McKee numbering (reversed when asked)
void cuthill_mckee(int n, const int *row, const int *col, bool reverse, int *nn_map) {
  std::vector<int> deg(n);
  par_for((size_t)n, 65536, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      int d = 0;
      for (int p = row[i]; p < row[i + 1]; ++p) d += col[p] != (int)i;
      deg[i] = d;
    }
  });
  // decreasing degree, lower index first among equals
  auto before = [&](int a, int b) { return deg[a] != deg[b] ? deg[a] > deg[b] : a < b; };
  std::vector<int> seeds(n);
  std::iota(seeds.begin(), seeds.end(), 0);
  std::sort(seeds.begin(), seeds.end(), before);
  std::vector<char> seen(n, 0);
  std::vector<int> order;
  order.reserve(n);
  std::vector<int> nb;
  size_t head = 0, next_seed = 0;
  while ((int)order.size() < n) {
    if (head == order.size()) {  // the queue is empty: the next component
      while (seen[seeds[next_seed]]) ++next_seed;
      const int s = seeds[next_seed];
      seen[s] = 1;
      order.push_back(s);
    }
    const int v = order[head++];
    nb.clear();
    for (int p = row[v]; p < row[v + 1]; ++p) {
      const int u = col[p];
      if (u != v && !seen[u]) {
        seen[u] = 1;
        nb.push_back(u);
      }
    }
    std::sort(nb.begin(), nb.end(), before);
    order.insert(order.end(), nb.begin(), nb.end());
  }
  for (int k = 0; k < n; ++k) nn_map[order[k]] = reverse ? n - 1 - k : k;
}

template <typename T>
T *alloc64(size_t count) {
  // LACE_CALLOC's allocation (posix_memalign(64)), so free() releases it
  void *p = nullptr;
  const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
  if (posix_memalign(&p, 64, (bytes / 64 + 1) * 64) != 0) return nullptr;
  return (T *)p;
}

// A <- A permuted: row i is row P[i] of A with columns c -> Pinv[c], sorted
// by column (ld values per entry: 1 for CSR, blocksize^2 for BCSR)
int permute_in_place(data_d_matrix *A, const int *P, const int *Pinv, int ld) {
  const int n = A->num_rows;
  const int *row = A->row, *col = A->col;
  const double *val = A->val;
  const int nz = row[n];
  int *r2 = alloc64<int>((size_t)n + 1), *c2 = alloc64<int>((size_t)nz);
  double *v2 = alloc64<double>((size_t)nz * ld);
  if (!r2 || !c2 || !v2) {
    free(r2);
    free(c2);
    free(v2);
    return DEV_ERR_HOST_ALLOC;
  }
  r2[0] = 0;
  for (int i = 0; i < n; ++i) r2[i + 1] = r2[i] + (row[P[i] + 1] - row[P[i]]);
  par_for((size_t)n, 4096, [&](size_t b, size_t e) {
    std::vector<std::pair<int, int>> ent;  // (new column, old position)
    for (size_t i = b; i < e; ++i) {
      const int o = P[i];
      ent.clear();
      for (int p = row[o]; p < row[o + 1]; ++p) ent.emplace_back(Pinv[col[p]], p);
      std::stable_sort(ent.begin(), ent.end(),
                       [](const std::pair<int, int> &x, const std::pair<int, int> &y) { return x.first < y.first; });
      int q = r2[i];
      for (const auto &e2 : ent) {
        c2[q] = e2.first;
        memcpy(v2 + (size_t)q * ld, val + (size_t)e2.second * ld, sizeof(double) * ld);
        ++q;
      }
    }
  });
  free(A->row);
  free(A->col);
  free(A->val);
  A->row = r2;
  A->col = c2;
  A->val = v2;
  return 0;
}

}  // namespace

extern "C" void data_reorder_cuthill_mckee(data_d_matrix *A, int *nn_map, bool reverse) {
  if (!A || !nn_map) {
    lace::set_err(DEV_ERR_INVALID_PTR);
    return;
  }
  const int rc = check_graph(A->num_rows, A->row, A->col);
  if (rc) {
    lace::set_err(rc);
    return;
  }
  cuthill_mckee(A->num_rows, A->row, A->col, reverse, nn_map);
  lace::set_err(0);
}

extern "C" int data_sparse_reorder(data_d_matrix *A, int *P, int *Pinv, int reorder) {
  if (!A || !P || !Pinv) return lace::set_err(DEV_ERR_INVALID_PTR);
  const bool bcsr = A->storage_type == Magma_BCSR;
  if (!bcsr && A->storage_type != Magma_CSR) return lace::set_err(DEV_ERR_NOT_SUPPORTED);
  if (reorder == 3) return lace::set_err(DEV_ERR_NOT_SUPPORTED);  // AMD: SuiteSparse
  const int n = A->num_rows;
  int rc = check_graph(n, A->row, A->col);
  if (rc) return lace::set_err(rc);
  if (n > 0 && A->row[n] > 0 && !A->val) return lace::set_err(DEV_ERR_INVALID_PTR);
  if (reorder == 1 || reorder == 2) {
    cuthill_mckee(n, A->row, A->col, reorder == 2, Pinv);
    for (int k = 0; k < n; ++k) P[Pinv[k]] = k;
  } else {
    for (int k = 0; k < n; ++k) P[k] = Pinv[k] = k;
  }
  if (n == 0) return lace::set_err(0);
  const int ld = bcsr ? A->blocksize * A->blocksize : 1;
  if (ld < 1) return lace::set_err(DEV_ERR_ILLEGAL_VALUE);
  rc = permute_in_place(A, P, Pinv, ld);
  return lace::set_err(rc);
}
