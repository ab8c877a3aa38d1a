// Host construction of the assembled-Hessian sparsity pattern of a tet mesh
// and of the index maps that make assembly a deterministic gather.
//
// simkit assembles K = J^T blockdiag(He) J with scipy (stable_neo_hookean.py:536-537);
// the nonzeros of K are the 3x3 blocks (v, w) of every pair of vertices that
// share a tet.  Here that pattern is built directly from the connectivity:
// block rows are vertices, block columns are sorted ascending, so the scalar
// expansion (row 3v+i, column 3w+j) is scipy's canonical CSR pattern.
//
// For each block slot the list of per-tet blocks summed into it is stored in
// tet order (hc_src = tet*16 + code), so that the device gather sums in a
// fixed order and the assembled values are bitwise reproducible.
//   code 0..3   diagonal block (a,a) of the tet
//   code 4..9   off-diagonal block (a,b), a < b, index offdiag_index(a,b)
//   code 10..15 the transpose of block (b,a) for a > b
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "../../include/simkit_gb300.h"

namespace skg {
int fail(int status, const char* fmt, ...);
}

static int offdiag_index_h(int a, int b) { return a == 0 ? (b - 1) : (a == 1 ? (b + 1) : 5); }

extern "C" int skg_pattern_build(const int32_t* T, int64_t n, int64_t t, int64_t* n_blocks, int32_t* rowptr,
                                 int32_t* col, int32_t* diag, int32_t* hc_ptr, int32_t* hc_src, int32_t* v2t_ptr,
                                 int32_t* v2t) {
  if (!T || !n_blocks || n <= 0 || t < 0) return skg::fail(SKG_ERR_ARG, "pattern: bad arguments");
  if (16 * t > INT32_MAX || n > INT32_MAX / 2) return skg::fail(SKG_ERR_CAPACITY, "pattern: mesh too large for int32 maps");
  for (int64_t e = 0; e < t; ++e) {
    for (int a = 0; a < 4; ++a) {
      const int32_t v = T[4 * e + a];
      if (v < 0 || v >= n) return skg::fail(SKG_ERR_ARG, "pattern: tet %lld has vertex %d out of range", (long long)e, v);
      for (int b = 0; b < a; ++b)
        if (T[4 * e + b] == v) return skg::fail(SKG_ERR_ARG, "pattern: tet %lld repeats vertex %d", (long long)e, v);
    }
  }
  // vertex -> incident (tet, corner), in tet order
  std::vector<int32_t> vptr(n + 1, 0);
  for (int64_t k = 0; k < 4 * t; ++k) vptr[T[k] + 1]++;
  for (int64_t v = 0; v < n; ++v) vptr[v + 1] += vptr[v];
  std::vector<int32_t> vinc(4 * t);
  {
    std::vector<int32_t> pos(vptr.begin(), vptr.end() - 1);
    for (int64_t e = 0; e < t; ++e)
      for (int a = 0; a < 4; ++a) vinc[pos[T[4 * e + a]]++] = (int32_t)(4 * e + a);
  }
  // block rows: sorted unique neighbours (including the vertex itself)
  std::vector<int32_t> rp(n + 1, 0);
  std::vector<int32_t> cols;
  cols.reserve(16 * (size_t)n);
  std::vector<int32_t> nb;
  nb.reserve(64);
  for (int64_t v = 0; v < n; ++v) {
    nb.clear();
    nb.push_back((int32_t)v);
    for (int32_t k = vptr[v]; k < vptr[v + 1]; ++k) {
      const int64_t e = vinc[k] >> 2;
      for (int b = 0; b < 4; ++b) nb.push_back(T[4 * e + b]);
    }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    cols.insert(cols.end(), nb.begin(), nb.end());
    rp[v + 1] = (int32_t)cols.size();
  }
  const int64_t nblk = (int64_t)cols.size();
  *n_blocks = nblk;
  if (!rowptr) return SKG_OK;  // size query

  std::copy(rp.begin(), rp.end(), rowptr);
  std::copy(cols.begin(), cols.end(), col);
  auto slot_of = [&](int32_t v, int32_t w) -> int32_t {
    const int32_t* b = cols.data() + rp[v];
    const int32_t* e = cols.data() + rp[v + 1];
    return (int32_t)(std::lower_bound(b, e, w) - cols.data());
  };
  for (int64_t v = 0; v < n; ++v) diag[v] = slot_of((int32_t)v, (int32_t)v);
  // contributions per slot, counted then filled in tet order
  std::vector<int32_t> cnt(nblk + 1, 0);
  std::vector<int32_t> slots(16 * (size_t)t);
  for (int64_t e = 0; e < t; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        const int32_t s = slot_of(T[4 * e + a], T[4 * e + b]);
        slots[16 * e + 4 * a + b] = s;
        cnt[s + 1]++;
      }
  for (int64_t s = 0; s < nblk; ++s) cnt[s + 1] += cnt[s];
  std::copy(cnt.begin(), cnt.end(), hc_ptr);
  std::vector<int32_t> fillpos(cnt.begin(), cnt.end() - 1);
  for (int64_t e = 0; e < t; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        const int code = a == b ? a : (a < b ? 4 + offdiag_index_h(a, b) : 10 + offdiag_index_h(b, a));
        hc_src[fillpos[slots[16 * e + 4 * a + b]]++] = (int32_t)(16 * e + code);
      }
  if (v2t_ptr) std::copy(vptr.begin(), vptr.end(), v2t_ptr);
  if (v2t) std::copy(vinc.begin(), vinc.end(), v2t);
  return SKG_OK;
}
