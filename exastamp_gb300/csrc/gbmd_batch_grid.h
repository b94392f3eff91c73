// gbmd_batch_grid.h -- the cell grid of one batched replica, shared by the
// batch kernel (gbmd_batch.cu) and its host-side argument checks.  Plain
// C++ with host/device decorations under nvcc, so a CPU test can compile it
// with g++ alone.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GBMD_HD __host__ __device__
#else
#define GBMD_HD
#endif

namespace gbmd {

// Cells per edge of a periodic replica box with edges L[3]: cells of at
// least rcut / S (S = stencil radius in cells), at least S per edge, and at
// most maxc cells in all.  Each edge count is clamped to maxc before the
// double-to-int conversion, so a huge (or infinite) edge cannot saturate the
// int or overflow the product; products beyond 8 * maxc are first halved
// along the longest edge, so the final one-cell-at-a-time coarsening runs at
// most a few thousand iterations.  Coarser cells still cover rcut.  Returns
// the cell count.
GBMD_HD inline int batch_grid_dims(const double L[3], double rcut, int S, int maxc, int nc[3]) {
  const double cell_min = rcut / S * (1.0 + 0x1p-40);
  for (int d = 0; d < 3; ++d) {
    const double qd = fmin(floor(L[d] / cell_min), (double)maxc);
    const int q = qd >= 1.0 ? (int)qd : 1;
    nc[d] = q < S ? S : q;
  }
  auto longest = [&]() {
    int dm = 0;
    for (int d = 1; d < 3; ++d)
      if (nc[d] > nc[dm]) dm = d;
    return dm;
  };
  while ((int64_t)nc[0] * nc[1] * nc[2] > 8 * (int64_t)maxc) {
    const int dm = longest();
    const int h = (nc[dm] + 1) / 2;
    nc[dm] = h < S ? S : h;
  }
  while ((int64_t)nc[0] * nc[1] * nc[2] > maxc) {
    const int dm = longest();
    if (nc[dm] <= S) break;  // maxc >= S^3 always holds for the kernels' limits
    nc[dm] -= 1;
  }
  return nc[0] * nc[1] * nc[2];
}

// Host check of one replica box [lo, hi): finite, non-empty edges.
inline bool batch_box_ok(const double lo[3], const double hi[3]) {
  for (int d = 0; d < 3; ++d)
    if (!std::isfinite(lo[d]) || !std::isfinite(hi[d]) || !(hi[d] > lo[d])) return false;
  return true;
}

}  // namespace gbmd
