// lj_cells.cuh -- cell-grid walks shared by the list builder and the
// cell-tiled force kernel (they must enumerate neighbour cells identically:
// the tiled rows store "k-th neighbour cell, slot in it").
#pragma once

#include "lj_nlist.h"

namespace ljg {

__device__ __forceinline__ int wrap_cell(int c, int nc) {
  c %= nc;
  return c < 0 ? c + nc : c;
}

// Visits the candidate cells of particle i's cell.  Along an axis with fewer
// than 3 cells every cell is visited once; otherwise c-1, c, c+1 (wrapped when
// periodic, clipped when open).
template <typename F>
__device__ __forceinline__ void for_neighbour_cells(int cid, const CellGrid& g, F&& f) {
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  int lo[3], hi[3];
  const int c[3] = {cx, cy, cz};
  for (int d = 0; d < 3; d++) {
    if (g.nc[d] < 3) {
      lo[d] = 0;
      hi[d] = g.nc[d] - 1;
    } else if (g.periodic) {
      lo[d] = c[d] - 1;
      hi[d] = c[d] + 1;
    } else {
      lo[d] = max(c[d] - 1, 0);
      hi[d] = min(c[d] + 1, g.nc[d] - 1);
    }
  }
  for (int z = lo[2]; z <= hi[2]; z++)
    for (int y = lo[1]; y <= hi[1]; y++)
      for (int x = lo[0]; x <= hi[0]; x++) {
        const int wx = g.nc[0] < 3 ? x : wrap_cell(x, g.nc[0]);
        const int wy = g.nc[1] < 3 ? y : wrap_cell(y, g.nc[1]);
        const int wz = g.nc[2] < 3 ? z : wrap_cell(z, g.nc[2]);
        f((wz * g.nc[1] + wy) * g.nc[0] + wx);
      }
}

// The k-th cell for_neighbour_cells visits (same order), or -1 when k is past
// the last; *count receives how many it visits.  Lets a CTA enumerate the
// neighbourhood with one thread per cell.
__device__ __forceinline__ int neighbour_cell_at(int cid, const CellGrid& g, int k, int* count) {
  const int c[3] = {cid % g.nc[0], (cid / g.nc[0]) % g.nc[1], cid / (g.nc[0] * g.nc[1])};
  int lo[3], len[3];
  for (int d = 0; d < 3; d++) {
    int a, b;
    if (g.nc[d] < 3) {
      a = 0;
      b = g.nc[d] - 1;
    } else if (g.periodic) {
      a = c[d] - 1;
      b = c[d] + 1;
    } else {
      a = max(c[d] - 1, 0);
      b = min(c[d] + 1, g.nc[d] - 1);
    }
    lo[d] = a;
    len[d] = b - a + 1;
  }
  *count = len[0] * len[1] * len[2];
  if (k >= *count) return -1;
  const int x = lo[0] + k % len[0], y = lo[1] + (k / len[0]) % len[1],
            z = lo[2] + k / (len[0] * len[1]);
  const int wx = g.nc[0] < 3 ? x : wrap_cell(x, g.nc[0]);
  const int wy = g.nc[1] < 3 ? y : wrap_cell(y, g.nc[1]);
  const int wz = g.nc[2] < 3 ? z : wrap_cell(z, g.nc[2]);
  return (wz * g.nc[1] + wy) * g.nc[0] + wx;
}

}  // namespace ljg
