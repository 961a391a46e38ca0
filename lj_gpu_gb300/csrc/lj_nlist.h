// lj_nlist.h -- cell grid and launchers of the on-device neighbour build.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "lj_internal.h"

namespace ljg {

struct CellGrid {
  int nc[3];
  int ncells;
  int periodic;
  double lo[3];     // grid origin
  double inv_w[3];  // cells per unit length
};

struct BuildArgs {
  const double* q;  // AoS double4, device
  int n;
  CellGrid grid;
  double search;
  double box[3];
  double unit[3];   // length per fixed unit
  int aniso;
  const int64_t* start;
  const int32_t* order;
  const int4* cq;
  const int32_t* cell;
  int want_half, want_full;
  // 0: membership exactly r2 < search^2 in FP64 (the reference's list);
  // 1: a superset that may add pairs within the FP32 band outside the
  //    sphere (Verlet lists whose users apply the cutoff themselves)
  int superset;
  // launch_build_rows_split: candidates closer than this go to the near rows
  double near;
};

double key_to_double(unsigned long long k);
cudaError_t launch_minmax(const double* q, int n, unsigned long long* out6, cudaStream_t s);
// `guard` (optional): the kernels do nothing while *guard == 0.
cudaError_t launch_bin(const double* q, int n, const CellGrid& g, int32_t* cell, int32_t* count,
                       cudaStream_t s, const int32_t* guard = nullptr);
cudaError_t launch_place(const int32_t* cell, int n, const int64_t* start, int32_t* cursor,
                         int ncells, const int4* qfix, int32_t* order, int4* cq, cudaStream_t s,
                         const int32_t* guard = nullptr);

// Sorts the slots of every cell by particle index (out of place).
cudaError_t launch_sort_cells(const int64_t* start, int ncells, const int32_t* order,
                              const int4* cq, int32_t* order2, int4* cq2, cudaStream_t s,
                              const int32_t* guard = nullptr);
// Warp-cooperative build into padded rows (row i at i * maxrow, cnt[i]
// entries; half: j > i only).  Rows longer than maxrow set *overflow.
cudaError_t launch_build_rows(const BuildArgs& a, bool half, int maxrow, int32_t* rows,
                              int32_t* cnt, int32_t* overflow, cudaStream_t s,
                              const int32_t* guard = nullptr);
// Full superset rows in two parts: candidates with FP32 r2 below near^2
// (BuildArgs::near) into rows / cnt (row i at i * maxrow), the others into
// rows2 / cnt2 (i * maxrow2), each in walk order.
cudaError_t launch_build_rows_split(const BuildArgs& a, int maxrow, int32_t* rows, int32_t* cnt,
                                    int maxrow2, int32_t* rows2, int32_t* cnt2,
                                    int32_t* overflow, cudaStream_t s,
                                    const int32_t* guard = nullptr);
// Local-index rows for the cell-tiled gather (full rows, slot-indexed).
cudaError_t launch_build_rows_local(const BuildArgs& a, int maxrow, int maxc_shift,
                                    uint16_t* rows, int32_t* cnt, int32_t* overflow,
                                    cudaStream_t s);
cudaError_t launch_compact_padded(const int32_t* cnt, const int32_t* rows, int maxrow,
                                  const int64_t* off, int n, int32_t* out, cudaStream_t s,
                                  const int32_t* guard = nullptr);

// Batch (one grid per replica, cells numbered from each replica's cell_base).
cudaError_t launch_bin_batch(const double* q, int n, const int32_t* rid, const ReplicaInfo* reps,
                             int ncells, int32_t* cell, int32_t* count, cudaStream_t s,
                             const int32_t* guard = nullptr);
// rows2 / cnt2 (optional, each part maxrow wide): rows in a near part (r2 at
// the build below each replica's near2u, into rows / cnt) and a far part.
cudaError_t launch_build_rows_batch(const double* q, const ReplicaInfo* reps,
                                    const int32_t* cell_rid, int ncells, double sl2,
                                    const int64_t* start, const int32_t* order, const int4* cq,
                                    int maxrow, int32_t* rows, int32_t* cnt, int32_t* rows2,
                                    int32_t* cnt2, int32_t* overflow, cudaStream_t s,
                                    const int32_t* guard = nullptr);

}  // namespace ljg
