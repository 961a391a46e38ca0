/*
 * lj_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see lj_oracle.h).
 *
 * Plain C restatement of the reference CPU path.  Every routine cites the
 * reference lines whose arithmetic it follows; the operation order inside the
 * force loops is the reference's, and the library is compiled with the flags
 * of cpu_ref/Makefile (-O3 -march=native, GCC's default contraction), which
 * reproduces the reference build bit for bit on x86-64.
 */
#include "lj_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Mersenne twister (Matsumoto & Nishimura 1998), the std::mt19937 and
 * std::mt19937_64 parameter sets.                                           */
/* ------------------------------------------------------------------------ */
void lj_or_mt32_seed(lj_or_mt32* g, uint32_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 624; i++) {
    uint32_t prev = g->mt[i - 1];
    g->mt[i] = 1812433253u * (prev ^ (prev >> 30)) + (uint32_t)i;
  }
  g->idx = 624;
}

static void mt32_twist(lj_or_mt32* g) {
  for (int i = 0; i < 624; i++) {
    uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
    uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
    if (y & 1u) v ^= 0x9908b0dfu;
    g->mt[i] = v;
  }
  g->idx = 0;
}

uint32_t lj_or_mt32_next(lj_or_mt32* g) {
  if (g->idx >= 624) mt32_twist(g);
  uint32_t y = g->mt[g->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

void lj_or_mt64_seed(lj_or_mt64* g, uint64_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 312; i++) {
    uint64_t prev = g->mt[i - 1];
    g->mt[i] = 6364136223846793005ull * (prev ^ (prev >> 62)) + (uint64_t)i;
  }
  g->idx = 312;
}

static void mt64_twist(lj_or_mt64* g) {
  for (int i = 0; i < 312; i++) {
    uint64_t y = (g->mt[i] & 0xFFFFFFFF80000000ull) | (g->mt[(i + 1) % 312] & 0x7FFFFFFFull);
    uint64_t v = g->mt[(i + 156) % 312] ^ (y >> 1);
    if (y & 1ull) v ^= 0xB5026F5AA96619E9ull;
    g->mt[i] = v;
  }
  g->idx = 0;
}

uint64_t lj_or_mt64_next(lj_or_mt64* g) {
  if (g->idx >= 312) mt64_twist(g);
  uint64_t y = g->mt[g->idx++];
  y ^= (y >> 29) & 0x5555555555555555ull;
  y ^= (y << 17) & 0x71D67FFFEDA60000ull;
  y ^= (y << 37) & 0xFFF7EEE000000000ull;
  y ^= y >> 43;
  return y;
}

/* The generators are evaluated without multiply-add contraction so that the
 * jittered coordinates do not depend on the host's FMA support. */
#define LJ_NO_CONTRACT __attribute__((optimize("fp-contract=off")))

/* libstdc++ generate_canonical<double, 53>: ceil(53 / log2(range)) draws,
 * summed with weights range^k in double, divided by range^m, clamped below 1. */
LJ_NO_CONTRACT double lj_or_uniform32(lj_or_mt32* g, double a, double b) {
  double sum = 0.0, scale = 1.0;
  for (int k = 0; k < 2; k++) {
    sum += (double)lj_or_mt32_next(g) * scale;
    scale *= 4294967296.0;
  }
  double c = sum / scale;
  if (c >= 1.0) c = nextafter(1.0, 0.0);
  return c * (b - a) + a;
}

LJ_NO_CONTRACT double lj_or_uniform64(lj_or_mt64* g, double a, double b) {
  double c = (double)lj_or_mt64_next(g) / 18446744073709551616.0;
  if (c >= 1.0) c = nextafter(1.0, 0.0);
  return c * (b - a) + a;
}

/* ------------------------------------------------------------------------ */
/* System set-up                                                             */
/* ------------------------------------------------------------------------ */
/* cpu_ref/force_aos.cpp:142-169 with add_particle :43-51 */
int lj_or_init_reference(double density, double L, double* q4, int cap) {
  lj_or_mt32 g;
  lj_or_mt32_seed(&g, 2u);
  const double s = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  const double hs = s * 0.5;
  const int sx = (int)(L / s), sy = (int)(L / s), sz = (int)(L / s);
  const double site[4][3] = {{0, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
  int n = 0;
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const double x = ix * s, y = iy * s, z = iz * s;
        for (int k = 0; k < 4; k++) {
          if (n >= cap) return -1;
          /* x + hs is evaluated exactly as the reference's add_particle args */
          const double bx = site[k][0] != 0 ? x + hs : x;
          const double by = site[k][1] != 0 ? y + hs : y;
          const double bz = site[k][2] != 0 ? z + hs : z;
          q4[4 * n + 0] = bx + lj_or_uniform32(&g, 0.0, 0.1);
          q4[4 * n + 1] = by + lj_or_uniform32(&g, 0.0, 0.1);
          q4[4 * n + 2] = bz + lj_or_uniform32(&g, 0.0, 0.1);
          q4[4 * n + 3] = 0.0;
          n++;
        }
      }
  return n;
}

LJ_NO_CONTRACT static double wrap_into(double x, double L) {
  if (x >= L) x -= L;
  if (x < 0.0) x += L;
  if (x >= L) x = 0.0; /* -tiny + L rounds up to L */
  return x;
}

LJ_NO_CONTRACT int lj_or_init_fcc_periodic(int ncell, double density, double jitter, uint64_t seed,
                            double* q4, int cap, double* box_len) {
  lj_or_mt64 g;
  lj_or_mt64_seed(&g, seed);
  const double a = pow(4.0 / density, 1.0 / 3.0);
  const double L = ncell * a;
  const double ha = 0.5 * a;
  const double site[4][3] = {{0, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
  int n = 0;
  for (int iz = 0; iz < ncell; iz++)
    for (int iy = 0; iy < ncell; iy++)
      for (int ix = 0; ix < ncell; ix++)
        for (int k = 0; k < 4; k++) {
          if (n >= cap) return -1;
          const double bx = ix * a + site[k][0] * ha;
          const double by = iy * a + site[k][1] * ha;
          const double bz = iz * a + site[k][2] * ha;
          const double jx = lj_or_uniform64(&g, -jitter, jitter);
          const double jy = lj_or_uniform64(&g, -jitter, jitter);
          const double jz = lj_or_uniform64(&g, -jitter, jitter);
          q4[4 * n + 0] = wrap_into(bx + jx, L);
          q4[4 * n + 1] = wrap_into(by + jy, L);
          q4[4 * n + 2] = wrap_into(bz + jz, L);
          q4[4 * n + 3] = 0.0;
          n++;
        }
  if (box_len) *box_len = L;
  return n;
}

/* ------------------------------------------------------------------------ */
/* Neighbour lists                                                           */
/* ------------------------------------------------------------------------ */
static inline double min_image(double d, double L) {
  if (d > 0.5 * L) return d - L;
  if (d < -0.5 * L) return d + L;
  return d;
}

/* makepair's distance (cpu_ref/force_aos.cpp:131-135): dx = q_i - q_j */
static inline double pair_r2(const double* q4, int i, int j, const double* box) {
  double dx = q4[4 * i + 0] - q4[4 * j + 0];
  double dy = q4[4 * i + 1] - q4[4 * j + 1];
  double dz = q4[4 * i + 2] - q4[4 * j + 2];
  if (box) {
    dx = min_image(dx, box[0]);
    dy = min_image(dy, box[1]);
    dz = min_image(dz, box[2]);
  }
  return dx * dx + dy * dy + dz * dz;
}

/* makepair + sortpair (cpu_ref/force_aos.cpp:100-140).  Pairs are registered
 * with i < j in (i, j) loop order, so each CSR row comes out ascending in j;
 * pointer[i] is the exclusive prefix sum of number_of_partners. */
int64_t lj_or_build_half_brute(const double* q4, int n, double sl2, const double* box,
                               int32_t* np, int32_t* ptr, int32_t* list, int64_t cap) {
  int64_t pos = 0;
  for (int i = 0; i < n; i++) {
    ptr[i] = (int32_t)pos;
    int cnt = 0;
    for (int j = i + 1; j < n; j++) {
      if (pair_r2(q4, i, j, box) < sl2) {
        if (pos >= cap) return -1;
        list[pos++] = j;
        cnt++;
      }
    }
    np[i] = cnt;
  }
  return pos;
}

static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* Cell-grid version: same membership test, rows sorted ascending, so the CSR
 * is identical to the brute-force one. */
int64_t lj_or_build_list_cells(const double* q4, int n, double sl2, const double* box,
                               int full, int32_t* np, int32_t* ptr, int32_t* list,
                               int64_t cap) {
  return lj_or_build_rows_cells(q4, n, sl2, box, full, 0, n, np, ptr, list, cap);
}

/* Rows [row0, row1) of the cell-grid list (np and ptr indexed by i - row0,
 * ptr relative to list): the rows lj_or_build_list_cells gives for them. */
int64_t lj_or_build_rows_cells(const double* q4, int n, double sl2, const double* box,
                               int full, int row0, int row1, int32_t* np, int32_t* ptr,
                               int32_t* list, int64_t cap) {
  if (n <= 0 || row0 >= row1) return 0;
  if (row0 < 0 || row1 > n) return -1;
  const double rs = sqrt(sl2);
  double lo[3], ext[3];
  int nc[3];
  for (int d = 0; d < 3; d++) {
    if (box) {
      lo[d] = 0.0;
      ext[d] = box[d];
      nc[d] = (int)floor(box[d] / rs);
    } else {
      double mn = q4[d], mx = q4[d];
      for (int i = 1; i < n; i++) {
        const double v = q4[4 * i + d];
        if (v < mn) mn = v;
        if (v > mx) mx = v;
      }
      lo[d] = mn;
      ext[d] = (mx - mn) + 1e-9 * (1.0 + fabs(mx) + fabs(mn));
      nc[d] = (int)floor(ext[d] / rs);
    }
    if (nc[d] < 1) nc[d] = 1;
    if (nc[d] > 1024) nc[d] = 1024;
  }
  /* periodic grids with fewer than 3 cells per axis would visit a cell twice */
  if (box && (nc[0] < 3 || nc[1] < 3 || nc[2] < 3)) nc[0] = nc[1] = nc[2] = 1;
  const int64_t ncells = (int64_t)nc[0] * nc[1] * nc[2];
  int32_t* head = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ncells + 1));
  int32_t* cell_of = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* row = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  memset(head, 0, sizeof(int32_t) * (size_t)(ncells + 1));
  for (int i = 0; i < n; i++) {
    int c[3];
    for (int d = 0; d < 3; d++) {
      int ci = (int)floor((q4[4 * i + d] - lo[d]) / ext[d] * nc[d]);
      if (ci < 0) ci = box ? ((ci % nc[d]) + nc[d]) % nc[d] : 0;
      if (ci >= nc[d]) ci = box ? ci % nc[d] : nc[d] - 1;
      c[d] = ci;
    }
    cell_of[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
    head[cell_of[i] + 1]++;
  }
  for (int64_t c = 0; c < ncells; c++) head[c + 1] += head[c];
  {
    int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (size_t)ncells);
    memcpy(fill, head, sizeof(int32_t) * (size_t)ncells);
    for (int i = 0; i < n; i++) order[fill[cell_of[i]]++] = i;
    free(fill);
  }
  int64_t pos = 0;
  int overflow = 0;
  for (int i = row0; i < row1 && !overflow; i++) {
    const int ci = cell_of[i];
    const int cx = ci % nc[0], cy = (ci / nc[0]) % nc[1], cz = ci / (nc[0] * nc[1]);
    int cnt = 0;
    const int rx = nc[0] >= 3 ? 1 : (nc[0] == 1 ? 0 : 1);
    const int ry = nc[1] >= 3 ? 1 : (nc[1] == 1 ? 0 : 1);
    const int rz = nc[2] >= 3 ? 1 : (nc[2] == 1 ? 0 : 1);
    for (int dz = -rz; dz <= rz; dz++)
      for (int dy = -ry; dy <= ry; dy++)
        for (int dx = -rx; dx <= rx; dx++) {
          int x = cx + dx, y = cy + dy, z = cz + dz;
          if (box) {
            x = (x + nc[0]) % nc[0];
            y = (y + nc[1]) % nc[1];
            z = (z + nc[2]) % nc[2];
          } else if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) {
            continue;
          }
          const int c = (z * nc[1] + y) * nc[0] + x;
          for (int32_t k = head[c]; k < head[c + 1]; k++) {
            const int j = order[k];
            if (full ? (j == i) : (j <= i)) continue;
            if (pair_r2(q4, i, j, box) < sl2) row[cnt++] = j;
          }
        }
    qsort(row, (size_t)cnt, sizeof(int32_t), cmp_i32);
    if (pos + cnt > cap) {
      overflow = 1;
      break;
    }
    ptr[i - row0] = (int32_t)pos;
    np[i - row0] = cnt;
    memcpy(list + pos, row, sizeof(int32_t) * (size_t)cnt);
    pos += cnt;
  }
  free(head);
  free(cell_of);
  free(order);
  free(row);
  return overflow ? -1 : pos;
}

void lj_or_csr_to_pairs(int n, const int32_t* np, const int32_t* ptr, const int32_t* list,
                        int32_t* ip, int32_t* jp) {
  int64_t k = 0;
  for (int i = 0; i < n; i++)
    for (int m = 0; m < np[i]; m++) {
      ip[k] = i;
      jp[k] = list[ptr[i] + m];
      k++;
    }
}

/* ------------------------------------------------------------------------ */
/* Force routines                                                            */
/* ------------------------------------------------------------------------ */
/* cpu_ref/force_aos.cpp:171-190 */
void lj_or_force_pair_aos(const double* q4, double* p4, int64_t npairs, const int32_t* ip,
                          const int32_t* jp, double cl2, double dt, const double* box) {
  for (int64_t k = 0; k < npairs; k++) {
    const int i = ip[k], j = jp[k];
    double dx = q4[4 * j + 0] - q4[4 * i + 0];
    double dy = q4[4 * j + 1] - q4[4 * i + 1];
    double dz = q4[4 * j + 2] - q4[4 * i + 2];
    if (box) {
      dx = min_image(dx, box[0]);
      dy = min_image(dy, box[1]);
      dz = min_image(dz, box[2]);
    }
    const double r2 = (dx * dx + dy * dy + dz * dz);
    if (r2 > cl2) continue;
    const double r6 = r2 * r2 * r2;
    const double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2)) * dt;
    p4[4 * i + 0] += df * dx;
    p4[4 * i + 1] += df * dy;
    p4[4 * i + 2] += df * dz;
    p4[4 * j + 0] -= df * dx;
    p4[4 * j + 1] -= df * dy;
    p4[4 * j + 2] -= df * dz;
  }
}

/* cpu_ref/force_aos.cpp:192-224 */
void lj_or_force_sorted_aos(const double* q4, double* p4, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box) {
  for (int i = 0; i < n; i++) {
    const double qx = q4[4 * i + 0], qy = q4[4 * i + 1], qz = q4[4 * i + 2];
    const int cnt = np[i];
    const int kp = ptr[i];
    double pfx = 0, pfy = 0, pfz = 0;
    for (int k = 0; k < cnt; k++) {
      const int j = list[kp + k];
      double dx = q4[4 * j + 0] - qx;
      double dy = q4[4 * j + 1] - qy;
      double dz = q4[4 * j + 2] - qz;
      if (box) {
        dx = min_image(dx, box[0]);
        dy = min_image(dy, box[1]);
        dz = min_image(dz, box[2]);
      }
      const double r2 = (dx * dx + dy * dy + dz * dz);
      if (r2 > cl2) continue;
      const double r6 = r2 * r2 * r2;
      const double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2)) * dt;
      pfx += df * dx;
      pfy += df * dy;
      pfz += df * dz;
      p4[4 * j + 0] -= df * dx;
      p4[4 * j + 1] -= df * dy;
      p4[4 * j + 2] -= df * dz;
    }
    p4[4 * i + 0] += pfx;
    p4[4 * i + 1] += pfy;
    p4[4 * i + 2] += pfz;
  }
}

/* cpu_ref/force_soa.cpp:163-195 */
void lj_or_force_sorted_soa(const double* qx, const double* qy, const double* qz,
                            double* px, double* py, double* pz, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box) {
  for (int i = 0; i < n; i++) {
    const double xi = qx[i], yi = qy[i], zi = qz[i];
    const int cnt = np[i];
    const int kp = ptr[i];
    double pfx = 0, pfy = 0, pfz = 0;
    for (int k = 0; k < cnt; k++) {
      const int j = list[kp + k];
      double dx = qx[j] - xi;
      double dy = qy[j] - yi;
      double dz = qz[j] - zi;
      if (box) {
        dx = min_image(dx, box[0]);
        dy = min_image(dy, box[1]);
        dz = min_image(dz, box[2]);
      }
      const double r2 = (dx * dx + dy * dy + dz * dz);
      if (r2 > cl2) continue;
      const double r6 = r2 * r2 * r2;
      const double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2)) * dt;
      pfx += df * dx;
      pfy += df * dy;
      pfz += df * dz;
      px[j] -= df * dx;
      py[j] -= df * dy;
      pz[j] -= df * dz;
    }
    px[i] += pfx;
    py[i] += pfy;
    pz[i] += pfz;
  }
}

int lj_or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Gather over the full list: each row only writes its own p_i, so rows are
 * independent and run in parallel (cuda/kernel.cuh:67-100 semantics). */
void lj_or_force_gather_aos(const double* q4, double* p4, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box, int nthreads) {
  lj_or_force_gather_rows_aos(q4, p4, 0, n, np, ptr, list, cl2, dt, box, nthreads);
}

/* The gather for rows [row0, row1) only (np, ptr indexed by i - row0). */
void lj_or_force_gather_rows_aos(const double* q4, double* p4, int row0, int row1,
                                 const int32_t* np, const int32_t* ptr, const int32_t* list,
                                 double cl2, double dt, const double* box, int nthreads) {
#ifdef _OPENMP
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#else
  (void)nthreads;
#endif
  for (int i = row0; i < row1; i++) {
    const double qx = q4[4 * i + 0], qy = q4[4 * i + 1], qz = q4[4 * i + 2];
    const int cnt = np[i - row0];
    const int kp = ptr[i - row0];
    double pfx = 0, pfy = 0, pfz = 0;
    for (int k = 0; k < cnt; k++) {
      const int j = list[kp + k];
      double dx = q4[4 * j + 0] - qx;
      double dy = q4[4 * j + 1] - qy;
      double dz = q4[4 * j + 2] - qz;
      if (box) {
        dx = min_image(dx, box[0]);
        dy = min_image(dy, box[1]);
        dz = min_image(dz, box[2]);
      }
      const double r2 = (dx * dx + dy * dy + dz * dz);
      if (r2 > cl2) continue;
      const double r6 = r2 * r2 * r2;
      const double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2)) * dt;
      pfx += df * dx;
      pfy += df * dy;
      pfz += df * dz;
    }
    p4[4 * i + 0] += pfx;
    p4[4 * i + 1] += pfy;
    p4[4 * i + 2] += pfz;
  }
}

/* ------------------------------------------------------------------------ */
/* Energies and drift (project extension)                                    */
/* ------------------------------------------------------------------------ */
double lj_or_potential_half(const double* q4, int n, const int32_t* np, const int32_t* ptr,
                            const int32_t* list, double cl2, const double* box) {
  double u = 0.0;
  for (int i = 0; i < n; i++)
    for (int k = 0; k < np[i]; k++) {
      const int j = list[ptr[i] + k];
      double dx = q4[4 * j + 0] - q4[4 * i + 0];
      double dy = q4[4 * j + 1] - q4[4 * i + 1];
      double dz = q4[4 * j + 2] - q4[4 * i + 2];
      if (box) {
        dx = min_image(dx, box[0]);
        dy = min_image(dy, box[1]);
        dz = min_image(dz, box[2]);
      }
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > cl2) continue;
      const double ir6 = 1.0 / (r2 * r2 * r2);
      u += 4.0 * ir6 * (ir6 - 1.0);
    }
  return u;
}

double lj_or_kinetic(const double* p4, int n) {
  double k = 0.0;
  for (int i = 0; i < n; i++)
    k += 0.5 * (p4[4 * i] * p4[4 * i] + p4[4 * i + 1] * p4[4 * i + 1] +
                p4[4 * i + 2] * p4[4 * i + 2]);
  return k;
}

void lj_or_drift(double* q4, const double* p4, int n, double dt, const double* box) {
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      double x = q4[4 * i + d] + p4[4 * i + d] * dt;
      if (box) x = wrap_into(x, box[d]);
      q4[4 * i + d] = x;
    }
}
