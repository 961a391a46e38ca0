/*
 * lj_oracle.h -- CPU oracle for the Lennard-Jones neighbour-list force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C, the arithmetic
 * of the reference CPU routines (cpu_ref/force_aos.cpp, cpu_ref/force_soa.cpp)
 * so that the CUDA engine can be checked against it.  Only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py may load it.
 * The engine itself never links or calls anything in this directory.
 *
 * Conventions shared with the reference:
 *   - q, p AoS are double[n][4] (x, y, z, w; w unused), SoA are three double[n].
 *   - the CSR half list holds, for every i, the j > i with r2 < search^2,
 *     rows ascending in j (makepair + sortpair, cpu_ref/force_aos.cpp:100-140).
 *   - the force routine is a kick: p += F * dt with
 *       df = ((24 r^6 - 48) / (r^6 r^6 r^2)) * dt, skipped when r2 > cl2
 *     (cpu_ref/force_aos.cpp:206-218), dx = q_j - q_i.
 *   - box == NULL means open boundaries (the reference has no periodic box);
 *     box != NULL applies a single minimum-image shift per component, which
 *     is exact for coordinates wrapped into [0, L).
 */
#ifndef LJ_ORACLE_H
#define LJ_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- random numbers: std::mt19937 / mt19937_64 + libstdc++ canonical ---- */
typedef struct { uint32_t mt[624]; int idx; } lj_or_mt32;
typedef struct { uint64_t mt[312]; int idx; } lj_or_mt64;
void     lj_or_mt32_seed(lj_or_mt32* g, uint32_t seed);
uint32_t lj_or_mt32_next(lj_or_mt32* g);
void     lj_or_mt64_seed(lj_or_mt64* g, uint64_t seed);
uint64_t lj_or_mt64_next(lj_or_mt64* g);
/* std::uniform_real_distribution<double>(a, b) driven by std::mt19937 */
double   lj_or_uniform32(lj_or_mt32* g, double a, double b);
double   lj_or_uniform64(lj_or_mt64* g, double a, double b);

/* ---- system set-up ---- */
/* cpu_ref init(): FCC cells of side s = (4/density)^(1/3), floor(L/s) cells per
 * axis, 4 sites per cell, each coordinate jittered by U[0, 0.1) from
 * mt19937(2) in call order x, y, z (cpu_ref/force_aos.cpp:43-51,142-169).
 * Returns the particle count, or -1 if it exceeds cap. */
int lj_or_init_reference(double density, double L, double* q4, int cap);
/* Periodic FCC n^3 cells (N = 4 n^3) at the given density, lattice
 * a = (4/density)^(1/3), box L = n a, jitter U[-jitter, jitter) drawn from
 * mt19937_64(seed) in order x, y, z, coordinates wrapped into [0, L). */
int lj_or_init_fcc_periodic(int ncell, double density, double jitter, uint64_t seed,
                            double* q4, int cap, double* box_len);

/* ---- neighbour lists ---- */
/* i<j pairs with r2 < sl2, computed as makepair does (dx = q_i - q_j), rows
 * ascending in j; brute force O(N^2).  Writes number_of_partners[n],
 * pointer[n] and list[cap]; returns the number of entries or -1 on overflow. */
int64_t lj_or_build_half_brute(const double* q4, int n, double sl2, const double* box,
                               int32_t* np, int32_t* ptr, int32_t* list, int64_t cap);
/* Same list, built with a cell grid (identical output, O(N)). full != 0 gives
 * every j != i per row (the reference's full list, force_cuda.cu:133-135). */
int64_t lj_or_build_list_cells(const double* q4, int n, double sl2, const double* box,
                               int full, int32_t* np, int32_t* ptr, int32_t* list,
                               int64_t cap);
/* rows [row0, row1) of the same list; np, ptr indexed by i - row0 */
int64_t lj_or_build_rows_cells(const double* q4, int n, double sl2, const double* box, int full,
                               int row0, int row1, int32_t* np, int32_t* ptr, int32_t* list,
                               int64_t cap);
/* (i, j) pair array in makepair order from a CSR half list. */
void lj_or_csr_to_pairs(int n, const int32_t* np, const int32_t* ptr, const int32_t* list,
                        int32_t* ip, int32_t* jp);

/* ---- force routines (kick p += F dt), FP64 ---- */
/* force_pair: scatter over an unsorted pair array (cpu_ref/force_aos.cpp:171-190) */
void lj_or_force_pair_aos(const double* q4, double* p4, int64_t npairs, const int32_t* ip,
                          const int32_t* jp, double cl2, double dt, const double* box);
/* force_sorted: scatter over the i-sorted half CSR (cpu_ref/force_aos.cpp:192-224) */
void lj_or_force_sorted_aos(const double* q4, double* p4, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box);
/* force_sorted SoA (cpu_ref/force_soa.cpp:163-195) */
void lj_or_force_sorted_soa(const double* qx, const double* qy, const double* qz,
                            double* px, double* py, double* pz, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box);
/* gather over a full CSR list, the CUDA reference's force_kernel_memopt
 * semantics (cuda/kernel.cuh:67-100): p_i += sum_j df * d.  nthreads <= 0 uses
 * every OpenMP thread, 1 runs serially. */
void lj_or_force_gather_aos(const double* q4, double* p4, int n, const int32_t* np,
                            const int32_t* ptr, const int32_t* list, double cl2, double dt,
                            const double* box, int nthreads);
/* the gather over rows [row0, row1); np, ptr indexed by i - row0 */
void lj_or_force_gather_rows_aos(const double* q4, double* p4, int row0, int row1,
                                 const int32_t* np, const int32_t* ptr, const int32_t* list,
                                 double cl2, double dt, const double* box, int nthreads);
int  lj_or_max_threads(void);

/* ---- energies and integration (project extension: the reference has none) ---- */
/* potential energy sum over the half list of 4 (r^-12 - r^-6) for r2 <= cl2 */
double lj_or_potential_half(const double* q4, int n, const int32_t* np, const int32_t* ptr,
                            const int32_t* list, double cl2, const double* box);
double lj_or_kinetic(const double* p4, int n);
/* positions drift q += p dt, then wrap into [0, L) when box != NULL */
void   lj_or_drift(double* q4, const double* p4, int n, double dt, const double* box);

#ifdef __cplusplus
}
#endif
#endif
