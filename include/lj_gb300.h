/*
 * lj_gb300.h -- C ABI of the GB300 Lennard-Jones neighbour-list force engine.
 *
 * The engine keeps the force-routine contract of the reference
 * (kohnakagawa/lj_gpu): positions q and momenta p, an i-sorted CSR neighbour
 * list given as number_of_partners / pointer / sorted_list, a cutoff CL2, and
 * the in-place kick
 *
 *     p_i += sum_j df(r_ij) * (q_j - q_i),   df = ((24 r^6 - 48) / r^14) * dt,
 *     pairs with r2 > CL2 skipped,
 *
 * applied symmetrically (p_j -= ...) for a half list, as cpu_ref
 * force_sorted does (cpu_ref/force_aos.cpp:192-224) and as the CUDA kernels do
 * (cuda/kernel.cuh:5-34 gather over the full list, :238-469 scatter over the
 * half list).
 *
 * Every entry point returns an int status (LJ_OK == 0) and never exits the
 * process.  Device-pointer entry points are stream ordered and asynchronous;
 * the stream argument is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  Memory passed in is owned by the caller.  A context is not thread
 * safe: use one per host thread.
 *
 * Layouts: AoS q/p are double[n][4] (x, y, z, w; w unused and untouched,
 * at least 16-byte aligned: the reference's double4 / cpu_ref q[N][4]).  SoA passes
 * the three coordinate arrays separately (cpu_ref/force_soa.cpp q[X], q[Y],
 * q[Z] rows).  Indices are int32, offsets in pointer[] are int32 (as in the
 * reference), list lengths are int64.
 */
#ifndef LJ_GB300_H
#define LJ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LJ_GB300_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
enum {
  LJ_OK = 0,
  LJ_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size or enum value        */
  LJ_ERR_BAD_LIST = 2,         /* list failed validation (check_loadedpair)   */
  LJ_ERR_CUDA = 3,             /* a CUDA runtime call failed                   */
  LJ_ERR_OUT_OF_MEMORY = 4,    /* device or pinned allocation failed           */
  LJ_ERR_LIST_OVERFLOW = 5,    /* a neighbour build exceeded its capacity      */
  LJ_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up           */
  LJ_ERR_NO_LIST = 7,          /* force called before a list was installed     */
  LJ_ERR_UNSUPPORTED = 8       /* combination not provided                     */
};

/* ---- enumerations ------------------------------------------------------- */
/* LJ_PREC_FP64: the reference's FP64 arithmetic.
 * LJ_PREC_MIXED: FP64 positions, momenta and kick; pair terms in two-float
 *   (float-float) arithmetic from 42-bit fixed-point separations, with
 *   compensated sums: per-particle force error about 1e-9 relative to FP64.
 * LJ_PREC_MIXED_FP32: as MIXED with single FP32 pair terms (faster; its
 *   per-particle error reaches ~1e-4 on particles whose pair terms cancel,
 *   ~1e-6 of the RMS force). */
enum { LJ_PREC_FP64 = 0, LJ_PREC_MIXED = 1, LJ_PREC_MIXED_FP32 = 2 };
enum { LJ_LIST_HALF = 0, LJ_LIST_FULL = 1 };
enum { LJ_WHERE_HOST = 0, LJ_WHERE_DEVICE = 1 };
/* Particle layouts (the entry point called): lj_force_aos, lj_force_soa,
 * lj_force_z (the reference's force_sorted / force_soa / force_sorted_z). */
enum { LJ_LAYOUT_AOS = 0, LJ_LAYOUT_SOA = 1, LJ_LAYOUT_Z = 2 };
enum {
  LJ_METHOD_AUTO = 0,         /* engine choice (tuned per precision)          */
  LJ_METHOD_GATHER_FULL = 1,  /* full list, each row writes only its own p_i  */
  LJ_METHOD_SCATTER_HALF = 2  /* half list, p_j updated with atomics          */
};

/* ---- options of one force call ------------------------------------------ */
typedef struct lj_force_opts {
  double dt;          /* kick length: p += F dt (reference dt)                 */
  double cl2;         /* squared cutoff (reference CL2); r2 > cl2 is skipped  */
  double box[3];      /* periodic box lengths, used when periodic != 0        */
  int32_t periodic;   /* 0: open boundaries (the reference), 1: minimum image */
  int32_t precision;  /* LJ_PREC_FP64, LJ_PREC_MIXED or LJ_PREC_MIXED_FP32     */
  int32_t method;     /* LJ_METHOD_*                                          */
  int32_t lanes;      /* lanes per i-particle, 0 = default, else 1,2,4,..,32  */
  int32_t block;      /* threads per block, 0 = default, else 64..256         */
  int32_t kernel;     /* kernel generation: 0 = default, 1 = simple strided,
                         2 = unrolled / compacted, 3 = cell-tiled (mixed
                         gather on a list from lj_list_build), 4 = unrolled
                         with 16-byte index loads (mixed gather, unroll 4),
                         5 = gather over the transposed ("ELL") copy of the
                         full list, entry k of row i at [i + k n], one lane
                         per row (the reference's force_kernel_memopt2 /
                         _unrolling2 layout, cuda/kernel.cuh:102-134,
                         547-620; mixed: every pair in the precision's own
                         terms, unroll 2 or 4); 3 and 4 fall back to 2 when
                         their list form is missing (see lj_force.cu)       */
  int32_t unroll;     /* entries per lane in flight (kernel 2), 0 = default   */
  int32_t ff_all;     /* LJ_PREC_MIXED gathers (kernels 2 and 4): 0 = pairs
                         beyond 2.1 sigma of the first call's positions in
                         FP32 terms, any pair closer than 2.0 sigma in
                         two-float terms (the default); 1 = every pair in
                         two-float terms                                     */
} lj_force_opts;

/* dt = 0.001, cl2 = 9.0 (cpu_ref/force_aos.cpp:14,31-33), open box, FP64, auto */
void lj_force_opts_default(lj_force_opts* opts);

typedef struct lj_ctx lj_ctx;

int lj_abi_version(void);
const char* lj_status_string(int status);

/* ---- context ------------------------------------------------------------ */
int lj_ctx_create(lj_ctx** out, int device);
void lj_ctx_destroy(lj_ctx* ctx);
/* message of the last failing call on this context ("" if none) */
const char* lj_ctx_last_error(const lj_ctx* ctx);
/* stream used by every later call on ctx (cudaStream_t as void*) */
int lj_ctx_set_stream(lj_ctx* ctx, void* stream);
/* Per-stage device timing of force calls (the reference times with
 * gettimeofday around 100 calls, cuda/force_cuda.cu:330-341; this records
 * CUDA events around the engine's own launches).  on = 1 enables and resets
 * the sums, 0 disables. */
int lj_ctx_set_timing(lj_ctx* ctx, int32_t on);
/* ms[0]: position-image passes, ms[1]: pair kernels, ms[2]: both, summed
 * over *calls force calls since the last reset (synchronises). */
int lj_ctx_get_timing(lj_ctx* ctx, double* ms, int64_t* calls);
/* L2 persistence for the randomly gathered j positions: with hit_ratio in
 * (0, 1], the pair kernel of
 * every later mixed force call on ctx runs with an access-policy window over
 * the fixed-point position image (persisting hits for that fraction of it,
 * streaming misses), and the context reserves that many bytes of L2 as
 * persisting (its own limit, restored when the context is destroyed).
 * 0 (the default) turns it off.  A cache hint: results are unchanged.  The
 * window is an attribute of the context's stream, so force calls on a
 * context without one (lj_ctx_set_stream) return LJ_ERR_UNSUPPORTED while
 * it is on.  The MD loop's captured graphs do not use it. */
int lj_ctx_set_l2_window(lj_ctx* ctx, double hit_ratio);

/* ---- neighbour lists ---------------------------------------------------- */
/* Installs an i-sorted CSR list for n particles (replaces the reference's
 * copy_to_gpu of sorted_list / number_of_partners / pointer,
 * cuda/force_cuda.cu:302-312).  The arrays are copied into the context, so
 * the caller may free them afterwards.  Validation follows check_loadedpair
 * (cuda/force_cuda.cu:183-201) plus row bounds:
 *   0 <= number_of_partners[i] < n, 0 <= pointer[i] <= n_entries,
 *   pointer[i] + number_of_partners[i] <= n_entries, 0 <= sorted_list[k] < n.
 * kind: LJ_LIST_HALF (each unordered pair once, as makepair with
 * EN_ACTION_REACTION builds it) or LJ_LIST_FULL (each pair in both rows).
 * Rows are copied into a compact layout (row i directly after row i - 1),
 * so pointer may describe any non-overlapping placement; lj_list_get_csr
 * returns the compact form.  A half list is expanded on the device into the
 * full list the gather kernels use; both are kept. */
int lj_list_set_csr(lj_ctx* ctx, int32_t n, const int32_t* number_of_partners,
                    const int32_t* pointer, const int32_t* sorted_list, int64_t n_entries,
                    int32_t kind, int32_t where);
/* Installs the reference's unsorted (i, j) pair arrays (register_pair,
 * cpu_ref/force_aos.cpp:60-74) and sorts them into a half CSR on the device
 * exactly as sortpair does (cpu_ref/force_aos.cpp:100-120): rows in i order,
 * entries of a row in pair-array order. */
int lj_list_set_pairs(lj_ctx* ctx, int32_t n, const int32_t* i_particles,
                      const int32_t* j_particles, int64_t n_pairs, int32_t where);
/* Copies the installed list (kind LJ_LIST_HALF or LJ_LIST_FULL) into caller
 * arrays of the given location.  *n_entries receives the entry count; if
 * capacity is too small nothing is copied and LJ_ERR_LIST_OVERFLOW is
 * returned. */
int lj_list_get_csr(lj_ctx* ctx, int32_t kind, int32_t* number_of_partners, int32_t* pointer,
                    int32_t* sorted_list, int64_t capacity, int64_t* n_entries, int32_t where);
/* Installs a list given in the reference's transposed ("ELL") layout: entry
 * k of row i at transposed_list[i + k * width], width >= n, ell_len ints in
 * the array (make_transposed_pairlist, cuda/force_cuda.cu:229-240, the input
 * of its memopt2/memopt3/unrolling kernels).  Converted to the compact CSR on
 * the device; validation as lj_list_set_csr plus the array bounds. */
int lj_list_set_ell(lj_ctx* ctx, int32_t n, const int32_t* number_of_partners,
                    const int32_t* transposed_list, int64_t width, int64_t ell_len,
                    int32_t kind, int32_t where);
/* Exports the installed list in that layout (zero-filled first, as the
 * reference does); ell_len must be >= max_row * width. */
int lj_list_get_ell(lj_ctx* ctx, int32_t kind, int32_t* number_of_partners,
                    int32_t* transposed_list, int64_t width, int64_t ell_len, int32_t where);
/* Host helpers for the reference's list files and row order (no GPU):
 *   lj_list_shuffle_rows: random_shfl (cuda/force_cuda.cu:255-263), one
 *     std::mt19937(seed) shuffling every row in i order, in place;
 *   lj_cache_write_text / lj_cache_read_text: the CUDA driver's text cache
 *     (.cache_pair_{half,all}.dat, cuda/force_cuda.cu:165-227); the reader
 *     checks the particle count and the arrays as loadpair and
 *     check_loadedpair do;
 *   lj_pairdat_write / lj_pairdat_read: cpu_ref's binary pair.dat
 *     (cpu_ref/force_aos.cpp:603-620), fixed-size arrays of 400,000 partner
 *     counts and 12,000,000 (i, j) pairs. */
int lj_list_shuffle_rows(int32_t n, const int32_t* number_of_partners, const int32_t* pointer,
                         int32_t* sorted_list, uint32_t seed);
int lj_cache_write_text(const char* path, int32_t n, const int32_t* number_of_partners,
                        const int32_t* pointer, const int32_t* sorted_list, int64_t n_entries);
int lj_cache_read_text(const char* path, int32_t n, int32_t* number_of_partners, int32_t* pointer,
                       int32_t* sorted_list, int64_t capacity, int64_t* n_entries);
int lj_pairdat_write(const char* path, int32_t n, const int32_t* i_particles,
                     const int32_t* j_particles, int64_t n_pairs);
int lj_pairdat_read(const char* path, int32_t n, int32_t* number_of_partners,
                    int32_t* i_particles, int32_t* j_particles, int64_t capacity,
                    int64_t* n_pairs);
/* Number of particles and entries of the installed list (0 if none). */
int lj_list_info(const lj_ctx* ctx, int32_t kind, int32_t* n, int64_t* n_entries,
                 int32_t* max_row);

/* ---- force calls (device pointers) -------------------------------------- */
/* One force call p += F dt with the installed list: the context equivalent of
 * one force_kernel_* launch (cuda/force_cuda.cu:334) or one cpu_ref
 * force_sorted() call.  q and p are AoS double[n][4] on the device. */
int lj_force_aos(lj_ctx* ctx, const double* q, double* p, int32_t n, const lj_force_opts* opts);
/* SoA variant (cpu_ref/force_soa.cpp:163-195); six device arrays of n doubles */
int lj_force_soa(lj_ctx* ctx, const double* qx, const double* qy, const double* qz, double* px,
                 double* py, double* pz, int32_t n, const lj_force_opts* opts);

/* Interleaved layout z[n][8] = {q.x, q.y, q.z, q.w, p.x, p.y, p.z, p.w}, one
 * 64-byte record per particle (cpu_ref force_sorted_z,
 * cpu_ref/force_aos.cpp:226-258); q is read, p updated in place. */
int lj_force_z(lj_ctx* ctx, double* z, int32_t n, const lj_force_opts* opts);

/* Stateless FP64 drop-in for a reference kernel launch: the argument list of
 * force_kernel_* (cuda/kernel.cuh:5-13) on AoS double4 buffers, with the list
 * kind saying whether list is a full list (gather, like force_kernel_memopt /
 * warp_unroll) or a half list (scatter with atomics, like the _with_aar
 * kernels).  box == NULL gives open boundaries.  Allocates nothing and does
 * not validate the list (the reference kernels do not either). */
int lj_force_csr_fp64_aos(const double* q, double* p, int32_t n, double dt, double cl2,
                          const int32_t* sorted_list, const int32_t* number_of_partners,
                          const int32_t* pointer, int32_t kind, const double* box,
                          void* stream);
/* force_pair on the device (cpu_ref/force_aos.cpp:171-190): FP64 scatter over
 * an unsorted (i, j) pair array, both ends updated with atomics.  The pair
 * indices are not validated (force_pair does not either): each must be in
 * [0, n). */
int lj_force_pairs_fp64_aos(const double* q, double* p, int32_t n, double dt, double cl2,
                            const int32_t* i_particles, const int32_t* j_particles,
                            int64_t n_pairs, const double* box, void* stream);

/* Mixed-precision force call over a FULL CSR list that allocates nothing
 * (no cudaMalloc, no cudaFree, no allocating library call).  This entry point
 * has no counterpart in the reference.  It exists for callers that cannot
 * allocate device memory: hosts that own every allocation through their own
 * pool, real-time loops where an allocation's implicit synchronisation is not
 * allowed, plugin hosts that forbid it.  Its scratch, the fixed-point
 * position image, lives in one static device array sized for at most
 * LJ_NOALLOC_MAX_PARTICLES particles (16 MiB held by every GPU that loads the
 * library); larger n returns LJ_ERR_INVALID_ARGUMENT.  Every call shares that
 * array, so calls that overlap on the GPU race: order them.  The first call on
 * a device looks up the array's device address; make it before any stream
 * capture.  Open boundaries (box == NULL) choose the fixed-point frame on the
 * device (no host round trip).  The list is used as given and not validated
 * (as in lj_force_pairs_fp64_aos): every index must lie in [0, n), or the
 * kernel reads positions past the caller's arrays and past the scratch
 * image.  Same arithmetic and launch shape as lj_force_aos with
 * LJ_PREC_MIXED, LJ_METHOD_GATHER_FULL, kernel 2, 4 lanes per row, 4 entries
 * in flight, 128 threads per block and ff_all = 1 (every pair in two-float
 * terms): the two give identical bits. */
#define LJ_NOALLOC_MAX_PARTICLES 1048576
int lj_force_mixed_noalloc_aos(const double* q, double* p, int32_t n, double dt, double cl2,
                               const int32_t* sorted_list, const int32_t* number_of_partners,
                               const int32_t* pointer, const double* box, void* stream);

/* ---- system set-up (host memory, no GPU needed) -------------------------- */
/* The reference's init() (cpu_ref/force_aos.cpp:142-169, add_particle :43-51):
 * FCC cells of side (4/density)^(1/3), floor(box_len / side) cells per axis,
 * jitter U[0, 0.1) per coordinate from std::mt19937(2) in call order x, y, z.
 * q is AoS double[capacity][4]; *n_out receives the particle count.
 * LJ_ERR_LIST_OVERFLOW if capacity is too small (nothing is written then). */
int lj_init_reference(double density, double box_len, double* q, int32_t capacity,
                      int32_t* n_out);
/* Periodic FCC of ncell^3 cells (N = 4 ncell^3) at the given density, box
 * L = ncell (4/density)^(1/3), each coordinate jittered by U[-jitter, jitter)
 * from std::mt19937_64(seed) in order x, y, z and wrapped into [0, L).
 * No reference counterpart (the reference has no periodic box). */
int lj_init_fcc(int32_t ncell, double density, double jitter, uint64_t seed, double* q,
                int32_t capacity, double* box_len);
/* Maxwell-Boltzmann momenta at temperature T (m = 1): N(0, T) per component
 * from std::mt19937_64(seed), total momentum removed.  p is AoS double[n][4].
 * No reference counterpart (the reference never integrates). */
int lj_init_momenta(double* p, int32_t n, double temperature, uint64_t seed);

/* ---- on-device neighbour build ------------------------------------------ */
enum { LJ_BUILD_HALF = 1, LJ_BUILD_FULL = 2 };
/* Builds the neighbour list of the AoS device positions q on the GPU with a
 * cell grid (cell side >= search_radius) and installs it in ctx, replacing
 * the reference's O(N^2) makepair + sortpair (cpu_ref/force_aos.cpp:100-140,
 * cuda/force_cuda.cu:122-163).  Membership is the reference's
 * r2 < search_radius^2 with dx = q_i - q_j (minimum image when box != NULL);
 * rows come out ascending in j, so the half list is exactly the reference's.
 * kinds: LJ_BUILD_HALF | LJ_BUILD_FULL (which lists to keep). */
int lj_list_build(lj_ctx* ctx, const double* q, int32_t n, double search_radius,
                  const double* box, int32_t kinds);

/* ---- molecular dynamics (project extension) ------------------------------- */
/* The reference never integrates: its 100 calls re-kick p from a fixed q
 * (cpu_ref/force_aos.cpp:592-601).  lj_md_run advances q and p with velocity
 * Verlet (m = 1) in a periodic box, using the force path above as the kick,
 * with on-device neighbour rebuilds whenever a particle has moved more than
 * skin/2 since the last build. */
typedef struct lj_md_params {
  double dt;              /* time step */
  double rc;              /* cutoff; list radius = rc + skin */
  double skin;            /* Verlet skin */
  double box[3];          /* periodic box lengths (each > 2 (rc + skin)) */
  int32_t precision;      /* LJ_PREC_MIXED (gather) or LJ_PREC_FP64 (scatter) */
  int32_t record_every;   /* energies every k steps (0: at 0 and at the end) */
  int32_t graph_steps;    /* steps per captured CUDA graph (0: 20, 1: no graph) */
  int32_t rebuild_every;  /* 0: rebuild when a particle moved > skin/2 since the
                             last build; k > 0: also every k steps */
  int32_t ff_all;         /* LJ_PREC_MIXED: 0 = pairs beyond 2.1 sigma at
                             the last rebuild in FP32 terms, any pair closer
                             than 2.0 sigma in two-float terms (the
                             default), 1 = every pair in two-float terms */
  int32_t chunk_graphs;   /* 0: the steps between records run as one launch of a
                             persistent graph (a WHILE node); 1: as chunk graphs
                             launched back to back from the host, whose kernels
                             profilers can capture one by one */
  int32_t kick_lanes;     /* lanes per row of the mixed gather kick: 0 = the
                             default (1 for LJ_PREC_MIXED, 4 for
                             LJ_PREC_MIXED_FP32), else 1, 2, 4 or 8 */
  int32_t reserved;
} lj_md_params;

typedef struct lj_md_record {
  int64_t step;
  double kinetic;    /* sum p^2 / 2 (FP64) */
  double potential;  /* sum over pairs r <= rc of 4 (r^-12 - r^-6), unshifted */
} lj_md_record;

typedef struct lj_md_stats {
  int64_t steps;
  int64_t rebuilds;       /* list builds after the initial one */
  double ms_total;        /* device time of the whole run */
  int64_t list_capacity;  /* entries reserved for the list */
  int64_t launches;       /* kernels launched by the run (-1: not counted) */
  int32_t loop_graph;     /* 1: the steps between records ran as one launch of a
                             persistent graph (a WHILE node counted down on the
                             device); 0: as back-to-back chunk graphs */
  int32_t initial_build;  /* 1: the run started with a list build; 0: it kept
                             the list of the context's previous run */
} lj_md_stats;

/* q, p: AoS device arrays (modified in place; p must hold the initial
 * momenta, e.g. from lj_init_momenta).  records may be NULL.  Positions are
 * wrapped into [0, L).  LJ_ERR_LIST_OVERFLOW if a rebuild would exceed the
 * list capacity (q, p are then partially advanced).  The context keeps the
 * neighbour list of a completed run: the next run with the same n, box, rc,
 * skin, precision and ff_all uses it unless a particle lies more than skin/2
 * from its position at that list's build (the Verlet criterion, checked on
 * the positions passed in), so runs that continue a trajectory skip the
 * initial build (stats->initial_build). */
int lj_md_run(lj_ctx* ctx, double* q, double* p, int32_t n, const lj_md_params* params,
              int32_t nsteps, lj_md_record* records, int32_t max_records, int32_t* n_records,
              lj_md_stats* stats);

/* lj_md_run over host arrays (AoS double[n][4], updated in place; page-locked
 * memory lets the copies overlap the run): q is copied to the device before
 * the initial list build, p beside that build on a second stream; at the end
 * q goes back beside the final half kick and p after it.  Returns once q and
 * p are back on the host.  Mirrors the reference's measure()
 * (cuda/force_cuda.cu:319-342: copy in, run, copy out) for the MD loop;
 * stats->ms_total includes the copies. */
int lj_md_run_host(lj_ctx* ctx, double* q, double* p, int32_t n, const lj_md_params* params,
                   int32_t nsteps, lj_md_record* records, int32_t max_records,
                   int32_t* n_records, lj_md_stats* stats);

/* ---- replica batches (project extension) --------------------------------- */
/* Many independent periodic systems of uneven size in one velocity-Verlet
 * loop (mixed precision): q, p hold the replicas back to back (AoS device
 * arrays of n_total particles); replica r owns particles
 * [offsets[r], offsets[r+1]) (host array of n_replicas + 1) in the cubic box
 * boxes[3 r .. 3 r + 2] (host).  params->box is ignored.  Every stage runs
 * once over the whole batch; the rows are split into size classes by their
 * expected length and each class's gather launch shape is timed and chosen at
 * start-up.  energies (host, may be NULL): per record, per replica,
 * (kinetic, potential).  class_shapes (host, may be NULL, 9 ints): per class
 * (rows, lanes, entries in flight).  The reference has no batching. */
int lj_batch_run(lj_ctx* ctx, double* q, double* p, int32_t n_total, int32_t n_replicas,
                 const int32_t* offsets, const double* boxes, const lj_md_params* params,
                 int32_t nsteps, double* energies, int32_t max_records, int32_t* n_records,
                 lj_md_stats* stats, int32_t* class_shapes);

/* ---- autotuner ------------------------------------------------------------ */
/* Times candidate launch shapes of one force call (method gather/scatter,
 * kernel generation, lanes per row, entries in flight, block size) on the
 * installed list and the device AoS positions q, `reps` calls each, and
 * returns the fastest in *best (the other fields are copied from *opts).
 * The caller's momenta are not touched (a scratch array is used).  The
 * winner is remembered: later calls with the same precision and boundary
 * kind that leave method = AUTO and every launch field 0 use it, until the
 * list changes.  The reference picks its kernel and THREAD_BLOCK by hand
 * (cuda/force_cuda.cu:45,378-383). */
int lj_autotune_aos(lj_ctx* ctx, const double* q, int32_t n, const lj_force_opts* opts,
                    int32_t reps, lj_force_opts* best, double* ms_best);

/* The tuner over launch shapes, list layouts and particle layouts, with a
 * persistent cache.  Every launch shape is timed on AoS positions (kernel 5
 * is the transposed-list layout); the three fastest are timed again on each
 * other particle layout asked for in `layouts` (bit 1 << LJ_LAYOUT_*, 0 =
 * AoS only), from copies of q the tuner makes.  The key of the problem
 * (`key`): GPU name and SM count, class of n (log2), class of the mean full
 * row length (the density at a given cutoff: round(2 log2(mean))), precision,
 * boundary kind, the requested method and the layout set.  With a cache file
 * (`cache_path`, NULL = none) a key found there returns its entry without
 * timing anything (from_cache = 1); otherwise the winner is appended to the
 * file.  The winner is remembered in the context for calls of its layout
 * that leave method = AUTO and every launch field 0, as lj_autotune_aos. */
typedef struct lj_tune_result {
  lj_force_opts best;   /* *opts with the winner's method and launch fields */
  int32_t layout;       /* LJ_LAYOUT_* of the winner                        */
  int32_t from_cache;   /* 1: read from the cache file, nothing was timed   */
  int32_t timed;        /* (shape, layout) candidates timed                 */
  int32_t reserved;
  double ms;            /* the winner's time per call (from the cache when
                           from_cache)                                       */
  char key[160];        /* the problem's cache key (NUL-terminated)          */
} lj_tune_result;
int lj_autotune(lj_ctx* ctx, const double* q, int32_t n, const lj_force_opts* opts,
                int32_t reps, int32_t layouts, const char* cache_path, lj_tune_result* out);

/* ---- host-buffer call (the reference's measure(), force_cuda.cu:319-342) - */
/* Uploads q and p from host memory, runs `calls` force calls on the installed
 * list, downloads p, and synchronises.  If the list was installed from host
 * memory it is uploaded again first, as copy_to_gpu does.  ms_total covers
 * the whole sequence, ms_calc only the force calls (either may be NULL). */
int lj_measure_aos(lj_ctx* ctx, const double* q_host, double* p_host, int32_t n,
                   const lj_force_opts* opts, int32_t calls, double* ms_total, double* ms_calc);

#ifdef __cplusplus
}
#endif
#endif /* LJ_GB300_H */
