// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Linked together with the reference's own cpu_ref/force_aos.cpp (LJ_SHIM_AOS)
// or cpu_ref/force_soa.cpp (LJ_SHIM_SOA), compiled unmodified from where they
// lie (see Makefile).  The reference keeps its state in globals; this shim
// declares them and exposes a C interface so tests can load inputs, run the
// reference's force routines and read p back.  Nothing here re-implements
// reference arithmetic.
#include <cstdint>
#include <cstring>

// Globals and routines defined by the reference translation unit.
#if defined(LJ_SHIM_AOS)
extern double q[400000][4];
extern double p[400000][4];
#define QX(i) q[i][0]
#define QY(i) q[i][1]
#define QZ(i) q[i][2]
#define PX(i) p[i][0]
#define PY(i) p[i][1]
#define PZ(i) p[i][2]
void force_sorted_z(void);
void force_sorted_z_intrin(void);
void force_intrin_mat_transpose(void);
void copy_to_z(void);
void copy_from_z(void);
#elif defined(LJ_SHIM_SOA)
extern double q[4][400000];
extern double p[4][400000];
#define QX(i) q[0][i]
#define QY(i) q[1][i]
#define QZ(i) q[2][i]
#define PX(i) p[0][i]
#define PY(i) p[1][i]
#define PZ(i) p[2][i]
#else
#error "define LJ_SHIM_AOS or LJ_SHIM_SOA"
#endif
extern double L;
extern int particle_number;
extern int number_of_pairs;
extern int number_of_partners[400000];
extern int i_particles[];
extern int j_particles[];
extern int pointer[400000];
extern int sorted_list[];
void init(void);
void makepair(void);
void sortpair(void);
void force_pair(void);
void force_sorted(void);
void force_next(void);
void force_intrin(void);
void savepair(void);
void loadpair(void);

static const int kMaxN = 400000;
static const long kMaxPairs = 30L * 400000L;

extern "C" {

int ref_capacity_particles(void) { return kMaxN; }
long ref_capacity_pairs(void) { return kMaxPairs; }
int ref_particle_number(void) { return particle_number; }
int ref_number_of_pairs(void) { return number_of_pairs; }

// Runs the reference init() (its compiled-in density and L).  The reference's
// jitter generator is a function-local static, so this is meaningful once per
// loaded library.
int ref_init(double box_len) {
  L = box_len;
  particle_number = 0;
  init();
  return particle_number;
}

int ref_set_positions(int n, const double* q4) {
  if (n < 0 || n > kMaxN) return -1;
  particle_number = n;
  for (int i = 0; i < n; i++) {
    QX(i) = q4[4 * i + 0];
    QY(i) = q4[4 * i + 1];
    QZ(i) = q4[4 * i + 2];
  }
  return n;
}

void ref_get_positions(double* q4) {
  for (int i = 0; i < particle_number; i++) {
    q4[4 * i + 0] = QX(i);
    q4[4 * i + 1] = QY(i);
    q4[4 * i + 2] = QZ(i);
    q4[4 * i + 3] = 0.0;
  }
}

void ref_set_momenta(const double* p4) {
  for (int i = 0; i < particle_number; i++) {
    PX(i) = p4[4 * i + 0];
    PY(i) = p4[4 * i + 1];
    PZ(i) = p4[4 * i + 2];
  }
}

void ref_get_momenta(double* p4) {
  for (int i = 0; i < particle_number; i++) {
    p4[4 * i + 0] = PX(i);
    p4[4 * i + 1] = PY(i);
    p4[4 * i + 2] = PZ(i);
    p4[4 * i + 3] = 0.0;
  }
}

// The reference's O(N^2) makepair() on the current positions.
int ref_makepair(void) {
  number_of_pairs = 0;
  makepair();
  return number_of_pairs;
}

// Installs an (i, j) pair array the way register_pair leaves it, then runs
// the reference's sortpair() to build the CSR.
int ref_set_pairs(long npairs, const int* ip, const int* jp) {
  if (npairs < 0 || npairs > kMaxPairs) return -1;
  for (int i = 0; i < particle_number; i++) number_of_partners[i] = 0;
  for (long k = 0; k < npairs; k++) {
    i_particles[k] = ip[k];
    j_particles[k] = jp[k];
    number_of_partners[ip[k]]++;
  }
  number_of_pairs = (int)npairs;
  sortpair();
  return number_of_pairs;
}

// After ref_makepair(): build the CSR with the reference's sortpair().
void ref_sortpair(void) { sortpair(); }

void ref_get_pairs(int* ip, int* jp) {
  std::memcpy(ip, i_particles, sizeof(int) * (size_t)number_of_pairs);
  std::memcpy(jp, j_particles, sizeof(int) * (size_t)number_of_pairs);
}

void ref_get_csr(int* np, int* ptr, int* list) {
  std::memcpy(np, number_of_partners, sizeof(int) * (size_t)particle_number);
  std::memcpy(ptr, pointer, sizeof(int) * (size_t)particle_number);
  std::memcpy(list, sorted_list, sizeof(int) * (size_t)number_of_pairs);
}

// The reference's binary pair cache, written / read in the current directory
// ("pair.dat", cpu_ref/force_aos.cpp:603-620).  savepair() runs makepair().
int ref_savepair_cwd(void) {
  number_of_pairs = 0;
  savepair();
  return number_of_pairs;
}

int ref_loadpair_cwd(void) {
  loadpair();
  return number_of_pairs;
}

// Runs `calls` invocations of the named reference routine (as measure() does).
int ref_run(const char* name, int calls) {
  void (*fn)(void) = nullptr;
  if (!std::strcmp(name, "pair")) fn = force_pair;
  else if (!std::strcmp(name, "sorted")) fn = force_sorted;
  else if (!std::strcmp(name, "next")) fn = force_next;
  else if (!std::strcmp(name, "intrin")) fn = force_intrin;
#if defined(LJ_SHIM_AOS)
  else if (!std::strcmp(name, "intrin_mat_transpose")) fn = force_intrin_mat_transpose;
  else if (!std::strcmp(name, "sorted_z") || !std::strcmp(name, "sorted_z_intrin")) {
    copy_to_z();
    void (*zf)(void) = !std::strcmp(name, "sorted_z") ? force_sorted_z : force_sorted_z_intrin;
    for (int c = 0; c < calls; c++) zf();
    copy_from_z();
    return 0;
  }
#endif
  if (!fn) return -1;
  for (int c = 0; c < calls; c++) fn();
  return 0;
}

}  // extern "C"
