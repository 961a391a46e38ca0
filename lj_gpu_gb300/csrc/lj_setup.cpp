// lj_setup.cpp -- host-side parts of the C ABI: system generators, row
// shuffling and the reference's pair-list file formats.
//
// The generators and the shuffle use the C++ standard library's std::mt19937 /
// std::mt19937_64, distributions and std::shuffle directly, so the streams are
// the reference's own whenever the same standard library is used (libstdc++
// here and on the reference's build).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "lj_gb300.h"

extern "C" {

// cpu_ref/force_aos.cpp:142-169 with add_particle :43-51
int lj_init_reference(double density, double box_len, double* q, int32_t capacity,
                      int32_t* n_out) {
  if (!(density > 0.0) || !(box_len > 0.0) || capacity < 0 || (!q && capacity > 0))
    return LJ_ERR_INVALID_ARGUMENT;
  const double s = 1.0 / std::pow(density * 0.25, 1.0 / 3.0);
  const double hs = s * 0.5;
  const long cells = static_cast<long>(box_len / s);
  const long total = 4 * cells * cells * cells;
  if (n_out) *n_out = (int32_t)total;
  if (total > capacity) return LJ_ERR_LIST_OVERFLOW;
  std::mt19937 mt(2);
  std::uniform_real_distribution<double> ud(0.0, 0.1);
  int32_t n = 0;
  auto add = [&](double x, double y, double z) {
    q[4 * n + 0] = x + ud(mt);
    q[4 * n + 1] = y + ud(mt);
    q[4 * n + 2] = z + ud(mt);
    q[4 * n + 3] = 0.0;
    n++;
  };
  for (long iz = 0; iz < cells; iz++)
    for (long iy = 0; iy < cells; iy++)
      for (long ix = 0; ix < cells; ix++) {
        const double x = ix * s, y = iy * s, z = iz * s;
        add(x, y, z);
        add(x, y + hs, z + hs);
        add(x + hs, y, z + hs);
        add(x + hs, y + hs, z);
      }
  return LJ_OK;
}

static double wrap_into(double x, double L) {
  if (x >= L) x -= L;
  if (x < 0.0) x += L;
  if (x >= L) x = 0.0;
  return x;
}

int lj_init_fcc(int32_t ncell, double density, double jitter, uint64_t seed, double* q,
                int32_t capacity, double* box_len) {
  if (ncell < 1 || !(density > 0.0) || !(jitter >= 0.0)) return LJ_ERR_INVALID_ARGUMENT;
  const long total = 4L * ncell * ncell * ncell;
  if (total > capacity || !q) return total > capacity ? LJ_ERR_LIST_OVERFLOW
                                                      : LJ_ERR_INVALID_ARGUMENT;
  const double a = std::pow(4.0 / density, 1.0 / 3.0);
  const double L = ncell * a, ha = 0.5 * a;
  std::mt19937_64 mt(seed);
  std::uniform_real_distribution<double> ud(-jitter, jitter);
  static const double site[4][3] = {{0, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
  long n = 0;
  for (int iz = 0; iz < ncell; iz++)
    for (int iy = 0; iy < ncell; iy++)
      for (int ix = 0; ix < ncell; ix++)
        for (int k = 0; k < 4; k++) {
          const double bx = ix * a + site[k][0] * ha;
          const double by = iy * a + site[k][1] * ha;
          const double bz = iz * a + site[k][2] * ha;
          const double jx = ud(mt), jy = ud(mt), jz = ud(mt);
          q[4 * n + 0] = wrap_into(bx + jx, L);
          q[4 * n + 1] = wrap_into(by + jy, L);
          q[4 * n + 2] = wrap_into(bz + jz, L);
          q[4 * n + 3] = 0.0;
          n++;
        }
  if (box_len) *box_len = L;
  return LJ_OK;
}

int lj_init_momenta(double* p, int32_t n, double temperature, uint64_t seed) {
  if (n < 0 || (n > 0 && !p) || !(temperature >= 0.0)) return LJ_ERR_INVALID_ARGUMENT;
  std::mt19937_64 mt(seed);
  std::normal_distribution<double> nd(0.0, std::sqrt(temperature));
  double s[3] = {0, 0, 0};
  for (int32_t i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++) {
      p[4 * i + d] = nd(mt);
      s[d] += p[4 * i + d];
    }
    p[4 * i + 3] = 0.0;
  }
  for (int d = 0; d < 3; d++) s[d] /= (n > 0 ? n : 1);
  for (int32_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) p[4 * i + d] -= s[d];
  return LJ_OK;
}

// random_shfl (cuda/force_cuda.cu:255-263): one std::mt19937(seed) shuffles
// every row in turn with std::shuffle, rows in i order.
int lj_list_shuffle_rows(int32_t n, const int32_t* np, const int32_t* ptr, int32_t* list,
                         uint32_t seed) {
  if (n < 0 || (n > 0 && (!np || !ptr || !list))) return LJ_ERR_INVALID_ARGUMENT;
  std::mt19937 mt(seed);
  for (int32_t i = 0; i < n; i++) {
    if (np[i] < 0 || ptr[i] < 0) return LJ_ERR_BAD_LIST;
    std::shuffle(list + ptr[i], list + ptr[i] + np[i], mt);
  }
  return LJ_OK;
}

// Text pair-list cache of the CUDA driver (makepaircache / loadpair,
// cuda/force_cuda.cu:165-227): "n npairs", then n lines "np ptr", then
// npairs lines "j".
int lj_cache_write_text(const char* path, int32_t n, const int32_t* np, const int32_t* ptr,
                        const int32_t* list, int64_t n_entries) {
  if (!path || n < 0 || n_entries < 0 || (n > 0 && (!np || !ptr)) || (n_entries > 0 && !list))
    return LJ_ERR_INVALID_ARGUMENT;
  FILE* fp = std::fopen(path, "w");
  if (!fp) return LJ_ERR_INVALID_ARGUMENT;
  std::fprintf(fp, "%d %lld\n", n, (long long)n_entries);
  for (int32_t i = 0; i < n; i++) std::fprintf(fp, "%d %d\n", np[i], ptr[i]);
  for (int64_t k = 0; k < n_entries; k++) std::fprintf(fp, "%d\n", list[k]);
  const bool ok = std::fclose(fp) == 0;
  return ok ? LJ_OK : LJ_ERR_INVALID_ARGUMENT;
}

// Reads it back; the particle count must match (else the cache "may be
// broken", loadpair), and the arrays are checked as check_loadedpair does.
int lj_cache_read_text(const char* path, int32_t n, int32_t* np, int32_t* ptr, int32_t* list,
                       int64_t capacity, int64_t* n_entries) {
  if (!path || n < 0 || (n > 0 && (!np || !ptr))) return LJ_ERR_INVALID_ARGUMENT;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return LJ_ERR_INVALID_ARGUMENT;
  int nn = 0;
  long long ne = 0;
  int rc = LJ_OK;
  if (std::fscanf(fp, "%d %lld", &nn, &ne) != 2 || nn != n || ne < 0) rc = LJ_ERR_BAD_LIST;
  if (rc == LJ_OK && n_entries) *n_entries = ne;
  if (rc == LJ_OK && ne > capacity) rc = LJ_ERR_LIST_OVERFLOW;
  for (int32_t i = 0; rc == LJ_OK && i < n; i++)
    if (std::fscanf(fp, "%d %d", &np[i], &ptr[i]) != 2) rc = LJ_ERR_BAD_LIST;
  for (long long k = 0; rc == LJ_OK && k < ne; k++)
    if (std::fscanf(fp, "%d", &list[k]) != 1) rc = LJ_ERR_BAD_LIST;
  std::fclose(fp);
  for (int32_t i = 0; rc == LJ_OK && i < n; i++)
    if (np[i] < 0 || np[i] >= n || ptr[i] < 0 || ptr[i] > ne || (long long)ptr[i] + np[i] > ne)
      rc = LJ_ERR_BAD_LIST;
  for (long long k = 0; rc == LJ_OK && k < ne; k++)
    if (list[k] < 0 || list[k] >= n) rc = LJ_ERR_BAD_LIST;
  return rc;
}

// Binary pair cache of cpu_ref (savepair / loadpair,
// cpu_ref/force_aos.cpp:603-620): int number_of_pairs, int
// number_of_partners[400000], int i_particles[12000000], int
// j_particles[12000000]; unused tails are zero.
static const int kPairDatN = 400000;
static const int64_t kPairDatPairs = 30LL * 400000LL;

int lj_pairdat_write(const char* path, int32_t n, const int32_t* i_particles,
                     const int32_t* j_particles, int64_t n_pairs) {
  if (!path || n < 0 || n > kPairDatN || n_pairs < 0 || n_pairs > kPairDatPairs ||
      (n_pairs > 0 && (!i_particles || !j_particles)))
    return LJ_ERR_INVALID_ARGUMENT;
  std::vector<int32_t> npart((size_t)kPairDatN, 0), buf((size_t)kPairDatPairs, 0);
  for (int64_t k = 0; k < n_pairs; k++) {
    if (i_particles[k] < 0 || i_particles[k] >= n) return LJ_ERR_BAD_LIST;
    npart[(size_t)i_particles[k]]++;
  }
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return LJ_ERR_INVALID_ARGUMENT;
  const int32_t np32 = (int32_t)n_pairs;
  bool ok = std::fwrite(&np32, sizeof np32, 1, fp) == 1;
  ok = ok && std::fwrite(npart.data(), sizeof(int32_t), npart.size(), fp) == npart.size();
  std::copy(i_particles, i_particles + n_pairs, buf.begin());
  ok = ok && std::fwrite(buf.data(), sizeof(int32_t), buf.size(), fp) == buf.size();
  std::fill(buf.begin(), buf.end(), 0);
  std::copy(j_particles, j_particles + n_pairs, buf.begin());
  ok = ok && std::fwrite(buf.data(), sizeof(int32_t), buf.size(), fp) == buf.size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? LJ_OK : LJ_ERR_INVALID_ARGUMENT;
}

int lj_pairdat_read(const char* path, int32_t n, int32_t* number_of_partners,
                    int32_t* i_particles, int32_t* j_particles, int64_t capacity,
                    int64_t* n_pairs) {
  if (!path || n < 0 || n > kPairDatN) return LJ_ERR_INVALID_ARGUMENT;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return LJ_ERR_INVALID_ARGUMENT;
  int32_t np32 = 0;
  std::vector<int32_t> npart((size_t)kPairDatN);
  bool ok = std::fread(&np32, sizeof np32, 1, fp) == 1 && np32 >= 0 && np32 <= kPairDatPairs;
  ok = ok && std::fread(npart.data(), sizeof(int32_t), npart.size(), fp) == npart.size();
  if (ok && n_pairs) *n_pairs = np32;
  if (ok && np32 > capacity) {
    std::fclose(fp);
    return LJ_ERR_LIST_OVERFLOW;
  }
  std::vector<int32_t> buf((size_t)kPairDatPairs);
  ok = ok && std::fread(buf.data(), sizeof(int32_t), buf.size(), fp) == buf.size();
  if (ok) std::copy(buf.begin(), buf.begin() + np32, i_particles);
  ok = ok && std::fread(buf.data(), sizeof(int32_t), buf.size(), fp) == buf.size();
  if (ok) std::copy(buf.begin(), buf.begin() + np32, j_particles);
  std::fclose(fp);
  if (!ok) return LJ_ERR_BAD_LIST;
  for (int32_t i = 0; i < n; i++) {
    if (number_of_partners) number_of_partners[i] = npart[(size_t)i];
  }
  for (int32_t k = 0; k < np32; k++)
    if (i_particles[k] < 0 || i_particles[k] >= n || j_particles[k] < 0 || j_particles[k] >= n)
      return LJ_ERR_BAD_LIST;
  return LJ_OK;
}

}  // extern "C"
