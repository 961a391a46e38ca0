// lj_setup.cpp -- host-side system set-up of the C ABI (generators).
//
// These use the C++ standard library's std::mt19937 / std::mt19937_64 and
// distributions directly, so the streams are the reference's own whenever the
// same standard library is used (libstdc++ here and on the reference's
// build).
#include <cmath>
#include <random>

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

}  // extern "C"
