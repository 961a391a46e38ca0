// lj_force.cu -- force-call entry of the kernels in lj_force_kernels.cuh:
// frames and position images, the FP64 force paths, force_pair, and the
// dispatch of the mixed paths to their own translation units.
#include "lj_force_kernels.cuh"

namespace ljg {

void make_fixed_frame(ForceLaunch& L) {
  auto axis_for = [](double scale, FixedAxis& ax) {
    int e;
    std::frexp(scale, &e);  // scale = f 2^e, f in [0.5, 1)
    ax.sigma = 64 - e;      // mult = scale 2^sigma in [2^63, 2^64)
    ax.mult = (unsigned long long)std::ldexp(scale, ax.sigma);
    ax.pad = 0;
  };
  if (L.box.on) {
    for (int d = 0; d < 3; d++) {
      const double scale = 4294967296.0 / L.box.len[d];
      axis_for(scale, L.axis[d]);
      L.unit[d] = L.box.len[d] / 4294967296.0;
    }
    L.aniso = !(L.box.len[0] == L.box.len[1] && L.box.len[1] == L.box.len[2]);
  } else {
    // the frame of coarse exponent 0; the kernels rescale it by the device's
    // choice (L.open_frame)
    for (int d = 0; d < 3; d++) {
      L.axis[d] = pow2_axis(0);
      L.unit[d] = 1.0;
    }
    L.aniso = 0;
  }
  for (int d = 0; d < 3; d++) L.origin[d] = 0;
}

void make_open_frame(ForceLaunch& L, int kf, const long long* origin) {
  for (int d = 0; d < 3; d++) {
    L.axis[d] = pow2_axis(kf - kFineBits);
    L.unit[d] = std::ldexp(1.0, kFineBits - kf);
    L.origin[d] = origin[d];
  }
  L.aniso = 0;
  L.open_frame = nullptr;
}

void make_device_frame(ForceLaunch& L, const long long* words) {
  make_fixed_frame(L);
  L.open_frame = words;
}

void host_open_frame(const double* mn, const double* mx, int* kf, long long* origin) {
  long long k;
  open_frame_from_bounds(mn, mx, &k, origin);
  *kf = (int)k;
}

cudaError_t launch_fixed_image(const ForceLaunch& L, cudaStream_t s) {
  const int n = L.csr.n;
  if (n == 0) return cudaSuccess;
  const int blocks = (n + 255) / 256;
  float4* acc = reinterpret_cast<float4*>(L.fscratch);
  const int acc_len = acc ? (L.precision == LJ_PREC_MIXED ? 2 : 1) : 0;
  const ImageFrame f0 = host_image_frame(L);
  if (L.part.soa)
    k_fixed_image<true><<<blocks, 256, 0, s>>>(L.part, n, f0, L.open_frame, L.qfix, acc, acc_len);
  else
    k_fixed_image<false><<<blocks, 256, 0, s>>>(L.part, n, f0, L.open_frame, L.qfix, acc, acc_len);
  return cudaGetLastError();
}

cudaError_t launch_open_frame_init(long long* words, cudaStream_t s) {
  k_open_frame_init<<<1, 32, 0, s>>>(reinterpret_cast<unsigned long long*>(words));
  return cudaGetLastError();
}

cudaError_t launch_open_bounds(const Particles& part, int n, long long* words, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int blocks = (n + 255) / 256;
  if (blocks > 152 * 4) blocks = 152 * 4;
  auto* w = reinterpret_cast<unsigned long long*>(words);
  if (part.soa) k_open_bounds<true><<<blocks, 256, 0, s>>>(part, n, w);
  else k_open_bounds<false><<<blocks, 256, 0, s>>>(part, n, w);
  return cudaGetLastError();
}

cudaError_t launch_force(const ForceLaunch& L, cudaStream_t s) {
  const int n = L.csr.n;
  if (n == 0) return cudaSuccess;
  const int block = L.block;
  const long long threads = (long long)n * L.lanes;
  const int blocks = (int)((threads + block - 1) / block);
  const bool pbc = L.box.on != 0, soa = L.part.soa != 0;
  const bool gather = L.method == LJ_METHOD_GATHER_FULL;
  if (L.precision == LJ_PREC_FP64) {
    if (!gather && L.kernel == 2) {
      const MixedConsts K = make_mixed_consts(L);
      // lanes per row on average: 1 -> 32 rows per warp, 2 -> 16, 4 -> 8, 8 or more -> 4
      auto go = [&](auto rows) -> cudaError_t {
        constexpr int R = decltype(rows)::value;
        const int cb = (n + R * kScatterWarps - 1) / (R * kScatterWarps);
        return dispatch_bools(pbc, soa, [&](auto P, auto S) {
          if (L.aniso)
            k_scatter_fp64_c<P.value, S.value, true, R>
                <<<cb, 32 * kScatterWarps, 0, s>>>(L.part, L.csr, L.qfix, K);
          else
            k_scatter_fp64_c<P.value, S.value, false, R>
                <<<cb, 32 * kScatterWarps, 0, s>>>(L.part, L.csr, L.qfix, K);
          return cudaGetLastError();
        });
      };
      if (L.lanes <= 1) return go(std::integral_constant<int, 32>{});
      if (L.lanes == 2) return go(std::integral_constant<int, 16>{});
      if (L.lanes == 4) return go(std::integral_constant<int, 8>{});
      return go(std::integral_constant<int, 4>{});
    }
    if (gather && L.kernel == 2) {
      const MixedConsts K = make_mixed_consts(L);
      const int cb = (n + kCompactWarps - 1) / kCompactWarps;
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        if (L.aniso)
          k_gather_fp64_c<P.value, S.value, true>
              <<<cb, 32 * kCompactWarps, 0, s>>>(L.part, L.csr, L.qfix, K);
        else
          k_gather_fp64_c<P.value, S.value, false>
              <<<cb, 32 * kCompactWarps, 0, s>>>(L.part, L.csr, L.qfix, K);
        return cudaGetLastError();
      });
    }
    const Fp64Consts K = make_fp64_consts(L.box, L.dt, L.cl2);
    return dispatch_lanes(L.lanes, [&](auto g) {
      return dispatch_bools(pbc, soa, [&](auto P, auto S) {
        constexpr int G = decltype(g)::value;
        if (gather)
          k_gather_fp64<G, P.value, S.value><<<blocks, block, 0, s>>>(L.part, L.csr, K);
        else
          k_scatter_fp64<G, P.value, S.value><<<blocks, block, 0, s>>>(L.part, L.csr, K);
        return cudaGetLastError();
      });
    });
  }
  const MixedConsts K = make_mixed_consts(L);
  if (L.precision == LJ_PREC_MIXED)  // two-float pair terms
    return gather ? launch_mixed_ff_gather(L, K, s) : launch_mixed_ff_scatter(L, K, s);
  return launch_mixed_fp32(L, K, s);
}

cudaError_t launch_fixed_image_sorted(const ForceLaunch& L, const int32_t* order, int4* cq,
                                      cudaStream_t s) {
  const int n = L.csr.n;
  if (n == 0) return cudaSuccess;
  const int blocks = (n + 255) / 256;
  const ImageFrame f0 = host_image_frame(L);
  if (L.part.soa)
    k_fixed_image_sorted<true><<<blocks, 256, 0, s>>>(L.part, n, order, f0, L.open_frame, cq);
  else
    k_fixed_image_sorted<false><<<blocks, 256, 0, s>>>(L.part, n, order, f0, L.open_frame, cq);
  return cudaGetLastError();
}

cudaError_t launch_partition_near(const ForceLaunch& L, const Csr& in, int32_t* out, int32_t* nn,
                                  const int32_t* guard, cudaStream_t s) {
  if (in.n == 0) return cudaSuccess;
  const MixedConsts K = make_mixed_consts(L);
  // one warp per row, capped near a few resident waves (grid-stride rows)
  const int blocks = (int)std::min<long long>(((long long)in.n * 32 + 127) / 128, 152 * 16);
  if (L.box.on) {
    if (L.aniso) k_partition_near<true, true><<<blocks, 128, 0, s>>>(in, L.qfix, K, out, nn, guard);
    else k_partition_near<true, false><<<blocks, 128, 0, s>>>(in, L.qfix, K, out, nn, guard);
  } else {
    k_partition_near<false, false><<<blocks, 128, 0, s>>>(in, L.qfix, K, out, nn, guard);
  }
  return cudaGetLastError();
}

cudaError_t launch_force_pairs(const Particles& part, int n, const int32_t* ip,
                               const int32_t* jp, int64_t npairs, const Periodic& box,
                               double dt, double cl2, cudaStream_t s) {
  (void)n;
  if (npairs == 0) return cudaSuccess;
  const Fp64Consts K = make_fp64_consts(box, dt, cl2);
  long long blocks = (npairs + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (box.on) k_pairs_fp64<true><<<(int)blocks, 256, 0, s>>>(part, ip, jp, npairs, K);
  else k_pairs_fp64<false><<<(int)blocks, 256, 0, s>>>(part, ip, jp, npairs, K);
  return cudaGetLastError();
}

}  // namespace ljg
