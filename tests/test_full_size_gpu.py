"""Parity and invariants at the benchmark sizes: 108,000 particles at rho = 1
and 0.5 (FCC 30^3 x 4), 1,000,188 and 8,001,504 particles (FCC 63^3 x 4 and
126^3 x 4, rho = 1), cutoff 3.0, search 3.3, periodic, jitter U[-0.05, 0.05)
from mt19937_64(20240601).

At 108k and 1M particles the oracle (cell-list build and force_sorted,
cpu_ref/force_aos.cpp:100-140 and :192-224 restated) finishes in seconds, so
the device-built list is compared entry by entry and the forces against the
oracle's.  At 8M particles only size-independent properties are checked:
* the full list has exactly twice the entries of the half list;
* FP64 scatter over the half list equals FP64 gather over the full list
  (different kernels and lists, one physics) within 1e-12, so no pair is
  missing from either list;
* the half-list scatter conserves momentum: sum_i dp_i = 0 to rounding;
* the mixed paths are within their tolerances of the FP64 path (two-float
  pair terms: the per-particle bar max_i |dF_i| / |F_i| <= 1e-5);
* the kick is linear in dt: a call at 2 dt gives twice the kick (dt enters
  as an exact power-of-two scale, and the gathers sum in a fixed order).
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

RC2, RS, DT, SEED = 9.0, 3.3, 0.005, 20240601
FP64_TOL = 1e-12
# two-float pair terms: per particle max |dF_i| / |F_i|, and max |dF_i| / rms|F|
MIXED_TOL = {"max_rel": 1e-5, "max_rel_rms": 1e-6}
# FP32 pair terms: normalised bars only
FP32_TOL = {"max_rel_rms": 1e-5, "global_rel": 2e-6}
TOL = {"mixed": MIXED_TOL, "mixed_fp32": FP32_TOL}


def _check(e, prec, *where):
    for k, tol in TOL[prec].items():
        assert e[k] <= tol, (where, prec, k, e)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _kick(engine, ctx, qd, L, precision, method, dt=DT):
    import torch
    pd = torch.zeros_like(qd)
    ctx.force_aos(qd, pd, engine.make_opts(dt=dt, cl2=RC2, box=L, precision=precision,
                                           method=method))
    torch.cuda.synchronize()
    return pd.cpu().numpy()


def _momentum_residual(p):
    """|sum_i dp_i| relative to sum_i |dp_i| (dp = p: every call starts at 0)."""
    return float(np.linalg.norm(p[:, :3].sum(axis=0)) / np.abs(p[:, :3]).sum())


@pytest.mark.parametrize("rho", [1.0, 0.5])
def test_108k_particles_against_the_oracle(engine, rho):
    """The force benchmarks' systems (108,000 particles, rho = 1 and 0.5):
    the device-built list entry by entry, every FP64 path within 1e-12 of the
    oracle per particle, both mixed paths within their bars, in AoS and SoA."""
    import torch
    q, L = ol.init_fcc_periodic(30, rho, 0.05, SEED)
    n = q.shape[0]
    assert n == 108000
    half = ol.build_list(q, RS, box=L)
    ref = ol.force_sorted_aos(q, np.zeros_like(q), *half, cl2=RC2, dt=DT, box=L)
    with engine.Context(0) as ctx:
        qd = _dev(q)
        ctx.build_list(qd, RS, box=L)
        for a, b in zip(ctx.get_list_csr("half"), half):
            assert np.array_equal(a, b)
        qs = [_dev(q[:, d].copy()) for d in range(3)]
        for prec in ("fp64", "mixed", "mixed_fp32"):
            for method in ("gather", "scatter"):
                for layout in ("aos", "soa"):
                    opts = engine.make_opts(dt=DT, cl2=RC2, box=L, precision=prec,
                                            method=method)
                    if layout == "aos":
                        pd = torch.zeros_like(qd)
                        ctx.force_aos(qd, pd, opts)
                        p = pd.cpu().numpy()
                    else:
                        ps = [torch.zeros(n, dtype=torch.float64, device="cuda")
                              for _ in range(3)]
                        ctx.force_soa(*qs, *ps, opts)
                        p = np.zeros_like(q)
                        for d in range(3):
                            p[:, d] = ps[d].cpu().numpy()
                    e = ol.rel_errors(p, ref)
                    if prec == "fp64":
                        assert e["max_rel"] <= FP64_TOL, (method, layout, e)
                    else:
                        _check(e, prec, method, layout)


def test_one_million_particles_against_the_oracle(engine):
    q, L = ol.init_fcc_periodic(63, 1.0, 0.05, SEED)
    n = q.shape[0]
    assert n == 1000188
    half = ol.build_list(q, RS, box=L, cap=90 * n)
    ref = ol.force_sorted_aos(q, np.zeros_like(q), *half, cl2=RC2, dt=DT, box=L)
    with engine.Context(0) as ctx:
        qd = _dev(q)
        ctx.build_list(qd, RS, box=L)
        got = ctx.get_list_csr("half")
        for a, b in zip(got, half):
            assert np.array_equal(a, b)
        _, e_full, _ = ctx.list_info("full")
        assert e_full == 2 * len(half[2])
        for method in ("scatter", "gather"):
            p = _kick(engine, ctx, qd, L, "fp64", method)
            e = ol.rel_errors(p, ref)
            assert e["max_rel"] <= FP64_TOL, (method, e)
            if method == "scatter":
                assert _momentum_residual(p) < 1e-12
        for prec in ("mixed", "mixed_fp32"):
            for method in ("gather", "scatter"):
                p = _kick(engine, ctx, qd, L, prec, method)
                _check(ol.rel_errors(p, ref), prec, method)


def test_eight_million_particles_invariants(engine):
    import torch
    q, L = engine.init_fcc(126, 1.0, 0.05, SEED)
    n = q.shape[0]
    assert n == 8001504
    with engine.Context(0) as ctx:
        qd = _dev(q)
        ctx.build_list(qd, RS, box=L)
        _, e_half, _ = ctx.list_info("half")
        _, e_full, _ = ctx.list_info("full")
        assert e_full == 2 * e_half
        # the jittered FCC lattice at rho = 1 has ~70.9 half partners within 3.3
        # (1M: 70,903,484 pairs); a uniform fluid would have (2 pi / 3) rho rs^3 = 75.3
        assert 68 * n < e_half < 74 * n

        scat = _kick(engine, ctx, qd, L, "fp64", "scatter")
        gath = _kick(engine, ctx, qd, L, "fp64", "gather")
        e = ol.rel_errors(gath, scat)
        assert e["max_rel"] <= FP64_TOL, e
        assert _momentum_residual(scat) < 1e-12

        gath2 = _kick(engine, ctx, qd, L, "fp64", "gather", dt=2 * DT)
        assert ol.rel_errors(gath2, 2 * gath)["max_rel"] <= 1e-15

        for prec in ("mixed", "mixed_fp32"):
            mixed = _kick(engine, ctx, qd, L, prec, "gather")
            _check(ol.rel_errors(mixed, scat), prec)
            mixed2 = _kick(engine, ctx, qd, L, prec, "gather", dt=2 * DT)
            assert ol.rel_errors(mixed2, 2 * mixed)["max_rel"] <= 1e-15, prec
        del qd
    torch.cuda.empty_cache()
