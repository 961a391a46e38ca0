"""The CPU oracle against the reference's known answers and golden vectors.

Pins: the C++ standard's known answers for the Mersenne twisters, the
reference's ref_data golden prints (cpu_ref/force_aos.cpp:622-630 format), and
fixtures produced by the reference's own cpu_ref routines (tests/golden/
make_golden.py).
"""
import ctypes as C
import platform

import numpy as np
import pytest

import oracle_lib as ol
from conftest import ROOT

X86 = platform.machine() in ("x86_64", "AMD64")


def _rng_state(size):
    return (C.c_uint8 * size)()


def test_mt19937_known_answers():
    # [rand.predef]: the 10000th consecutive invocation of a default-constructed
    # mt19937 yields 4123659995, of mt19937_64 9981545732273789042.
    O = ol.oracle()
    g = _rng_state(624 * 4 + 8)
    O.lj_or_mt32_seed(g, 5489)
    for _ in range(9999):
        O.lj_or_mt32_next(g)
    assert O.lj_or_mt32_next(g) == 4123659995
    g = _rng_state(312 * 8 + 8)
    O.lj_or_mt64_seed(g, 5489)
    for _ in range(9999):
        O.lj_or_mt64_next(g)
    assert O.lj_or_mt64_next(g) == 9981545732273789042


@pytest.mark.parametrize("fx", ["fixture_rho05", "fixture_rho1"])
def test_init_and_list_match_reference(fx, request):
    f = request.getfixturevalue(fx)
    density, L = f["meta"][0], f["meta"][1]
    q = ol.init_reference(density, L)
    assert np.array_equal(q, f["q"])  # positions bit for bit
    for builder in (ol.build_list, ol.build_half_brute):
        npp, ptr, lst = builder(q, 3.3)
        assert np.array_equal(npp, f["np"]) and np.array_equal(ptr, f["ptr"])
        assert np.array_equal(lst, f["list"])
    ii, jj = ol.csr_to_pairs(f["np"], f["ptr"], f["list"])
    assert np.array_equal(ii, f["i"]) and np.array_equal(jj, f["j"])


@pytest.mark.parametrize("fx", ["fixture_rho05", "fixture_rho1"])
def test_force_routines_match_reference(fx, request):
    f = request.getfixturevalue(fx)
    q, npp, ptr, lst = f["q"], f["np"], f["ptr"], f["list"]
    n = q.shape[0]
    calls = int(f["meta"][5])
    got = {
        "p_aos_sorted": ol.force_sorted_aos(q, np.zeros((n, 4)), npp, ptr, lst, calls=calls),
        "p_aos_pair": ol.force_pair_aos(q, np.zeros((n, 4)), f["i"], f["j"], calls=calls),
        "p_soa_sorted": ol.force_sorted_soa(q, np.zeros((n, 4)), npp, ptr, lst, calls=calls),
        "p_soa_pair": ol.force_pair_aos(q, np.zeros((n, 4)), f["i"], f["j"], calls=calls),
    }
    for k, p in got.items():
        ref = f[k]
        e = ol.rel_errors(p, ref)
        assert e["max_rel"] <= 1e-13, (k, e)
        if X86:  # same compiler, same flags: the restatement is the reference bit for bit
            assert np.array_equal(p[:, :3], ref[:, :3]), k
    # every reference routine (scalar, software-pipelined, AVX2, transposed,
    # interleaved) agrees with the scatter restatement to 1e-12 per particle
    base = got["p_aos_sorted"]
    for k in f:
        if k.startswith("p_"):
            assert ol.rel_errors(f[k], base)["max_rel"] <= 1e-12, k


def test_gather_full_equals_scatter_half(fixture_rho1):
    f = fixture_rho1
    q = f["q"]
    n = q.shape[0]
    fnp, fptr, flst = ol.build_list(q, 3.3, full=True)
    assert len(flst) == 2 * len(f["list"])
    g = ol.force_gather_aos(q, np.zeros((n, 4)), fnp, fptr, flst, calls=100, threads=2)
    assert ol.rel_errors(g, f["p_aos_sorted"])["max_rel"] <= 1e-12


def _golden(name):
    return (ROOT / "tests" / "golden" / name).read_text().split("\n")[:10]


@pytest.mark.parametrize("density,name", [(0.5, "ref_density0.5.dat"), (1.0, "ref_density1.dat")])
def test_reference_golden_prints(density, name):
    """The reference's own headline run: L = 50, 100 force_pair calls."""
    q = ol.init_reference(density, 50.0)
    assert q.shape[0] == {0.5: 62500, 1.0: 119164}[density]
    npp, ptr, lst = ol.build_list(q, 3.3)
    assert len(lst) == {0.5: 2268138, 1.0: 7839886}[density]
    ii, jj = ol.csr_to_pairs(npp, ptr, lst)
    p = ol.force_pair_aos(q, np.zeros_like(q), ii, jj, calls=100)
    assert ol.golden_rows(p) == _golden(name)


def test_periodic_list_cells_equal_brute():
    q, L = ol.init_fcc_periodic(4, 0.5, 0.05, seed=7)
    assert q.shape[0] == 256 and abs(L - 8.0) < 1e-12
    assert q[:, :3].min() >= 0.0 and q[:, :3].max() < L
    a = ol.build_list(q, 3.3, box=L)
    b = ol.build_half_brute(q, 3.3, box=L)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # bulk FCC at rho = 0.5 within r_s = 3.3: 4/3 pi 3.3^3 0.5 / 2 ~ 37.6 per particle
    assert 30 < len(a[2]) / q.shape[0] < 45


def test_periodic_forces_newton_third_law():
    q, L = ol.init_fcc_periodic(4, 1.0, 0.05, seed=11)
    npp, ptr, lst = ol.build_list(q, 3.3, box=L)
    p = ol.force_sorted_aos(q, np.zeros_like(q), npp, ptr, lst, dt=0.005, box=L)
    assert np.abs(p[:, :3].sum(axis=0)).max() < 1e-12
    fnp, fptr, flst = ol.build_list(q, 3.3, box=L, full=True)
    g = ol.force_gather_aos(q, np.zeros_like(q), fnp, fptr, flst, dt=0.005, box=L)
    assert ol.rel_errors(g, p)["max_rel"] <= 1e-12


def test_row_range_list_and_gather_equal_the_full_ones():
    """build_rows / force_gather_rows_aos (the CPU timing sample of the large
    system) give the rows and forces of the whole-system list and gather."""
    q, L = ol.init_fcc_periodic(5, 1.0, 0.05, seed=3)
    fnp, fptr, flst = ol.build_list(q, 3.3, box=L, full=True)
    g = ol.force_gather_aos(q, np.zeros_like(q), fnp, fptr, flst, dt=0.005, box=L)
    for r0, r1 in ((0, 37), (123, 500), (0, q.shape[0])):
        npp, ptr, lst = ol.build_rows(q, 3.3, r0, r1, box=L, full=True)
        assert np.array_equal(npp, fnp[r0:r1])
        assert np.array_equal(lst, flst[fptr[r0]:fptr[r0] + len(lst)])
        assert np.array_equal(ptr, fptr[r0:r1] - fptr[r0])
        p = ol.force_gather_rows_aos(q, np.zeros_like(q), r0, npp, ptr, lst, dt=0.005, box=L,
                                     threads=2)
        assert np.array_equal(p[r0:r1], g[r0:r1])
        assert not p[:r0].any() and not p[r1:].any()


@pytest.mark.skipif(not ol.ref_available(), reason="reference cpu_ref not built here (x86 only)")
def test_oracle_bitwise_vs_compiled_reference_random_input():
    """Random positions (not the lattice) through the reference's makepair /
    force_sorted and through the oracle: identical bits."""
    import multiprocessing as mp
    import sys
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import run_reference
    rng = np.random.default_rng(3)
    q = np.zeros((400, 4))
    q[:, :3] = rng.uniform(0.0, 9.0, size=(400, 3))
    res = run_reference("aos", q, 9.0)
    npp, ptr, lst = ol.build_list(q, 3.3)
    assert np.array_equal(lst, res["list"]) and np.array_equal(npp, res["np"])
    p = ol.force_sorted_aos(q, np.zeros_like(q), npp, ptr, lst, calls=3)
    # cpu_ref ran 100 calls; compare per-call linearity instead: rerun 100
    p100 = ol.force_sorted_aos(q, np.zeros_like(q), npp, ptr, lst, calls=100)
    assert np.array_equal(p100[:, :3], res["p_aos_sorted"][:, :3])
    assert np.isfinite(p).all()
