"""Parity of the CUDA force path with the oracle, through the C ABI.

FP64 path: <= 1e-12 relative per particle (norm of the 3-vector) against the
oracle's force_sorted (cpu_ref/force_aos.cpp:192-224 restated).
Mixed paths: one force evaluation against the FP64 oracle:
  "mixed" (two-float pair terms): the per-particle bar max_i |dF_i|/|F_i|
  <= 1e-5 (MIXED_TOL, with a tighter bound on the normalised error);
  "mixed_fp32" (single FP32 pair terms): normalised bars only (FP32_TOL).
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
# one two-float force evaluation vs FP64: max |dF_i| / |F_i| per particle, and
# max |dF_i| / rms|F|
MIXED_TOL = {"max_rel": 1e-5, "max_rel_rms": 1e-6}
# one FP32-pair-term evaluation vs FP64: max |dF_i| / rms|F| and ||dF|| / ||F||
FP32_TOL = {"max_rel_rms": 1e-5, "global_rel": 2e-6}
TOL = {"mixed": MIXED_TOL, "mixed_fp32": FP32_TOL}
MIXED_PRECS = list(TOL)


def check_mixed(e, prec, *where):
    for k, tol in TOL[prec].items():
        assert e[k] <= tol, (where, prec, k, e)


def _torch():
    import torch
    return torch


def dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    _torch().cuda.synchronize()
    return t.cpu().numpy()


SYSTEMS = {
    # name: (builder, box)
    "open_rho0.5": lambda: (ol.init_reference(0.5, 10.0), None),
    "open_rho1": lambda: (ol.init_reference(1.0, 8.0), None),
    "pbc_rho1": lambda: ol.init_fcc_periodic(6, 1.0, 0.05, seed=20240601),
    "pbc_rho0.5": lambda: ol.init_fcc_periodic(5, 0.5, 0.05, seed=99),
}


def system(name):
    q, box = SYSTEMS[name]()
    half = ol.build_list(q, 3.3, box=box)
    return q, box, half


def run_engine(engine, q, half, box, precision, method, layout, calls, dt, lanes=0, ctx=None,
               kernel=0, unroll=0, ff_all=False):
    own = ctx is None
    ctx = ctx or engine.Context(0)
    try:
        npp, ptr, lst = half
        ctx.set_list_csr(dev(npp), dev(ptr), dev(lst), kind="half")
        opts = engine.make_opts(dt=dt, cl2=9.0, box=box, precision=precision, method=method,
                                lanes=lanes, kernel=kernel, unroll=unroll, ff_all=ff_all)
        if layout == "aos":
            qd, pd = dev(q), dev(np.zeros_like(q))
            for _ in range(calls):
                ctx.force_aos(qd, pd, opts)
            return host(pd)
        qs = [dev(q[:, d].copy()) for d in range(3)]
        ps = [dev(np.zeros(q.shape[0])) for _ in range(3)]
        for _ in range(calls):
            ctx.force_soa(*qs, *ps, opts)
        out = np.zeros_like(q)
        for d in range(3):
            out[:, d] = host(ps[d])
        return out
    finally:
        if own:
            ctx.close()


def oracle_p(q, half, box, calls, dt):
    return ol.force_sorted_aos(q, np.zeros_like(q), *half, dt=dt, box=box, calls=calls)


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("method,kernel", [("scatter", 1), ("scatter", 2), ("gather", 1),
                                           ("gather", 2)])
@pytest.mark.parametrize("layout", ["aos", "soa"])
def test_fp64_matches_oracle(engine, name, method, kernel, layout):
    q, box, half = system(name)
    dt = 0.001 if box is None else 0.005
    ref = oracle_p(q, half, box, 10, dt)
    got = run_engine(engine, q, half, box, "fp64", method, layout, 10, dt, kernel=kernel)
    e = ol.rel_errors(got, ref)
    assert e["max_rel"] <= FP64_TOL, e


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_fp64_every_lane_width(engine, lanes):
    q, box, half = system("pbc_rho1")
    ref = oracle_p(q, half, box, 1, 0.005)
    for method in ("scatter", "gather"):
        got = run_engine(engine, q, half, box, "fp64", method, "aos", 1, 0.005, lanes=lanes)
        assert ol.rel_errors(got, ref)["max_rel"] <= FP64_TOL, (method, lanes)


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("method,kernel", [("gather", 1), ("gather", 2), ("scatter", 1),
                                           ("scatter", 2)])
@pytest.mark.parametrize("layout", ["aos", "soa"])
@pytest.mark.parametrize("prec", MIXED_PRECS)
def test_mixed_error_bounds(engine, name, method, kernel, layout, prec):
    q, box, half = system(name)
    dt = 0.005
    ref = oracle_p(q, half, box, 1, dt)
    got = run_engine(engine, q, half, box, prec, method, layout, 1, dt, kernel=kernel)
    check_mixed(ol.rel_errors(got, ref), prec, name, method, kernel, layout)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_mixed_every_lane_width(engine, lanes):
    q, box, half = system("pbc_rho1")
    ref = oracle_p(q, half, box, 1, 0.005)
    # two-float pair terms take 2 or 4 entries in flight per lane
    cases = {"mixed": (("gather", 1, [0]), ("gather", 2, [2, 4]), ("scatter", 2, [2, 4])),
             "mixed_fp32": (("gather", 1, [0]), ("gather", 2, [2, 4, 8]),
                            ("scatter", 2, [1, 2, 4, 8]))}
    for prec, runs in cases.items():
        for method, kernel, unrolls in runs:
            for unroll in unrolls:
                got = run_engine(engine, q, half, box, prec, method, "aos", 1, 0.005,
                                 lanes=lanes, kernel=kernel, unroll=unroll)
                check_mixed(ol.rel_errors(got, ref), prec, method, kernel, unroll)


def test_mixed_anisotropic_box(engine):
    q, L = ol.init_fcc_periodic(6, 1.0, 0.05, seed=5)
    box = np.array([L, L * 1.25, L * 0.9])
    q = q.copy()
    q[:, 1] *= 1.25
    q[:, 2] *= 0.9
    half = ol.build_list(q, 3.3, box=box)
    ref = oracle_p(q, half, box, 1, 0.005)
    for method in ("gather", "scatter"):
        for prec in MIXED_PRECS:
            got = run_engine(engine, q, half, box, prec, method, "aos", 1, 0.005)
            check_mixed(ol.rel_errors(got, ref), prec, method)
        got64 = run_engine(engine, q, half, box, "fp64", method, "aos", 1, 0.005)
        assert ol.rel_errors(got64, ref)["max_rel"] <= FP64_TOL


def planted_pairs(shift=0.0, spacing=12.0, g=8, seed=1, box=None):
    """g^3 isolated pairs at r2 within a few ulp of CL2 = 9, their centres
    `spacing` apart and shifted by `shift`; with a box the grid fills it and
    the pairs straddle its faces where the grid meets them."""
    rng = np.random.default_rng(seed)
    centres = np.stack(np.meshgrid(*[np.arange(g) * spacing] * 3, indexing="ij"),
                       -1).reshape(-1, 3) + shift
    m = centres.shape[0]
    dirs = rng.normal(size=(m, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    r = 3.0 * (1 + rng.integers(-6, 7, size=m) * 2.0 ** -52)
    q = np.zeros((2 * m, 4))
    q[0::2, :3] = centres
    q[1::2, :3] = centres + dirs * r[:, None]
    if box is not None:
        q[:, :3] = np.mod(q[:, :3], box)
    return q


def check_planted_mask(engine, q, box):
    """Every planted pair is masked as the reference's FP64 arithmetic masks
    it (a toggled pair would change F by |f(rc)| ~ 1e-2, i.e. 100 %), and the
    forces meet the bars."""
    half = ol.build_list(q, 3.3, box=box)
    assert len(half[2]) == q.shape[0] // 2
    ref = oracle_p(q, half, box, 1, 0.005)
    inside = np.linalg.norm(ref[:, :3], axis=1) > 0
    assert 0 < inside.sum() < q.shape[0]  # both sides of the surface are exercised
    for prec in MIXED_PRECS:
        for method, kernel in (("gather", 1), ("gather", 2), ("scatter", 1), ("scatter", 2)):
            got = run_engine(engine, q, half, box, prec, method, "aos", 1, 0.005,
                             kernel=kernel)
            assert np.array_equal(np.linalg.norm(got[:, :3], axis=1) > 0, inside), \
                (prec, method, kernel)
            assert ol.rel_errors(got, ref)["max_rel"] <= 1e-5, (prec, method, kernel)
    for method in ("gather", "scatter"):
        for kernel in (1, 2):
            got64 = run_engine(engine, q, half, box, "fp64", method, "aos", 1, 0.005,
                               kernel=kernel)
            assert ol.rel_errors(got64, ref)["max_rel"] <= FP64_TOL, (method, kernel)


def test_cutoff_boundary_pairs_follow_fp64_mask(engine):
    check_planted_mask(engine, planted_pairs(), None)


@pytest.mark.parametrize("shift", [1e3, 1e4, 1e5, -1e5])
def test_cutoff_mask_at_large_open_coordinates(engine, shift):
    """The planted pairs far from the origin: the open frame's quantum follows
    the system's extent (per-axis origin at the minimum coordinate), so the
    mask and the forces do not depend on where the system sits."""
    check_planted_mask(engine, planted_pairs(shift=shift), None)


def test_cutoff_mask_in_a_large_periodic_box(engine):
    """A periodic box of L = 5000 (coarse quantum L / 2^32 = 1.2e-6): pairs
    on a grid that fills the box, some straddling its faces."""
    L = 5000.0
    q = planted_pairs(spacing=L / 16, g=16, seed=3, box=L)
    check_planted_mask(engine, q, L)


def test_stateless_drop_in(engine):
    q, box, half = system("open_rho1")
    full = ol.build_list(q, 3.3, full=True)
    ref = oracle_p(q, half, None, 3, 0.001)
    for kind, (npp, ptr, lst) in (("half", half), ("full", full)):
        qd, pd = dev(q), dev(np.zeros_like(q))
        for _ in range(3):
            engine.force_csr_fp64_aos(qd, pd, 0.001, 9.0, dev(lst), dev(npp), dev(ptr),
                                      kind=kind)
        assert ol.rel_errors(host(pd), ref)["max_rel"] <= FP64_TOL, kind


def test_force_pair_entry(engine, fixture_rho05):
    f = fixture_rho05
    qd, pd = dev(f["q"]), dev(np.zeros_like(f["q"]))
    ii, jj = dev(f["i"]), dev(f["j"])
    for _ in range(100):
        engine.force_pairs_fp64_aos(qd, pd, 0.001, 9.0, ii, jj)
    assert ol.rel_errors(host(pd), f["p_aos_pair"])["max_rel"] <= FP64_TOL


@pytest.mark.parametrize("fx", ["fixture_rho05", "fixture_rho1"])
def test_reference_fixtures(engine, fx, request):
    """Engine vs the reference's own cpu_ref outputs (100 calls, dt = 0.001)."""
    f = request.getfixturevalue(fx)
    half = (f["np"], f["ptr"], f["list"])
    for layout, key in (("aos", "p_aos_sorted"), ("soa", "p_soa_sorted")):
        for method in ("scatter", "gather"):
            got = run_engine(engine, f["q"], half, None, "fp64", method, layout, 100, 0.001)
            assert ol.rel_errors(got, f[key])["max_rel"] <= FP64_TOL, (layout, method)


def test_full_list_expansion_is_reference_full_list(engine):
    q, box, half = system("pbc_rho0.5")
    full = ol.build_list(q, 3.3, box=box, full=True)
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]), kind="half")
        got = ctx.get_list_csr("full")
        for a, b in zip(got, full):
            assert np.array_equal(a, b)
        back = ctx.get_list_csr("half")
        for a, b in zip(back, half):
            assert np.array_equal(a, b)
        assert ctx.list_info("full")[2] == int(full[0].max())


def test_set_pairs_is_sortpair(engine, fixture_rho1):
    f = fixture_rho1
    n = f["q"].shape[0]
    with engine.Context(0) as ctx:
        for where in ("device", "host"):
            ii, jj = (dev(f["i"]), dev(f["j"])) if where == "device" else (f["i"], f["j"])
            ctx.set_list_pairs(n, ii, jj)
            got = ctx.get_list_csr("half")
            for a, b in zip(got, (f["np"], f["ptr"], f["list"])):
                assert np.array_equal(a, b), where
        # unsorted pair array: rows keep pair-array order (stable), as sortpair
        rng = np.random.default_rng(0)
        perm = rng.permutation(len(f["i"]))
        ii, jj = f["i"][perm].copy(), f["j"][perm].copy()
        order = np.argsort(ii, kind="stable")
        for src in ((dev(ii), dev(jj)), (ii, jj)):
            ctx.set_list_pairs(n, *src)
            npp, ptr, lst = ctx.get_list_csr("half")
            assert np.array_equal(npp, f["np"]) and np.array_equal(lst, jj[order])


def test_bad_lists_are_rejected(engine):
    q, box, half = system("open_rho0.5")
    npp, ptr, lst = half
    n = len(npp)
    with engine.Context(0) as ctx:
        with pytest.raises(engine.LJError) as e:
            ctx.force_aos(dev(q), dev(np.zeros_like(q)), engine.make_opts())
        assert e.value.status == engine.LJ_ERR_NO_LIST
        bad = lst.copy()
        bad[17] = n  # out of range j
        with pytest.raises(engine.LJError) as e:
            ctx.set_list_csr(dev(npp), dev(ptr), dev(bad))
        assert e.value.status == engine.LJ_ERR_BAD_LIST and "sorted_list[17]" in str(e.value)
        badn = npp.copy()
        badn[3] = -1
        with pytest.raises(engine.LJError) as e:
            ctx.set_list_csr(badn, ptr, lst)  # host arrays
        assert e.value.status == engine.LJ_ERR_BAD_LIST
        badp = ptr.copy()
        badp[0] = len(lst) - 1  # row 0 (np > 1) runs past the end
        with pytest.raises(engine.LJError) as e:
            ctx.set_list_csr(dev(npp), dev(badp), dev(lst))
        assert e.value.status == engine.LJ_ERR_BAD_LIST
        ctx.set_list_csr(dev(npp), dev(ptr), dev(lst))
        with pytest.raises(engine.LJError) as e:  # n mismatch
            ctx.force_aos(dev(q[:-1]), dev(np.zeros_like(q[:-1])), engine.make_opts())
        assert e.value.status == engine.LJ_ERR_INVALID_ARGUMENT
        with pytest.raises(engine.LJError):  # cutoff larger than half the box
            ctx.force_aos(dev(q), dev(np.zeros_like(q)), engine.make_opts(box=5.0))


def test_edge_cases(engine):
    rng = np.random.default_rng(4)
    # empty system, rows with np = 0, a single long row (> 1024 partners)
    with engine.Context(0) as ctx:
        e0 = np.zeros(0, np.int32)
        ctx.set_list_csr(e0, e0, e0, kind="half")
        ctx.force_aos(dev(np.zeros((0, 4))), dev(np.zeros((0, 4))), engine.make_opts())
    n = 3000
    q = np.zeros((n, 4))
    q[0, :3] = 20.0
    q[1:, :3] = 20.0 + rng.normal(scale=1.6, size=(n - 1, 3))
    npp = np.zeros(n, np.int32)
    npp[0] = n - 1
    ptr = np.full(n, n - 1, np.int32)
    ptr[0] = 0
    lst = np.arange(1, n, dtype=np.int32)
    half = (npp, ptr, lst)
    ref = oracle_p(q, half, None, 1, 0.001)
    for prec in ("fp64", "mixed", "mixed_fp32"):
        for method, kernel in (("scatter", 1), ("scatter", 2), ("gather", 1), ("gather", 2)):
            got = run_engine(engine, q, half, None, prec, method, "aos", 1, 0.001, kernel=kernel)
            e = ol.rel_errors(got, ref)
            if prec == "fp64":
                assert e["max_rel"] <= FP64_TOL, (method, e)
            elif prec == "mixed":
                check_mixed(e, prec, method, kernel)
            else:
                assert e["max_rel_rms"] <= 1e-4, (method, e)


def test_measure_host_buffers(engine, fixture_rho05):
    f = fixture_rho05
    with engine.Context(0) as ctx:
        ctx.set_list_csr(f["np"], f["ptr"], f["list"])  # host list, re-uploaded per measure
        p = np.zeros_like(f["q"])
        t_all, t_calc = ctx.measure_aos(np.ascontiguousarray(f["q"]), p, engine.make_opts(),
                                        calls=100)
        assert t_all >= t_calc > 0
        assert ol.rel_errors(p, f["p_aos_sorted"])["max_rel"] <= FP64_TOL


def test_golden_print_density05(engine):
    """The reference's headline case end to end on the GPU: N = 62,500, 100 calls."""
    q = ol.init_reference(0.5, 50.0)
    half = ol.build_list(q, 3.3)
    got = run_engine(engine, q, half, None, "fp64", "scatter", "aos", 100, 0.001)
    gold = [[float(v) for v in r.split()] for r in
            (ol.ROOT / "tests" / "golden" / "ref_density0.5.dat").read_text().split("\n")[:10]]
    rows = [[float(v) for v in r.split()] for r in ol.golden_rows(got)]
    assert np.abs(np.array(rows) - np.array(gold)).max() <= 1.5e-10


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_device_list_build_is_reference_list(engine, name):
    q, box, half = system(name)
    full = ol.build_list(q, 3.3, box=box, full=True)
    with engine.Context(0) as ctx:
        ctx.build_list(dev(q), 3.3, box=box)
        for kind, want in (("half", half), ("full", full)):
            got = ctx.get_list_csr(kind)
            for a, b in zip(got, want):
                assert np.array_equal(a, b), kind
        # and a build of one kind only
        ctx.build_list(dev(q), 3.3, box=box, kinds=("full",))
        assert ctx.list_info("half")[0] == 0
        for a, b in zip(ctx.get_list_csr("full"), full):
            assert np.array_equal(a, b)


def test_device_list_build_large_periodic(engine):
    """The headline system: 108,000 particles, rho = 0.5, L = 60."""
    q, L = ol.init_fcc_periodic(30, 0.5, 0.05, seed=20240601)
    half = ol.build_list(q, 3.3, box=L)
    with engine.Context(0) as ctx:
        ctx.build_list(dev(q), 3.3, box=L)
        got = ctx.get_list_csr("half")
        for a, b in zip(got, half):
            assert np.array_equal(a, b)


def test_non_compact_list_layout(engine):
    """Rows stored out of order with gaps between them (a valid CSR that is not
    compact): every kernel sees the same pairs as with the compact list."""
    q, box, half = system("pbc_rho0.5")
    npp, ptr, lst = half
    n = len(npp)
    rng = np.random.default_rng(8)
    order = rng.permutation(n)
    gap = 3
    new_ptr = np.zeros(n, np.int32)
    chunks, pos = [], 0
    for i in order:
        new_ptr[i] = pos
        chunks.append(lst[ptr[i]:ptr[i] + npp[i]])
        chunks.append(np.full(gap, -7 % n, np.int32))  # junk between rows
        pos += npp[i] + gap
    big = np.concatenate(chunks).astype(np.int32)
    ref = oracle_p(q, half, box, 1, 0.005)
    for method, kernel in (("scatter", 1), ("scatter", 2), ("gather", 1), ("gather", 2)):
        got = run_engine(engine, q, (npp, new_ptr, big), box, "fp64", method, "aos", 1, 0.005,
                         kernel=kernel)
        assert ol.rel_errors(got, ref)["max_rel"] <= FP64_TOL, (method, kernel)
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(npp), dev(new_ptr), dev(big))
        for a, b in zip(ctx.get_list_csr("half"), half):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["mixed", "mixed_fp32", "fp64"])
def test_autotune_picks_a_valid_shape_and_keeps_results(engine, prec):
    q, box, half = system("pbc_rho1")
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        npp, ptr, lst = half
        ctx.set_list_csr(dev(npp), dev(ptr), dev(lst))
        qd = dev(q)
        opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision=prec)
        best, ms = ctx.autotune(qd, opts, reps=2)
        assert ms > 0 and best.method in (1, 2) and best.kernel in (1, 2, 3, 4, 5)
        # the tuned shape is used by default-option calls and keeps parity
        for o in (opts, best):
            pd = dev(np.zeros_like(q))
            ctx.force_aos(qd, pd, o)
            e = ol.rel_errors(host(pd), ref)
            if prec == "fp64":
                assert e["max_rel"] <= FP64_TOL, e
            else:
                check_mixed(e, prec, o.kernel)


def test_interleaved_z_layout(engine):
    """force_sorted_z's interleaved z[N][8] = {q.xyzw, p.xyzw} records."""
    q, box, half = system("pbc_rho1")
    ref = oracle_p(q, half, box, 3, 0.005)
    z = np.zeros((q.shape[0], 8))
    z[:, :4] = q
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]))
        for prec in ("fp64", "mixed", "mixed_fp32"):
            zd = dev(z)
            for _ in range(3):
                ctx.force_z(zd, engine.make_opts(dt=0.005, cl2=9.0, box=box, precision=prec))
            out = host(zd)
            assert np.array_equal(out[:, :4], q)  # positions untouched
            e = ol.rel_errors(out[:, 4:8], ref)
            if prec == "fp64":
                assert e["max_rel"] <= FP64_TOL, e
            else:
                check_mixed(e, prec)


def test_transposed_list_round_trip(engine):
    """The reference's transposed layout list[i + k N] in and out."""
    q, box, half = system("pbc_rho0.5")
    full = ol.build_list(q, 3.3, box=box, full=True)
    n = q.shape[0]
    npp, ptr, lst = full
    width = n
    ell = np.zeros(int(npp.max()) * width, np.int32)
    for i in range(n):
        ell[i + np.arange(npp[i]) * width] = lst[ptr[i]:ptr[i] + npp[i]]
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        ctx.set_list_ell(dev(npp), dev(ell), width, kind="full")
        for a, b in zip(ctx.get_list_csr("full"), full):
            assert np.array_equal(a, b)
        np2, ell2 = ctx.get_list_ell(width)
        assert np.array_equal(np2, npp) and np.array_equal(ell2, ell)
        pd = dev(np.zeros_like(q))
        ctx.force_aos(dev(q), pd, engine.make_opts(dt=0.005, cl2=9.0, box=box))
        assert ol.rel_errors(host(pd), ref)["max_rel"] <= FP64_TOL
        bad = ell.copy()
        with pytest.raises(engine.LJError):  # array too short for the rows
            ctx.set_list_ell(dev(npp), dev(bad[:width]), width, kind="full")


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("layout", ["aos", "soa"])
@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_fp32"])
def test_transposed_list_gather_kernel5(engine, name, layout, prec):
    """Kernel 5 reads the transposed copy of the full list (entry k of row i
    at [i + k n], the layout of the reference's ELL kernels): the same bits
    as the row-major list with one lane per row and the same terms (FP64:
    kernel 1; mixed: kernel 2 with every pair in its own terms), and the
    oracle's bars."""
    q, box, half = system(name)
    ref = oracle_p(q, half, box, 2, 0.005)
    unrolls = [0] if prec == "fp64" else [2, 4]
    with engine.Context(0) as ctx:
        for u in unrolls:
            got = run_engine(engine, q, half, box, prec, "gather", layout, 2, 0.005, ctx=ctx,
                             kernel=5, unroll=u)
            row = run_engine(engine, q, half, box, prec, "gather", layout, 2, 0.005, ctx=ctx,
                             kernel=1 if prec == "fp64" else 2, lanes=1, unroll=u,
                             ff_all=prec == "mixed")
            assert np.array_equal(got, row), (u, np.abs(got - row).max())
            e = ol.rel_errors(got, ref)
            if prec == "fp64":
                assert e["max_rel"] <= FP64_TOL, e
            else:
                check_mixed(e, prec, u)


def test_kernel5_options_and_lists_from_ell(engine):
    """Kernel 5 takes one lane per row and unroll 2 or 4 (mixed); a list
    installed in the transposed layout runs it too, and a new list replaces
    its transposed copy."""
    q, box, half = system("pbc_rho0.5")
    full = ol.build_list(q, 3.3, box=box, full=True)
    n = q.shape[0]
    npp, ptr, lst = full
    ell = np.zeros(int(npp.max()) * n, np.int32)
    for i in range(n):
        ell[i + np.arange(npp[i]) * n] = lst[ptr[i]:ptr[i] + npp[i]]
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        ctx.set_list_ell(dev(npp), dev(ell), n, kind="full")
        qd = dev(q)
        for prec in ("fp64", "mixed"):
            pd = dev(np.zeros_like(q))
            ctx.force_aos(qd, pd, engine.make_opts(dt=0.005, cl2=9.0, box=box, precision=prec,
                                                   kernel=5))
            e = ol.rel_errors(host(pd), ref)
            assert e["max_rel"] <= (FP64_TOL if prec == "fp64" else MIXED_TOL["max_rel"]), e
        for bad in (dict(lanes=4), dict(precision="mixed", unroll=8)):
            kw = dict(dt=0.005, cl2=9.0, box=box, kernel=5)
            kw.update(bad)
            with pytest.raises(engine.LJError):
                ctx.force_aos(qd, dev(np.zeros_like(q)), engine.make_opts(**kw))
        # another list: its own transposed copy (a stale copy would not match)
        q2, box2, half2 = system("pbc_rho1")
        ctx.set_list_csr(dev(half2[0]), dev(half2[1]), dev(half2[2]))
        pd = dev(np.zeros_like(q2))
        ctx.force_aos(dev(q2), pd, engine.make_opts(dt=0.005, cl2=9.0, box=box2, kernel=5))
        ref2 = oracle_p(q2, half2, box2, 1, 0.005)
        assert ol.rel_errors(host(pd), ref2)["max_rel"] <= FP64_TOL


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_autotune_layouts_and_cache(engine, prec, tmp_path):
    """lj_autotune over launch shapes, the transposed list and the AoS, SoA
    and z layouts: the winner keeps parity in its layout, lands in the cache
    file under the problem's key, and a second context with the same key
    takes it from the cache without timing anything."""
    q, box, half = system("pbc_rho1")
    ref = oracle_p(q, half, box, 1, 0.005)
    cache = tmp_path / "tune.txt"
    results = []
    for _ in range(2):
        with engine.Context(0) as ctx:
            ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]))
            qd = dev(q)
            opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision=prec)
            r = ctx.autotune_layouts(qd, opts, reps=1, layouts=("aos", "soa", "z"), cache=cache)
            results.append(r)
            assert r["layout"] in ("aos", "soa", "z") and r["ms"] > 0
            assert r["opts"].kernel in (1, 2, 3, 4, 5) and r["opts"].method in (1, 2)
            # the winner, called in its layout with default launch fields and
            # with its explicit shape, keeps parity
            for o in (opts, r["opts"]):
                if r["layout"] == "aos":
                    pd = dev(np.zeros_like(q))
                    ctx.force_aos(qd, pd, o)
                    got = host(pd)
                elif r["layout"] == "soa":
                    qs = [dev(q[:, d].copy()) for d in range(3)]
                    ps = [dev(np.zeros(q.shape[0])) for _ in range(3)]
                    ctx.force_soa(*qs, *ps, o)
                    got = np.stack([host(x) for x in ps] + [np.zeros(q.shape[0])], axis=1)
                else:
                    z = np.zeros((q.shape[0], 8))
                    z[:, :4] = q
                    zd = dev(z)
                    ctx.force_z(zd, o)
                    got = host(zd)[:, 4:8]
                e = ol.rel_errors(got, ref)
                if prec == "fp64":
                    assert e["max_rel"] <= FP64_TOL, e
                else:
                    check_mixed(e, prec)
    first, second = results
    assert not first["from_cache"] and first["timed"] > 3
    assert second["from_cache"] and second["timed"] == 0
    assert second["key"] == first["key"] and f"prec{engine.make_opts(precision=prec).precision}" in first["key"]
    assert second["layout"] == first["layout"]
    for f in ("method", "kernel", "lanes", "unroll", "block"):
        assert getattr(second["opts"], f) == getattr(first["opts"], f), f
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and lines[0].startswith(first["key"] + " ")
    # another density is another key: timed, and appended to the same file
    q2, box2, half2 = system("pbc_rho0.5")
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(half2[0]), dev(half2[1]), dev(half2[2]))
        r = ctx.autotune_layouts(dev(q2), engine.make_opts(dt=0.005, cl2=9.0, box=box2,
                                                           precision=prec),
                                 reps=1, layouts=("aos", "soa", "z"), cache=cache)
    assert r["key"] != first["key"] and not r["from_cache"] and r["timed"] > 3
    assert len(cache.read_text().splitlines()) == 2


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("layout", ["aos", "soa"])
def test_cell_tiled_gather_on_device_built_lists(engine, name, layout):
    """Kernel 3 (cell-tiled, 16-bit local rows, FP32 pair terms; opt-in or
    autotuned) runs once the list was built on the device; it must meet the
    FP32-term bounds, and kernels 2 and 3 must see exactly the same pairs."""
    q, box, half = system(name)
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        qd = dev(q)
        ctx.build_list(qd, 3.3, box=box)
        outs = {}
        for kernel, lanes, unroll in ((3, 0, 0), (3, 2, 2), (3, 8, 4), (2, 4, 4)):
            opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision="mixed_fp32",
                                    method="gather", kernel=kernel, lanes=lanes, unroll=unroll)
            if layout == "aos":
                pd = dev(np.zeros_like(q))
                ctx.force_aos(qd, pd, opts)
                got = host(pd)
            else:
                qs = [dev(q[:, d].copy()) for d in range(3)]
                ps = [dev(np.zeros(q.shape[0])) for _ in range(3)]
                ctx.force_soa(*qs, *ps, opts)
                got = np.zeros_like(q)
                for d in range(3):
                    got[:, d] = host(ps[d])
            check_mixed(ol.rel_errors(got, ref), "mixed_fp32", kernel, lanes, unroll)
            outs[(kernel, lanes, unroll)] = got
        # same pairs: tiled vs unrolled differ only by FP32 summation order
        # (a few 1e-6 of the rms force); one pair more or less, even at the
        # cutoff (df ~ 4e-3), would differ by orders of magnitude more
        a, b = outs[(3, 0, 0)], outs[(2, 4, 4)]
        assert ol.rel_errors(a, b)["max_rel_rms"] <= 5e-6


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("layout", ["aos", "soa"])
@pytest.mark.parametrize("prec", MIXED_PRECS)
def test_vector_index_loads_kernel4(engine, name, layout, prec):
    """Kernel 4 (kernel 2 over the 16-byte-aligned copy of the full list, one
    16-byte index load per lane and step) meets the mixed bounds and sees the
    same pairs as kernel 2 (rows of any length, including rows shorter than
    4 and empty rows of open systems)."""
    q, box, half = system(name)
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        outs = {}
        for kernel, lanes in ((4, 0), (4, 2), (4, 8), (2, 4)):
            got = run_engine(engine, q, half, box, prec, "gather", layout, 1, 0.005,
                             lanes=lanes, ctx=ctx, kernel=kernel, unroll=4)
            check_mixed(ol.rel_errors(got, ref), prec, kernel, lanes)
            outs[(kernel, lanes)] = got
        same = 1e-7 if prec == "mixed" else 5e-6  # summation order only
        assert ol.rel_errors(outs[(4, 0)], outs[(2, 4)])["max_rel_rms"] <= same


@pytest.mark.parametrize("prec", MIXED_PRECS)
def test_kernel4_measure_uses_the_uploaded_list(engine, fixture_rho05, prec):
    """lj_measure_aos re-uploads a host list and refreshes the aligned copy
    from it inside the timed region; results match the FP64 oracle's bounds."""
    f = fixture_rho05
    half = (f["np"], f["ptr"], f["list"])
    with engine.Context(0) as ctx:
        ctx.set_list_csr(*half)
        fnp, fptr, flist = ctx.get_list_csr("full")
        ctx.set_list_csr(fnp, fptr, flist, kind="full")  # host full list
        opts = engine.make_opts(dt=0.001, cl2=9.0, precision=prec, method="gather",
                                kernel=4, unroll=4)
        p = np.zeros_like(f["q"])
        ctx.measure_aos(np.ascontiguousarray(f["q"]), p, opts, calls=1)
        e = ol.rel_errors(p, ol.force_sorted_aos(f["q"], np.zeros_like(f["q"]), *half,
                                                 dt=0.001, box=None, calls=1))
        check_mixed(e, prec)


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("kernel", [2, 4])
def test_two_float_split_and_full_terms(engine, name, kernel):
    """The two-float gather's near/far split (FP32 terms beyond 2.1 sigma,
    the default) and two-float terms for every pair (ff_all) both meet the
    per-particle bar; they differ only by the far terms' FP32 rounding."""
    q, box, half = system(name)
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]), kind="half")
        out = {}
        for ff_all in (False, True):
            pd = dev(np.zeros_like(q))
            ctx.force_aos(dev(q), pd, engine.make_opts(
                dt=0.005, cl2=9.0, box=box, precision="mixed", method="gather", kernel=kernel,
                unroll=4, ff_all=ff_all))
            out[ff_all] = host(pd)
            check_mixed(ol.rel_errors(out[ff_all], ref), "mixed", name, kernel, ff_all)
        # every pair two-float: ~1e-9 of FP64
        assert ol.rel_errors(out[True], ref)["max_rel"] <= 1e-7


@pytest.mark.parametrize("lanes", [0, 2, 8, 32])
def test_split_order_from_other_positions_keeps_precision(engine, lanes):
    """The near-first order is made from the positions of the first call;
    later calls with particles moved by up to 0.45 sigma (far past the 0.1
    sigma margin of the 2.1 sigma split) still meet the per-particle bar:
    the rows whose far pairs came closer than 2.0 sigma are queued, each
    once whatever the lanes per row, and those pairs get two-float terms."""
    q, box = ol.init_fcc_periodic(6, 1.0, 0.05, seed=20240601)
    rng = np.random.default_rng(8)
    q2 = q.copy()
    q2[:, :3] = np.mod(q2[:, :3] + rng.uniform(-0.26, 0.26, size=(q.shape[0], 3)), box)
    half = ol.build_list(q, 3.9, box=box)  # covers every pair within 3.0 of q2
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]), kind="half")
        opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision="mixed",
                                method="gather", lanes=lanes)
        for pos in (q, q2, q):
            pd = dev(np.zeros_like(q))
            ctx.force_aos(dev(pos), pd, opts)
            ref = oracle_p(pos, half, box, 1, 0.005)
            check_mixed(ol.rel_errors(host(pd), ref), "mixed", "moved")


@pytest.mark.parametrize("kernel", [2, 4])
def test_l2_window_keeps_results(engine, kernel):
    """The L2 persistence window over the position image is a cache hint:
    mixed force calls give the same bits with it and without it.  It is a
    stream attribute, so a context on the default stream refuses the call
    while it is on; ratios outside [0, 1] are rejected."""
    torch = _torch()
    q, box, half = system("pbc_rho1")
    opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision="mixed", method="gather",
                            kernel=kernel, unroll=4)
    out = {}
    side = torch.cuda.Stream()
    for ratio in (0.0, 1.0, 0.5):
        with engine.Context(0) as ctx:
            ctx.set_stream(side)
            ctx.set_l2_window(ratio)
            ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]), kind="half")
            qd = dev(q)
            torch.cuda.synchronize()
            pd = torch.zeros_like(qd)
            for _ in range(2):
                ctx.force_aos(qd, pd, opts)
            side.synchronize()
            out[ratio] = pd.cpu().numpy()
    assert np.array_equal(out[0.0], out[1.0]) and np.array_equal(out[0.0], out[0.5])
    with engine.Context(0) as ctx:
        for bad in (-0.1, 1.5):
            with pytest.raises(engine.LJError) as e:
                ctx.set_l2_window(bad)
            assert e.value.status == engine.LJ_ERR_INVALID_ARGUMENT
        ctx.set_l2_window(1.0)
        ctx.set_list_csr(dev(half[0]), dev(half[1]), dev(half[2]), kind="half")
        with pytest.raises(engine.LJError) as e:
            ctx.force_aos(dev(q), dev(np.zeros_like(q)), opts)
        assert e.value.status == engine.LJ_ERR_UNSUPPORTED


def test_launch_option_checks(engine, fixture_rho05):
    f = fixture_rho05
    with engine.Context(0) as ctx:
        ctx.set_list_csr(dev(f["np"]), dev(f["ptr"]), dev(f["list"]))
        qd, pd = dev(f["q"]), dev(np.zeros_like(f["q"]))
        for kw in (dict(kernel=6), dict(kernel=-1), dict(unroll=-1),
                   dict(precision="mixed", method="gather", kernel=4, unroll=2)):
            opts = engine.make_opts(**kw)
            with pytest.raises(engine.LJError) as e:
                ctx.force_aos(qd, pd, opts)
            assert e.value.status == engine.LJ_ERR_INVALID_ARGUMENT, kw
        # two-float pair terms take 2 or 4 entries in flight per lane
        for kw in (dict(method="gather", kernel=2, unroll=8), dict(method="scatter", unroll=1)):
            with pytest.raises(engine.LJError) as e:
                ctx.force_aos(qd, pd, engine.make_opts(precision="mixed", **kw))
            assert e.value.status == engine.LJ_ERR_UNSUPPORTED, kw


@pytest.mark.parametrize("kernel", [1, 2, 4])
@pytest.mark.parametrize("prec", MIXED_PRECS)
def test_open_box_frame_follows_the_coordinates(engine, kernel, prec):
    """Open boxes take their fixed-point frame from the per-axis bounds of
    the coordinates, chosen on the device each call: translating the system
    far from the origin and back within one context keeps every call within
    the mixed bounds, for both the gather and the scatter."""
    q, box, half = system("open_rho0.5")
    with engine.Context(0) as ctx:
        npp, ptr, lst = half
        ctx.set_list_csr(dev(npp), dev(ptr), dev(lst), kind="half")
        for method in ("gather", "scatter"):
            k = 2 if method == "scatter" and kernel == 4 else kernel
            opts = engine.make_opts(dt=0.001, cl2=9.0, precision=prec, method=method,
                                    kernel=k, unroll=4 if k > 1 else 0)
            for shift in (0.0, 100.0, 1e3, 1e4, 1e5, 0.0, -37.5, -1e5):
                qs = q.copy()
                qs[:, :3] += shift
                ref = oracle_p(qs, half, None, 1, 0.001)
                pd = dev(np.zeros_like(q))
                ctx.force_aos(dev(qs), pd, opts)
                check_mixed(ol.rel_errors(host(pd), ref), prec, method, shift)


@pytest.mark.parametrize("seed", range(6))
def test_random_systems_every_path(engine, seed):
    """Random systems: a jittered FCC lattice of random size and density with
    a random subset of sites removed (particle counts that are not multiples
    of 4, a warp or a block) in a random particle order, open or periodic,
    rows sorted or shuffled (random_shfl): every FP64 path within 1e-12 of
    the oracle, every mixed path within its bounds, and the device-built list
    equal to the oracle's."""
    rng = np.random.default_rng(1000 + seed)
    ncell = int(rng.integers(3, 8))
    rho = float(rng.uniform(0.4, 1.0))
    q0, L = ol.init_fcc_periodic(ncell, rho, 0.2, seed=77 + seed)
    keep = rng.permutation(q0.shape[0])[: int(q0.shape[0] * rng.uniform(0.6, 0.97))]
    q = np.ascontiguousarray(q0[keep])
    periodic = bool(seed % 2) and L > 2 * 3.3
    box = L if periodic else None
    half = ol.build_list(q, 3.3, box=box)
    if seed % 3 == 0:  # shuffled rows, as the reference's random_shfl leaves them
        engine.shuffle_rows(*half, seed=10)
    ref = oracle_p(q, half, box, 1, 0.005)
    with engine.Context(0) as ctx:
        for method, kernel in (("scatter", 1), ("scatter", 2), ("gather", 1), ("gather", 2)):
            got = run_engine(engine, q, half, box, "fp64", method, "aos", 1, 0.005, ctx=ctx,
                             kernel=kernel)
            assert ol.rel_errors(got, ref)["max_rel"] <= FP64_TOL, (seed, method, kernel)
        for prec in MIXED_PRECS:
            for method, kernel, unroll in (("gather", 1, 0), ("gather", 2, 4), ("gather", 4, 4),
                                           ("scatter", 1, 0), ("scatter", 2, 4)):
                got = run_engine(engine, q, half, box, prec, method,
                                 "soa" if seed % 2 else "aos", 1, 0.005, ctx=ctx, kernel=kernel,
                                 unroll=unroll)
                check_mixed(ol.rel_errors(got, ref), prec, seed, method, kernel)
        ctx.build_list(dev(q), 3.3, box=box)
        np_d, ptr_d, lst_d = ctx.get_list_csr("half")
        np_r, ptr_r, lst_r = ol.build_list(q, 3.3, box=box)
        assert np.array_equal(np_d, np_r) and np.array_equal(lst_d, lst_r), seed


def test_measure_checks_the_particle_count(engine, fixture_rho05):
    f = fixture_rho05
    with engine.Context(0) as ctx:
        q = np.ascontiguousarray(f["q"])
        with pytest.raises(engine.LJError) as e:  # no list yet
            ctx.measure_aos(q, np.zeros_like(q), engine.make_opts(), calls=1)
        assert e.value.status == engine.LJ_ERR_NO_LIST
        ctx.set_list_csr(f["np"], f["ptr"], f["list"])
        q2 = np.ascontiguousarray(np.concatenate([q, q[:7]]))  # 7 particles too many
        with pytest.raises(engine.LJError) as e:
            ctx.measure_aos(q2, np.zeros_like(q2), engine.make_opts(), calls=1)
        assert e.value.status == engine.LJ_ERR_INVALID_ARGUMENT
