"""Velocity-Verlet MD on the GPU against an FP64 oracle integration.

The reference has no integrator; the oracle composes its restated force
routine (cpu_ref/force_aos.cpp:192-224) into velocity Verlet: kick dt/2,
drift, kick dt/2, with the list rebuilt from scratch every step.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


oracle_vv = ol.velocity_verlet
periodic_diff = ol.periodic_diff


@pytest.mark.parametrize("graph_steps", [1, 8])
def test_fp64_md_matches_oracle_velocity_verlet(engine, graph_steps):
    q, L = ol.init_fcc_periodic(5, 0.8, 0.05, seed=12)  # 500 particles, L = claimed
    p = engine.init_momenta(q.shape[0], 1.0, seed=4)
    rc, skin, dt, steps = 2.5, 0.3, 0.005, 60
    qd, pd = _dev(q), _dev(p)
    prm = engine.make_md_params(dt, rc, skin, L, precision="fp64", record_every=20,
                                graph_steps=graph_steps)
    with engine.Context(0) as ctx:
        recs, stats = ctx.md_run(qd, pd, prm, steps)
    import torch
    torch.cuda.synchronize()
    qg, pg = qd.cpu().numpy(), pd.cpu().numpy()
    qo, po = oracle_vv(q, p, L, rc, dt, steps)
    assert np.abs(periodic_diff(qg, qo, L)).max() < 1e-11
    e = ol.rel_errors(pg, po)
    assert e["max_rel_rms"] < 1e-10, e
    assert [r[0] for r in recs] == [0, 20, 40, 60]
    assert stats["steps"] == steps and stats["rebuilds"] >= 1
    # energies of the FP64 run against the oracle's at the end
    half = ol.build_list(qo, rc, box=L)
    u = ol.potential_half(qo, *half, cl2=rc * rc, box=L)
    k = ol.oracle().lj_or_kinetic(po, po.shape[0])
    assert abs(recs[-1][2] - u) <= 1e-9 * abs(u) and abs(recs[-1][1] - k) <= 1e-9 * abs(k)


def test_mixed_md_tracks_fp64_and_conserves(engine):
    q, L = ol.init_fcc_periodic(6, 1.0, 0.05, seed=21)  # 864 particles
    p = engine.init_momenta(q.shape[0], 1.0, seed=9)
    rc, skin, dt = 2.5, 0.3, 0.005
    out = {}
    for prec in ("fp64", "mixed"):
        qd, pd = _dev(q), _dev(p)
        prm = engine.make_md_params(dt, rc, skin, L, precision=prec, record_every=50)
        with engine.Context(0) as ctx:
            recs, stats = ctx.md_run(qd, pd, prm, 200)
        import torch
        torch.cuda.synchronize()
        out[prec] = (qd.cpu().numpy(), pd.cpu().numpy(), recs, stats)
    qf, pf, rf, _ = out["fp64"]
    qm, pm, rm, sm = out["mixed"]
    # short trajectories stay together (chaos has not amplified FP32 errors yet)
    assert np.abs(periodic_diff(qm, qf, L)).max() < 1e-5
    # total momentum: the FP64 scatter applies +f and -f (zero to rounding);
    # the mixed gather evaluates f_ij and f_ji separately in FP32, so the sum
    # drifts at the FP32 rounding level of the forces
    assert np.abs(out["fp64"][1][:, :3].sum(axis=0)).max() < 1e-11
    assert np.abs(pm[:, :3].sum(axis=0)).max() < 1e-4
    # the cut (unshifted, as in the reference) potential jumps by |4(rc^-12 -
    # rc^-6)| ~ 0.016 whenever a pair crosses rc, so the total energy is not a
    # constant of this model; the mixed run must reproduce the FP64 energies
    e0 = rf[0][1] + rf[0][2]
    assert [r[0] for r in rm] == [r[0] for r in rf]
    for a, b in zip(rm, rf):
        assert abs((a[1] + a[2]) - (b[1] + b[2])) <= 1e-5 * abs(e0), (a, b)
        assert abs(a[2] - b[2]) <= 1e-5 * abs(b[2]), (a, b)
    assert sm["rebuilds"] >= 2


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_md_run_host_matches_the_device_run(engine, precision):
    """lj_md_run_host (host arrays in and out, the copies overlapped with the
    initial build and the final half kick) integrates as lj_md_run on device
    copies: identical positions and momenta for the mixed gather (to the
    rounding of the FP64 scatter's atomic sums for FP64), the same records,
    with page-locked tensors or plain numpy arrays; zero steps return q and p
    unchanged; a list overflow is reported as from lj_md_run."""
    import torch
    q, L = ol.init_fcc_periodic(6, 1.0, 0.05, seed=21)  # 864 particles
    p = engine.init_momenta(q.shape[0], 1.0, seed=9)
    prm = engine.make_md_params(0.005, 2.5, 0.3, L, precision=precision, record_every=20,
                                graph_steps=8)
    qd, pd = _dev(q), _dev(p)
    with engine.Context(0) as ctx:
        recs_d, st_d = ctx.md_run(qd, pd, prm, 50)
    torch.cuda.synchronize()
    ref_q, ref_p = qd.cpu().numpy(), pd.cpu().numpy()
    pinned = (torch.from_numpy(q.copy()).pin_memory(), torch.from_numpy(p.copy()).pin_memory())
    plain = (q.copy(), p.copy())
    for hq, hp in (pinned, plain):
        with engine.Context(0) as ctx:
            recs_h, st_h = ctx.md_run_host(hq, hp, prm, 50)
        hq_ = hq.numpy() if hasattr(hq, "numpy") else hq
        hp_ = hp.numpy() if hasattr(hp, "numpy") else hp
        if precision == "mixed":  # the gather kick is deterministic
            assert np.array_equal(hq_, ref_q) and np.array_equal(hp_, ref_p)
        else:  # the FP64 scatter adds with atomics: last bits vary run to run
            assert np.abs(periodic_diff(hq_, ref_q, L)).max() < 1e-10
            assert ol.rel_errors(hp_, ref_p)["max_rel_rms"] < 1e-9
        assert [r[0] for r in recs_h] == [r[0] for r in recs_d] == [0, 20, 40, 50]
        for a, b in zip(recs_h, recs_d):
            assert abs(a[1] - b[1]) <= 1e-12 * abs(b[1]) and abs(a[2] - b[2]) <= 1e-12 * abs(b[2])
        assert st_h["rebuilds"] == st_d["rebuilds"]
    q0, p0 = q.copy(), p.copy()
    with engine.Context(0) as ctx:
        ctx.md_run_host(q0, p0, prm, 0)
    assert np.array_equal(q0, q) and np.array_equal(p0, p)
    # the overflow case of test_md_list_overflow_is_reported, through the host entry
    qc, _ = ol.init_fcc_periodic(5, 1.0, 0.05, seed=3)
    with engine.Context(0) as ctx:
        with pytest.raises(engine.LJError) as e:
            ctx.md_run_host(qc.copy(), np.zeros_like(qc),
                            engine.make_md_params(0.005, 3.0, 0.3, 40.0, precision="mixed"), 5)
        assert e.value.status == engine.LJ_ERR_LIST_OVERFLOW


def test_runs_that_continue_a_trajectory_keep_the_list(engine):
    """A context keeps the neighbour list of its last completed run: a run
    that continues the trajectory (same n, box, rc, skin, list kind, and no
    particle beyond skin/2 from its position at that list's build) starts
    without a build and still follows the oracle's FP64 velocity Verlet.  A
    particle moved past skin/2, another skin or another precision forces
    the build."""
    import torch
    q, L = ol.init_fcc_periodic(6, 1.0, 0.05, seed=41)  # 864 particles
    p = engine.init_momenta(q.shape[0], 1.0, seed=6)
    rc, skin, dt = 2.5, 0.3, 0.005
    prm = engine.make_md_params(dt, rc, skin, L, precision="mixed", graph_steps=8)
    qd, pd = _dev(q), _dev(p)
    with engine.Context(0) as ctx:
        _, a = ctx.md_run(qd, pd, prm, 30, max_records=0)
        _, b = ctx.md_run(qd, pd, prm, 30, max_records=0)
        assert a["initial_build"] == 1 and b["initial_build"] == 0, (a, b)
        torch.cuda.synchronize()
        qo, po = oracle_vv(q, p, L, rc, dt, 60)
        assert np.abs(periodic_diff(qd.cpu().numpy(), qo, L)).max() < 1e-7
        assert ol.rel_errors(pd.cpu().numpy(), po)["max_rel_rms"] < 1e-6
        # the host entry keeps it as well
        hq, hp = qd.cpu().numpy().copy(), pd.cpu().numpy().copy()
        _, c = ctx.md_run_host(hq, hp, prm, 5, max_records=0)
        _, c2 = ctx.md_run_host(hq, hp, prm, 5, max_records=0)
        assert c2["initial_build"] == 0
        # one particle moved past skin/2 since the last build (it lies within
        # skin/2 = 0.15 of its position there, so 0.35 more is past it)
        hq[7, 0] = (hq[7, 0] + 0.35) % L
        _, d = ctx.md_run_host(hq, hp, prm, 1, max_records=0)
        assert d["initial_build"] == 1
        # another skin, another precision
        _, e = ctx.md_run_host(hq, hp, engine.make_md_params(dt, rc, 0.35, L), 1, max_records=0)
        assert e["initial_build"] == 1
        _, g = ctx.md_run_host(hq, hp, engine.make_md_params(dt, rc, 0.35, L, precision="fp64"),
                               1, max_records=0)
        assert g["initial_build"] == 1
        _, h = ctx.md_run_host(hq, hp, engine.make_md_params(dt, rc, 0.35, L, precision="fp64"),
                               1, max_records=0)
        assert h["initial_build"] == 0
    # FP64 (compacted half list): a continued run on the kept list follows the
    # oracle to the FP64 path's own bar
    prm64 = engine.make_md_params(dt, rc, skin, L, precision="fp64", graph_steps=8)
    qd, pd = _dev(q), _dev(p)
    with engine.Context(0) as ctx:
        _, a = ctx.md_run(qd, pd, prm64, 30, max_records=0)
        _, b = ctx.md_run(qd, pd, prm64, 30, max_records=0)
    assert a["initial_build"] == 1 and b["initial_build"] == 0
    torch.cuda.synchronize()
    assert np.abs(periodic_diff(qd.cpu().numpy(), qo, L)).max() < 1e-11
    assert ol.rel_errors(pd.cpu().numpy(), po)["max_rel_rms"] < 1e-10


def test_md_list_overflow_is_reported(engine):
    # 500 particles packed into a corner of a large box: the capacity estimate
    # from the mean density is far too small (64 entries for ~150 partners
    # within rc + skin = 3.3), and the run must say so
    q, _ = ol.init_fcc_periodic(5, 1.0, 0.05, seed=3)
    L = 40.0
    p = np.zeros_like(q)
    qd, pd = _dev(q), _dev(p)
    prm = engine.make_md_params(0.005, 3.0, 0.3, L, precision="mixed")
    with engine.Context(0) as ctx:
        with pytest.raises(engine.LJError) as e:
            ctx.md_run(qd, pd, prm, 5)
        assert e.value.status == engine.LJ_ERR_LIST_OVERFLOW


def _oracle_vv_box(q, p, box, rc, dt, steps):
    q, p = q.copy(), p.copy()
    O = ol.oracle()
    b = np.ascontiguousarray(box, np.float64)
    for _ in range(steps):
        half = ol.build_list(q, rc + 0.2, box=b)
        ol.force_sorted_aos(q, p, *half, cl2=rc * rc, dt=0.5 * dt, box=b)
        O.lj_or_drift(q, p, q.shape[0], dt, b.ctypes.data)
        half = ol.build_list(q, rc + 0.2, box=b)
        ol.force_sorted_aos(q, p, *half, cl2=rc * rc, dt=0.5 * dt, box=b)
    return q, p


def test_md_in_a_non_cubic_box(engine):
    """An orthorhombic box (per-axis fixed-point frame in the drift, the list
    build and the force kernels): FP64 against the oracle's integrator, mixed
    against FP64."""
    q, L = ol.init_fcc_periodic(5, 0.8, 0.05, seed=31)
    stretch = np.array([1.25, 1.0, 0.9])
    q[:, :3] *= stretch
    box = L * stretch
    p = engine.init_momenta(q.shape[0], 1.0, seed=5)
    rc, skin, dt, steps = 2.5, 0.3, 0.005, 40
    out = {}
    for prec in ("fp64", "mixed"):
        qd, pd = _dev(q), _dev(p)
        prm = engine.make_md_params(dt, rc, skin, box, precision=prec, record_every=steps)
        with engine.Context(0) as ctx:
            ctx.md_run(qd, pd, prm, steps)
        import torch
        torch.cuda.synchronize()
        out[prec] = (qd.cpu().numpy(), pd.cpu().numpy())
    qo, po = _oracle_vv_box(q, p, box, rc, dt, steps)
    d = out["fp64"][0][:, :3] - qo[:, :3]
    d -= box * np.round(d / box)
    assert np.abs(d).max() < 1e-11
    assert ol.rel_errors(out["fp64"][1], po)["max_rel_rms"] < 1e-10
    d = out["mixed"][0][:, :3] - out["fp64"][0][:, :3]
    d -= box * np.round(d / box)
    assert np.abs(d).max() < 1e-5


def test_loop_graph_and_chunk_graphs_agree_bit_for_bit(engine):
    """The persistent WHILE-node loop and the host-launched chunk graphs run
    the same captured steps: identical positions and momenta, the same
    records (to the rounding of their atomic sums), and the stats say which
    form ran.  kick_lanes = 4 (four lanes per row in the
    two-float kick) sums in another order: within the mixed bars of the
    default's momenta, and against the oracle's FP64 integrator."""
    import torch
    q, L = ol.init_fcc_periodic(6, 1.0, 0.05, seed=41)  # 864 particles
    p = engine.init_momenta(q.shape[0], 1.0, seed=6)
    rc, skin, dt, steps = 2.5, 0.3, 0.005, 60
    out = {}
    for name, kw in (("loop", {}), ("chunks", {"chunk_graphs": True}),
                     ("lanes4", {"kick_lanes": 4})):
        qd, pd = _dev(q), _dev(p)
        prm = engine.make_md_params(dt, rc, skin, L, precision="mixed", record_every=20,
                                    graph_steps=8, **kw)
        with engine.Context(0) as ctx:
            recs, stats = ctx.md_run(qd, pd, prm, steps)
        torch.cuda.synchronize()
        out[name] = (qd.cpu().numpy(), pd.cpu().numpy(), recs, stats)
    assert out["loop"][3]["loop_graph"] == 1 and out["chunks"][3]["loop_graph"] == 0
    assert np.array_equal(out["loop"][0], out["chunks"][0])
    assert np.array_equal(out["loop"][1], out["chunks"][1])
    # energy records are sums with atomics (their order varies run to run)
    for a, b in zip(out["loop"][2], out["chunks"][2]):
        assert a[0] == b[0] and abs(a[1] - b[1]) <= 1e-12 * abs(b[1])
        assert abs(a[2] - b[2]) <= 1e-12 * abs(b[2])
    assert out["loop"][3]["rebuilds"] == out["chunks"][3]["rebuilds"] >= 1
    qo, po = oracle_vv(q, p, L, rc, dt, steps)
    for name in ("loop", "lanes4"):
        assert np.abs(periodic_diff(out[name][0], qo, L)).max() < 1e-7, name
        assert ol.rel_errors(out[name][1], po)["max_rel_rms"] < 1e-6, name
    assert ol.rel_errors(out["lanes4"][1], out["loop"][1])["max_rel_rms"] < 1e-7
    with engine.Context(0) as ctx:
        with pytest.raises(engine.LJError):
            ctx.md_run(_dev(q), _dev(p), engine.make_md_params(dt, rc, skin, L, kick_lanes=3), 1)
