"""Replica batches: one velocity-Verlet loop over many independent periodic
systems of uneven size and density, checked replica by replica against the
single-system FP64 MD of the same replica, and (the 512-replica batching
workload) against the oracle's FP64 velocity Verlet."""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

SPECS = [(4, 1.0), (5, 0.5), (6, 0.8), (4, 0.8), (7, 1.0), (5, 1.0)]  # (FCC cells, density)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make_batch(engine):
    qs, ps, boxes, offs = [], [], [], [0]
    for k, (nc, rho) in enumerate(SPECS):
        q, L = ol.init_fcc_periodic(nc, rho, 0.05, seed=100 + k)
        p = engine.init_momenta(q.shape[0], 1.0, seed=200 + k)
        qs.append(q)
        ps.append(p)
        boxes.append([L, L, L])
        offs.append(offs[-1] + q.shape[0])
    return np.concatenate(qs), np.concatenate(ps), np.array(boxes), np.array(offs, np.int32)


def periodic_diff(a, b, L):
    d = a[:, :3] - b[:, :3]
    return d - L * np.round(d / L)


def test_batch_replicas_follow_their_own_dynamics(engine):
    import torch
    q, p, boxes, offs = make_batch(engine)
    rc, skin, dt, steps = 2.5, 0.3, 0.005, 100
    qd, pd = _dev(q), _dev(p)
    prm = engine.make_md_params(dt, rc, skin, 1.0, precision="mixed", record_every=50)
    with engine.Context(0) as ctx:
        en, stats, shapes = ctx.batch_run(qd, pd, offs, boxes, prm, steps)
    torch.cuda.synchronize()
    qb, pb = qd.cpu().numpy(), pd.cpu().numpy()
    assert en.shape == (3, len(SPECS), 2) and stats["rebuilds"] >= 1
    assert shapes[:, 0].sum() == q.shape[0]  # every row is in one size class
    for r, (nc, rho) in enumerate(SPECS):
        a, b = offs[r], offs[r + 1]
        L = boxes[r, 0]
        q1, p1 = _dev(q[a:b]), _dev(p[a:b])
        prm1 = engine.make_md_params(dt, rc, skin, L, precision="fp64", record_every=50)
        with engine.Context(0) as ctx:
            recs, _ = ctx.md_run(q1, p1, prm1, steps)
        torch.cuda.synchronize()
        qf = q1.cpu().numpy()
        assert np.abs(periodic_diff(qb[a:b], qf, L)).max() < 1e-4, r
        for k, rec in enumerate(recs):
            e_b = en[k, r, 0] + en[k, r, 1]
            e_f = rec[1] + rec[2]
            assert abs(e_b - e_f) <= 1e-5 * abs(e_f), (r, k, e_b, e_f)


def c4_batch(engine, seed=20240601):
    """The 512-replica batch of the batching workload (bench.py --workload
    batch_512): N log-uniform in [256, 16384] -> round((N/4)^(1/3)) FCC cells,
    rho from {0.5, 0.8, 1.0}, jitter 0.05, MB momenta at T* = 1."""
    rng = np.random.default_rng(seed)
    qs, ps, boxes, offs, rhos = [], [], [], [0], []
    for r in range(512):
        ndraw = float(np.exp(rng.uniform(np.log(256), np.log(16384))))
        nc = int(round((ndraw / 4) ** (1 / 3)))
        rho = float(rng.choice([0.5, 0.8, 1.0]))
        q, L = ol.init_fcc_periodic(nc, rho, 0.05, seed=seed + 1000 + r)
        qs.append(q)
        ps.append(engine.init_momenta(q.shape[0], 1.0, seed=seed + 5000 + r))
        boxes.append([L, L, L])
        offs.append(offs[-1] + q.shape[0])
        rhos.append(rho)
    return (np.concatenate(qs), np.concatenate(ps), np.array(boxes), np.array(offs, np.int32),
            np.array(rhos))


def test_batch_512_replicas_against_the_oracle(engine):
    """All 512 replicas of the batching workload in one batched mixed MD run
    of 40 steps; the smallest and the largest replica and the first replica of
    every density are compared with the oracle's FP64 velocity Verlet."""
    import torch
    q, p, boxes, offs, rhos = c4_batch(engine)
    rc, skin, dt, steps = 2.5, 0.3, 0.005, 40
    qd, pd = _dev(q), _dev(p)
    prm = engine.make_md_params(dt, rc, skin, 1.0, precision="mixed", record_every=steps)
    with engine.Context(0) as ctx:
        en, stats, shapes = ctx.batch_run(qd, pd, offs, boxes, prm, steps)
    torch.cuda.synchronize()
    qb, pb = qd.cpu().numpy(), pd.cpu().numpy()
    sizes = np.diff(offs)
    assert shapes[:, 0].sum() == q.shape[0]
    assert (shapes[:, 0] > 0).sum() >= 2  # rows fall into more than one size class
    sample = {int(np.argmin(sizes)), int(np.argmax(sizes))}
    sample |= {int(np.flatnonzero(rhos == rho)[0]) for rho in (0.5, 0.8, 1.0)}
    for r in sorted(sample):
        a, b = offs[r], offs[r + 1]
        L = boxes[r, 0]
        qo, po = ol.velocity_verlet(q[a:b], p[a:b], L, rc, dt, steps)
        assert np.abs(ol.periodic_diff(qb[a:b], qo, L)).max() < 1e-6, r
        e = ol.rel_errors(pb[a:b], po)
        assert e["max_rel_rms"] < 1e-6, (r, e)
        # the final record's energies against the oracle's
        half = ol.build_list(qo, rc, box=L)
        u = ol.potential_half(qo, *half, cl2=rc * rc, box=L)
        k = ol.oracle().lj_or_kinetic(po, po.shape[0])
        assert abs(en[-1, r, 1] - u) <= 1e-7 * abs(u), (r, en[-1, r, 1], u)
        assert abs(en[-1, r, 0] - k) <= 1e-7 * abs(k), (r, en[-1, r, 0], k)
