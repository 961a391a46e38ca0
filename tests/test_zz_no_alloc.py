"""The allocation-free mixed force entry point, through the C ABI.

Some callers cannot allocate device memory: their host owns every
allocation (a pooled allocator the engine cannot see), or an allocation's
implicit device synchronisation is not allowed where they call us.
lj_force_mixed_noalloc_aos serves them with a static scratch array.  This
file checks, on two calls in a row:
  * its result is bit for bit that of the regular mixed entry point
    (lj_force_aos, which allocates its scratch in the context) run with the
    same launch shape (kernel 2, 4 lanes, 4 entries in flight, 128 threads)
    and every pair in two-float terms (ff_all);
  * both meet the mixed bar against the FP64 oracle (per particle
    max |dF_i| / |F_i| <= 1e-5);
  * after the first call on the device, further calls change neither the
    device's free memory nor the caching allocator's statistics.
Collected last on purpose; it also runs alone.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

MIXED_MAX_REL = 1e-5  # max |dF_i| / |F_i| per particle, as in test_force_gpu.py


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _system(case):
    if case == "pbc_rho1":
        return ol.init_fcc_periodic(6, 1.0, 0.05, seed=3)
    if case == "pbc_rho0.5_108k":
        return ol.init_fcc_periodic(30, 0.5, 0.05, seed=20240601)
    q = ol.init_reference(0.5, 10.0)
    if case == "open_far":
        q = q.copy()
        q[:, :3] += 1e4
    return q, None


@pytest.mark.parametrize("case", ["pbc_rho1", "pbc_rho0.5_108k", "open_rho0.5", "open_far"])
def test_noalloc_matches_regular_entry_two_calls(engine, case):
    import torch
    q, box = _system(case)
    npp, ptr_, lst = ol.build_list(q, 3.3, box=box, full=True)
    half = ol.build_list(q, 3.3, box=box)
    ref = ol.force_sorted_aos(q, np.zeros_like(q), *half, cl2=9.0, dt=0.005, box=box)
    qd = _dev(q)
    d_np, d_ptr, d_lst = _dev(npp), _dev(ptr_), _dev(lst)
    p_new = torch.zeros_like(qd)
    p_old = torch.zeros_like(qd)
    opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision="mixed", method="gather",
                            kernel=2, lanes=4, unroll=4, block=128, ff_all=True)
    with engine.Context(0) as ctx:
        ctx.set_list_csr(d_np, d_ptr, d_lst, kind="full")
        for call in range(2):
            engine.force_mixed_noalloc_aos(qd, p_new, 0.005, 9.0, d_lst, d_np, d_ptr, box=box)
            ctx.force_aos(qd, p_old, opts)
            torch.cuda.synchronize()
            a, b = p_new.cpu().numpy(), p_old.cpu().numpy()
            assert np.isfinite(a).all()
            assert np.array_equal(a, b), (call, np.abs(a - b).max())
            e = ol.rel_errors(a, ref * (call + 1))
            assert e["max_rel"] <= MIXED_MAX_REL, (call, e)


def test_noalloc_calls_allocate_nothing(engine):
    """After the first call on the device (its set-up), periodic and open-box
    calls leave the device's free memory and torch's allocator untouched."""
    import torch
    out = {}
    for case in ("pbc_rho1", "open_rho0.5"):
        q, box = _system(case)
        npp, ptr_, lst = ol.build_list(q, 3.3, box=box, full=True)
        qd, pd = _dev(q), _dev(np.zeros_like(q))
        d_np, d_ptr, d_lst = _dev(npp), _dev(ptr_), _dev(lst)
        out[case] = (qd, pd, d_np, d_ptr, d_lst, box)
    for qd, pd, d_np, d_ptr, d_lst, box in out.values():  # set-up on this device
        engine.force_mixed_noalloc_aos(qd, pd, 0.005, 9.0, d_lst, d_np, d_ptr, box=box)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        for qd, pd, d_np, d_ptr, d_lst, box in out.values():
            engine.force_mixed_noalloc_aos(qd, pd, 0.005, 9.0, d_lst, d_np, d_ptr, box=box)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0
    for k in ("allocation.all.allocated", "segment.all.allocated", "reserved_bytes.all.current"):
        assert stats1.get(k) == stats0.get(k), k


def test_noalloc_rejects_oversize_and_bad_arguments(engine):
    L = engine.lib()
    n = engine.NOALLOC_MAX_PARTICLES + 1
    st = L.lj_force_mixed_noalloc_aos(16, 16, n, 0.005, 9.0, 16, 16, 16, None, None)
    assert st == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_force_mixed_noalloc_aos(8, 16, 10, 0.005, 9.0, 16, 16, 16, None,
                                        None) == engine.LJ_ERR_INVALID_ARGUMENT
    for dt in (float("inf"), float("-inf"), float("nan")):
        assert L.lj_force_mixed_noalloc_aos(16, 16, 10, dt, 9.0, 16, 16, 16, None,
                                            None) == engine.LJ_ERR_INVALID_ARGUMENT, dt
    assert L.lj_force_mixed_noalloc_aos(None, None, 0, 0.005, 9.0, None, None, None, None,
                                        None) == engine.LJ_OK
