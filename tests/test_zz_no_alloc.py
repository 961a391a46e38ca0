"""The allocation-free mixed force entry point, through the C ABI.

Some callers cannot allocate device memory (their host owns every allocation,
or an allocation's implicit synchronisation is not allowed where they call
us).  lj_force_mixed_noalloc_aos serves them with a static scratch array; this
file checks it against the regular mixed entry point (lj_force_aos, which
allocates its scratch in the context) on two calls in a row, with the mixed
tolerance of the parity tests.  Collected last on purpose; it also runs alone.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5  # max |dF_i| / rms|F|, as in test_force_gpu.py


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("case", ["pbc_rho1", "pbc_rho0.5_108k", "open_rho0.5"])
def test_noalloc_matches_regular_entry_two_calls(engine, case):
    import torch
    if case == "pbc_rho1":
        q, box = ol.init_fcc_periodic(6, 1.0, 0.05, seed=3)
    elif case == "pbc_rho0.5_108k":
        q, box = ol.init_fcc_periodic(30, 0.5, 0.05, seed=20240601)
    else:
        q, box = ol.init_reference(0.5, 10.0), None
    npp, ptr_, lst = ol.build_list(q, 3.3, box=box, full=True)
    qd = _dev(q)
    d_np, d_ptr, d_lst = _dev(npp), _dev(ptr_), _dev(lst)
    p_new = torch.zeros_like(qd)
    p_old = torch.zeros_like(qd)
    opts = engine.make_opts(dt=0.005, cl2=9.0, box=box, precision="mixed", method="gather")
    with engine.Context(0) as ctx:
        ctx.set_list_csr(d_np, d_ptr, d_lst, kind="full")
        for call in range(2):
            engine.force_mixed_noalloc_aos(qd, p_new, 0.005, 9.0, d_lst, d_np, d_ptr, box=box)
            ctx.force_aos(qd, p_old, opts)
            torch.cuda.synchronize()
            a, b = p_new.cpu().numpy(), p_old.cpu().numpy()
            e = ol.rel_errors(a, b)
            assert e["max_rel_rms"] <= MIXED_TOL, (call, e)
            assert np.isfinite(a).all()


def test_noalloc_rejects_oversize_and_bad_arguments(engine):
    L = engine.lib()
    n = engine.NOALLOC_MAX_PARTICLES + 1
    st = L.lj_force_mixed_noalloc_aos(16, 16, n, 0.005, 9.0, 16, 16, 16, None, None)
    assert st == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_force_mixed_noalloc_aos(8, 16, 10, 0.005, 9.0, 16, 16, 16, None,
                                        None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_force_mixed_noalloc_aos(None, None, 0, 0.005, 9.0, None, None, None, None,
                                        None) == engine.LJ_OK
