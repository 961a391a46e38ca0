"""The C ABI library without a GPU: it loads, exports exactly what
include/lj_gb300.h declares, and rejects bad arguments before any launch."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT


def header_functions():
    text = (ROOT / "include" / "lj_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lj_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine):
    L = engine.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    # the ctypes binding covers the whole ABI
    assert sorted(engine.EXPORTED) == names


def test_abi_basics(engine):
    L = engine.lib()
    assert L.lj_abi_version() == 1
    assert L.lj_status_string(0) == b"ok"
    assert L.lj_status_string(engine.LJ_ERR_BAD_LIST).startswith(b"neighbour list")
    o = engine.ForceOpts()
    L.lj_force_opts_default(C.byref(o))
    assert (o.dt, o.cl2, o.periodic, o.precision, o.method) == (0.001, 9.0, 0, 0, 0)


def test_argument_checks_need_no_gpu(engine):
    L = engine.lib()
    q = np.zeros((4, 4))
    # negative n, bad list kind, misaligned AoS pointer: rejected up front
    assert L.lj_force_csr_fp64_aos(q.ctypes.data, q.ctypes.data, -1, 0.001, 9.0, None, None,
                                   None, 0, None, None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_force_csr_fp64_aos(q.ctypes.data, q.ctypes.data, 4, 0.001, 9.0, 1, 1, 1, 7,
                                   None, None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_force_csr_fp64_aos(q.ctypes.data + 8, q.ctypes.data, 4, 0.001, 9.0, 1, 1, 1, 0,
                                   None, None) == engine.LJ_ERR_INVALID_ARGUMENT
    # n = 0 is a no-op
    assert L.lj_force_csr_fp64_aos(None, None, 0, 0.001, 9.0, None, None, None, 0, None,
                                   None) == 0
    assert L.lj_force_pairs_fp64_aos(None, None, 0, 0.001, 9.0, None, None, -5, None,
                                     None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_ctx_create(None, 0) == engine.LJ_ERR_INVALID_ARGUMENT
    # entries that take a context reject a missing one before any CUDA call
    prm = engine.make_md_params(0.005, 2.5, 0.3, 10.0)
    assert L.lj_md_run_host(None, q.ctypes.data, q.ctypes.data, 4, prm, 1, None, 0, None,
                            None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_md_run(None, q.ctypes.data, q.ctypes.data, 4, prm, 1, None, 0, None,
                       None) == engine.LJ_ERR_INVALID_ARGUMENT
    assert L.lj_ctx_set_l2_window(None, 0.5) == engine.LJ_ERR_INVALID_ARGUMENT


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device path")
def test_context_without_device_fails_cleanly(engine):
    with pytest.raises(engine.LJError) as e:
        engine.Context(0)
    assert e.value.status == engine.LJ_ERR_CUDA


def test_engine_does_not_import_oracle():
    """The product package never loads the oracle or any CPU force path."""
    pkg = ROOT / "lj_gpu_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cpp")):
        assert "oracle" not in f.read_text().lower(), f


def test_setup_generators_match_oracle(engine):
    """The engine's host generators reproduce the oracle (and so the reference's
    init(), pinned bitwise in test_oracle.py)."""
    import oracle_lib as ol
    for density, L in ((0.5, 10.0), (1.0, 8.0), (0.5, 50.0)):
        assert np.array_equal(engine.init_reference(density, L), ol.init_reference(density, L))
    q, L = engine.init_fcc(5, 0.5, 0.05, seed=99)
    q2, L2 = ol.init_fcc_periodic(5, 0.5, 0.05, seed=99)
    assert L == L2 and np.array_equal(q, q2)
    p = engine.init_momenta(20000, 1.0, seed=3)
    assert np.abs(p[:, :3].sum(axis=0)).max() < 1e-9
    assert abs(p[:, :3].var() - 1.0) < 0.03 and (p[:, 3] == 0).all()
