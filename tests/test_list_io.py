"""Host helpers for the reference's list formats and row order (no GPU):
random_shfl, the CUDA driver's text cache and cpu_ref's binary pair.dat."""
import multiprocessing as mp
import os

import numpy as np
import pytest

import oracle_lib as ol


def test_shuffle_rows_is_a_seeded_per_row_permutation(engine, fixture_rho1):
    f = fixture_rho1
    npp, ptr = f["np"], f["ptr"]
    a = f["list"].copy()
    b = f["list"].copy()
    c = f["list"].copy()
    engine.shuffle_rows(npp, ptr, a, seed=10)
    engine.shuffle_rows(npp, ptr, b, seed=10)
    engine.shuffle_rows(npp, ptr, c, seed=11)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert not np.array_equal(a, f["list"])
    for i in range(len(npp)):
        s = slice(ptr[i], ptr[i] + npp[i])
        assert np.array_equal(np.sort(a[s]), f["list"][s])


def test_text_cache_round_trip_and_broken_cache(engine, fixture_rho05, tmp_path):
    f = fixture_rho05
    path = tmp_path / ".cache_pair_half.dat"
    engine.cache_write_text(path, f["np"], f["ptr"], f["list"])
    head = path.read_text().split("\n")[:2]
    assert head[0] == f"{len(f['np'])} {len(f['list'])}"
    assert head[1] == f"{f['np'][0]} {f['ptr'][0]}"
    npp, ptr, lst = engine.cache_read_text(path, len(f["np"]), len(f["list"]))
    for a, b in zip((npp, ptr, lst), (f["np"], f["ptr"], f["list"])):
        assert np.array_equal(a, b)
    with pytest.raises(engine.LJError) as e:  # particle count differs: "may be broken"
        engine.cache_read_text(path, len(f["np"]) + 1, len(f["list"]))
    assert e.value.status == engine.LJ_ERR_BAD_LIST
    bad = path.read_text().split("\n")
    bad[-2] = str(len(f["np"]))  # an out-of-range j
    path.write_text("\n".join(bad))
    with pytest.raises(engine.LJError):
        engine.cache_read_text(path, len(f["np"]), len(f["list"]))


def test_pairdat_round_trip(engine, fixture_rho05, tmp_path):
    f = fixture_rho05
    n = len(f["np"])
    path = tmp_path / "pair.dat"
    engine.pairdat_write(path, n, f["i"], f["j"])
    assert os.path.getsize(path) == 4 * (1 + 400000 + 2 * 12000000)
    npp, ii, jj = engine.pairdat_read(path, n, len(f["i"]))
    assert np.array_equal(npp, f["np"]) and np.array_equal(ii, f["i"]) and np.array_equal(jj, f["j"])


def _reference_pairdat(q, workdir, out):
    os.chdir(workdir)
    R = ol.load_ref("aos")
    R.ref_set_positions(q.shape[0], np.ascontiguousarray(q))
    npairs = R.ref_savepair_cwd()
    ii = np.zeros(npairs, np.int32)
    jj = np.zeros(npairs, np.int32)
    R.ref_get_pairs(ii, jj)
    out.put((ii, jj))


def _reference_loadpair(q, workdir, out):
    os.chdir(workdir)
    R = ol.load_ref("aos")
    R.ref_set_positions(q.shape[0], np.ascontiguousarray(q))
    npairs = R.ref_loadpair_cwd()
    ii = np.zeros(npairs, np.int32)
    jj = np.zeros(npairs, np.int32)
    R.ref_get_pairs(ii, jj)
    out.put((ii, jj))


@pytest.mark.skipif(not ol.ref_available(), reason="reference cpu_ref not built here (x86 only)")
def test_pairdat_is_the_reference_format(engine, fixture_rho05, tmp_path):
    """A pair.dat written by the reference's own savepair() is read by the
    engine, and one written by the engine is read by the reference's loadpair()."""
    f = fixture_rho05
    ctx = mp.get_context("spawn")
    qu = ctx.Queue()
    (tmp_path / "ref").mkdir()
    pr = ctx.Process(target=_reference_pairdat, args=(f["q"], str(tmp_path / "ref"), qu))
    pr.start()
    ii, jj = qu.get()
    pr.join()
    n = f["q"].shape[0]
    npp, ei, ej = engine.pairdat_read(tmp_path / "ref" / "pair.dat", n, len(ii))
    assert np.array_equal(ei, ii) and np.array_equal(ej, jj) and npp.sum() == len(ii)
    (tmp_path / "mine").mkdir()
    engine.pairdat_write(tmp_path / "mine" / "pair.dat", n, f["i"], f["j"])
    pr = ctx.Process(target=_reference_loadpair, args=(f["q"], str(tmp_path / "mine"), qu))
    pr.start()
    ri, rj = qu.get()
    pr.join()
    assert np.array_equal(ri, f["i"]) and np.array_equal(rj, f["j"])
