"""The reference's own CUDA kernels on the same GB300, beside the engine.

The reference's cuda/kernel.cuh is compiled unmodified into a cubin
(oracle/_ref/refcuda.cubin, `make -C oracle refcuda`) and launched with its
own argument list and launch geometry (THREAD_BLOCK 128, one thread or one
warp per particle; cuda/force_cuda.cu:45,319-342,398-443).  On the
reference's own open-boundary systems (init(), cpu_ref/force_aos.cpp:142-169)
every kernel is first checked against the oracle's FP64 force_sorted, then
timed (one call per sample, L2 flushed before each) beside the engine's FP64
and mixed paths on the same list.  Run with -s to see the table.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ol.refcuda_available(),
                                 reason="reference CUDA cubin not built (needs the reference "
                                        "checkout where build() ran)")]

# (kernel, list kind, list form, threads per particle) -- force_cuda.cu:418-441
GATHER = [("force_kernel_plain", "full", "csr", 1), ("force_kernel_memopt", "full", "csr", 1),
          ("force_kernel_memopt3", "full", "ell", 1),
          ("force_kernel_unrolling2", "full", "ell", 1),
          ("force_kernel_warp_unroll", "full", "csr", 32),
          ("force_kernel_warp_unroll2", "full", "csr", 32)]
SCATTER = [("force_kernel_plain_with_aar", "half", "csr", 1),
           ("force_kernel_memopt3_with_aar", "half", "ell", 1),
           ("force_kernel_warp_unroll_with_aar", "half", "csr", 32)]
THREAD_BLOCK = 128
DT, CL2 = 0.001, 9.0


def _time(torch, fn, flush, samples=10):
    fn()
    tot = 0.0
    for _ in range(samples):
        flush.add_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        tot += a.elapsed_time(b)
    return tot / samples


@pytest.mark.parametrize("density,L", [(0.5, 50.0), (1.0, 50.0)])
def test_reference_cuda_kernels_beside_the_engine(engine, density, L):
    import torch
    dev = torch.device("cuda", 0)
    torch.zeros(1, device=dev)  # runtime context current before the cubin loads
    lib, table = ol.load_refcuda()
    q = ol.init_reference(density, L)
    n = q.shape[0]
    half = ol.build_list(q, 3.3)
    P = len(half[2])
    ref = ol.force_sorted_aos(q, np.zeros_like(q), *half, cl2=CL2, dt=DT)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rows = []
    with engine.Context(0, stream=torch.cuda.current_stream()) as ctx:
        ctx.set_list_csr(*[d(a) for a in half])
        lists = {"half": {"csr": [d(a) for a in half]}, "full": {"csr": [d(a) for a in
                                                                        ctx.get_list_csr("full")]}}
        for kind in ("half", "full"):
            npp, ell = ctx.get_list_ell(n, kind=kind)
            lists[kind]["ell"] = [d(npp), d(ell), None]
        q4, q3 = d(q), d(q[:, :3])
        for name, kind, form, tpp in GATHER + SCATTER:
            for vec, qd in (("double3", q3), ("double4", q4)):
                k = table[(name, vec)]
                npp, lst = lists[kind][form][0], lists[kind][form][2 if form == "csr" else 1]
                ptrd = lists[kind][form][1] if form == "csr" else None
                grid = (n * tpp - 1) // THREAD_BLOCK + 1
                pd = torch.zeros_like(qd)

                def call(pd=pd, qd=qd, k=k, grid=grid, lst=lst, npp=npp, ptrd=ptrd):
                    st = lib.rc_launch(k, grid, THREAD_BLOCK, qd.data_ptr(), pd.data_ptr(), n,
                                       DT, CL2, lst.data_ptr(), npp.data_ptr(),
                                       ptrd.data_ptr() if ptrd is not None else None,
                                       torch.cuda.current_stream().cuda_stream)
                    assert st == 0, (name, vec, st)
                call()
                got = np.zeros_like(q)
                got[:, :3] = pd[:, :3].cpu().numpy()
                e = ol.rel_errors(got, ref)
                assert e["max_rel"] <= 1e-12, (name, vec, e)  # the comparator is the reference
                ms = _time(torch, call, flush)
                rows.append((f"reference {name}<{vec}>", ms))
        qd, pd = d(q), d(np.zeros_like(q))
        for prec, method in (("fp64", "scatter"), ("fp64", "gather"), ("mixed", "gather"),
                             ("mixed", "scatter")):
            opts = engine.make_opts(dt=DT, cl2=CL2, precision=prec, method=method)
            ms = _time(torch, lambda: ctx.force_aos(qd, pd, opts), flush)
            rows.append((f"engine {prec}/{method}", ms))
    best_ref = min(ms for nm, ms in rows if nm.startswith("reference"))
    best_eng = min(ms for nm, ms in rows if nm.startswith("engine mixed"))
    print(f"\nN = {n}, rho = {density}, L = {L} (open), P = {P} half pairs; "
          "one call, L2 flushed before each")
    for nm, ms in sorted(rows, key=lambda r: r[1]):
        print(f"  {nm:58s} {ms * 1e3:9.1f} us  {P / ms / 1e6:8.2f} G pair/s")
    print(f"  engine mixed / best reference kernel: {best_ref / best_eng:.1f}x")
    assert best_eng < best_ref
