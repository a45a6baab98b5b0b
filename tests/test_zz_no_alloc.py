"""The allocation-free DPLUSGS entry point (cf_DPLUSGS_noalloc) against the
context-based one (cf_DPLUSGS).

Callers that may not allocate device memory - a solver loop captured into a
CUDA graph, a latency-bound loop that cannot afford the device-wide
synchronisation of cudaMalloc/cudaFree, a host whose memory manager owns the
whole device - use the entry point without a context, whose only scratch is
a fixed file-scope device array.  Two calls in a row, on different inputs,
must give what the existing entry point gives (the scratch keeps the
previous call's contents, so the second call checks that nothing stale is
read) and what the C oracle gives, bit for bit, and a grid larger than the
array allows must be refused.

This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

import cases
import routines

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _to_dev(arrays):
    import torch
    return [torch.from_numpy(a).cuda() for a in arrays]


def test_noalloc_dplusgs_matches_context_entry_point(cuda_lib):
    import torch
    import channel_flow_gb300 as cf

    dims = cases.GRIDS[2]
    g = cases.grid(dims)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        for seed in (3, 29):                      # two calls in a row
            a = cases.dt_case(g, seed)
            want = _to_dev(a)
            got = _to_dev(a)
            er_want = ctx.DPLUSGS(cases.DELTA_T, *want)
            er_got = cf.dplusgs_noalloc(g, cases.DELTA_T, *got)
            torch.cuda.synchronize()
            for i in cases.LU_OUT:
                w = want[i].cpu().numpy()
                o = got[i].cpu().numpy()
                scale = max(float(np.max(np.abs(w))), 1e-300)
                assert float(np.max(np.abs(o - w))) / scale <= RTOL, f"seed {seed} slot {i}"
            np.testing.assert_allclose(er_got, er_want, rtol=RTOL, atol=0)
    finally:
        ctx.close()


def test_noalloc_dplusgs_equals_oracle_bit_for_bit(port, cuda_lib):
    """The entry point is compiled without FMA contraction, like the exact
    build: every written array equals the C oracle's DPLUSGS (the
    defined-index restatement of the reference's) bit for bit; the residual
    norms, summed in another order, agree to 1e-12."""
    import torch
    import channel_flow_gb300 as cf

    r = routines.BY_NAME["DPLUSGS"]
    for dims in (cases.GRIDS[0], cases.GRIDS[2]):
        g = cases.grid(dims)
        for seed in (5, 31):                      # two calls in a row per grid
            a = cases.dt_case(g, seed)
            want = cases.copy_case(a)
            er_want = routines.run_cpu(port, r, g, want)
            got = _to_dev(a)
            er_got = cf.dplusgs_noalloc(g, cases.DELTA_T, *got)
            torch.cuda.synchronize()
            host = [x.cpu().numpy() for x in got]
            diff = routines.compare(r, g, host, want)
            assert all(v == 0 for v in diff.values()), f"{dims} seed {seed}: differing entries per slot {diff}"
            np.testing.assert_allclose(er_got, er_want, rtol=RTOL, atol=0)


def test_noalloc_rejects_grids_beyond_its_scratch(cuda_lib):
    import ctypes as C

    import torch
    from channel_flow_gb300 import _lib

    # ceil(2000/32) * ceil(2000/8) * 600 reduction blocks > 262144; the size
    # is checked before any pointer is touched or any kernel is launched
    g = _lib.cf_grid()
    cuda_lib.cf_grid_reference(C.byref(g), 600, 2000, 2000)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptrs = _lib.ptr_array([dummy.data_ptr()] * 64)
    er = np.zeros(5)
    e = [er[n:].ctypes.data for n in range(5)]
    rc = cuda_lib.cf_DPLUSGS_noalloc(C.byref(g), None, cases.DELTA_T, *e, ptrs)
    assert rc == _lib.CF_ERR_ARG
    assert np.all(er == 0)
