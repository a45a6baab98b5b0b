"""Routines called on registered host arrays, with the stream-ordered copies.

A reference-style caller keeps its fields in host memory (the reference's
double[X_np][Y_m][Z_m] arrays); it registers them, and the routines run on
their device mirrors.  Here the copies go through cf_upload_async and
cf_download_async on two side streams ordered by CUDA events against the
context's stream, with two sets of arrays alternating as a pipelined caller
would use them.  In the no-FMA build every written array equals the C
oracle's bit for bit, for each of the two sets.
"""
import numpy as np
import pytest

import cases
import routines

pytestmark = pytest.mark.gpu
DIMS = (16, 12, 10)


def _pinned_copy(torch, a):
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy().reshape(a.shape)
    t[...] = a
    return t


def test_async_copies_of_registered_arrays_equal_oracle(port, cuda_lib):
    import torch
    import channel_flow_gb300 as cf
    r = routines.BY_NAME["Flux_X_limiter"]
    g = cases.grid(DIMS)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        comp = torch.cuda.current_stream()
        h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
        sets, wants = [], []
        for seed in (4, 5):
            a = r.build(g, seed)
            want = cases.copy_case(a)
            routines.run_cpu(port, r, g, want)
            wants.append(want)
            host = [_pinned_copy(torch, x) for x in a]
            for x in host:
                ctx.register(x)
            sets.append(host)
        uploaded = []
        for host in sets:
            for x in host:
                ctx.upload_async(x, h2d.cuda_stream)
            up = torch.cuda.Event()
            up.record(h2d)
            uploaded.append(up)
        h2d.synchronize()
        for host in sets:
            for i in r.outputs:
                host[i][...] = np.nan          # the download must overwrite these
        done = []
        for host, up in zip(sets, uploaded):
            comp.wait_event(up)
            ctx.flux(r.name, host)
            computed = torch.cuda.Event()
            computed.record(comp)
            d2h.wait_event(computed)
            for i in r.outputs:
                ctx.download_async(host[i], d2h.cuda_stream)
            ev = torch.cuda.Event()
            ev.record(d2h)
            done.append(ev)
        for ev in done:
            ev.synchronize()
        for host, want in zip(sets, wants):
            diff = routines.compare(r, g, host, want)
            assert all(v == 0 for v in diff.values()), diff
        for host in sets:
            for x in host:
                ctx.lib.cf_unregister(ctx.h, x.ctypes.data)
    finally:
        ctx.close()


def test_async_copy_of_unregistered_array_is_an_error(cuda_lib):
    import torch
    import channel_flow_gb300 as cf
    g = cases.grid(DIMS)
    ctx = cf.Context(g, precision="fp64")
    try:
        a = np.zeros(g.shape)
        with pytest.raises(RuntimeError, match="not registered"):
            ctx.upload_async(a, torch.cuda.current_stream().cuda_stream)
        with pytest.raises(RuntimeError, match="not registered"):
            ctx.download_async(a, torch.cuda.current_stream().cuda_stream)
    finally:
        ctx.close()
