"""The contracted FP64 build's reciprocal (cf_reciprocal_check: the
hardware's approximate FP64 reciprocal refined by two Newton-Raphson steps,
used by the kernels in place of divisions) against the correctly rounded
1/d, on random doubles over the normal range and on edge values: within one
unit in the last place."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    assert np.all(np.sign(a) == np.sign(b))
    return np.abs(ia - ib)


def test_reciprocal_within_one_ulp(cuda_lib):
    import torch
    rng = np.random.default_rng(5)
    n = 1 << 20
    mag = 10.0 ** rng.uniform(-300, 300, n)
    d = mag * rng.choice([-1.0, 1.0], n)
    tiny = np.finfo(np.float64).tiny
    edges = np.array([1.0, -1.0, 2.0, 0.5, 3.0, 1.0 / 3.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0),
                      np.finfo(np.float64).max / 8, tiny * 4, 1e-300, 1e300, 0.007, 1.4, 287.0, 1e-8])
    d = np.concatenate([d, edges, -edges])
    dev = torch.from_numpy(d).cuda()
    out = torch.empty_like(dev)
    rc = cuda_lib.cf_reciprocal_check(None, dev.data_ptr(), out.data_ptr(), d.size)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = 1.0 / d
    assert np.all(np.isfinite(got))
    u = _ulps(got, want)
    assert int(u.max()) <= 1, (int(u.max()), d[int(np.argmax(u))])
