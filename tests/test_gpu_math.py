"""Accuracy of the plain path's FP64 exp / log / reciprocal (fp64_math.cuh) on the GPU.

Each is compared in ulps against CUDA's own function (torch on float64 CUDA tensors) and against an
extended-precision host reference (numpy long double: 64-bit mantissa on x86-64, 113-bit on aarch64).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ia, ib = a.view(np.int64), b.view(np.int64)
    ia = np.where(ia < 0, np.int64(-(2 ** 63)) - ia, ia)
    ib = np.where(ib < 0, np.int64(-(2 ** 63)) - ib, ib)
    return np.abs(ia - ib)


def _run(which, x):
    import torch
    import combustion_gb300 as cb
    t = torch.from_numpy(x).cuda()
    return cb.fp64_math(which, t).cpu().numpy(), t


def test_exp():
    import torch
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-700, 700, 1 << 20), rng.uniform(-1, 1, 1 << 18), rng.uniform(-1e-6, 1e-6, 1 << 16),
                        np.arange(-700, 700, 0.001953125)])
    y, t = _run("exp", x)
    ref_cuda = torch.exp(t).cpu().numpy()
    ref_ld = np.exp(x.astype(np.longdouble)).astype(np.float64)
    assert _ulps(y, ref_cuda).max() <= 2
    assert _ulps(y, ref_ld).max() <= 1
    special = np.array([np.inf, -np.inf, np.nan, 710.0, -746.0, -720.0, 708.5, 0.0, -0.0])
    ys, ts = _run("exp", special)
    np.testing.assert_array_equal(ys, torch.exp(ts).cpu().numpy())


def test_log():
    import torch
    rng = np.random.default_rng(1)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 1 << 20), rng.uniform(0.5, 2.0, 1 << 18),
                        1.0 + rng.uniform(-1e-3, 1e-3, 1 << 16), rng.uniform(200.0, 4000.0, 1 << 16)])
    y, t = _run("log", x)
    ref_cuda = torch.log(t).cpu().numpy()
    ref_ld = np.log(x.astype(np.longdouble)).astype(np.float64)
    assert _ulps(y, ref_cuda).max() <= 2
    err = _ulps(y, ref_ld)
    assert err.max() <= 2 and (err > 1).mean() < 1e-4
    special = np.array([0.0, -0.0, -1.0, np.inf, np.nan, 5e-324, 1.0])
    ys, ts = _run("log", special)
    np.testing.assert_array_equal(ys, torch.log(ts).cpu().numpy())


def test_reciprocal():
    rng = np.random.default_rng(2)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 1 << 20) * rng.choice([-1.0, 1.0], 1 << 20),
                        rng.uniform(1.0, 2.0, 1 << 18)])
    y, _ = _run("rcp", x)
    assert _ulps(y, 1.0 / x).max() <= 1
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1e308])
    ys, _ = _run("rcp", special)
    with np.errstate(divide="ignore", over="ignore"):
        np.testing.assert_array_equal(ys, 1.0 / special)
