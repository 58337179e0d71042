"""The learned transport surrogate through the C ABI: the device cell generator against the host one,
the tcgen05 GEMM forward and backward against the FP64 network restatement (oracle/mlp.py), training,
the trust gate and audit, the ensemble gate with a calibrated error bound, and what the trained network
gains over the plain and mixed-precision transport kernels.

Stated error bars: network outputs within 2e-3 and gradients within 1e-2 (norm-relative, per layer) of
the restatement that rounds the same values to BF16; within 3e-2 / 6e-2 of the unrounded FP64 network.
"""
import time

import numpy as np
import pytest

import util
from oracle import mlp

pytestmark = pytest.mark.gpu


def _mech(config):
    import combustion_gb300 as cb
    from combustion_gb300 import synthetic
    m = util.mechanism(config)
    mech = cb.Mechanism(m)
    mech.transport_setup(*synthetic.transport_scales(m))
    return mech


def _nrel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_device_cells_match_host_generator():
    from combustion_gb300 import surrogate as S
    from combustion_gb300 import synthetic
    m = util.mechanism("k53")
    mech = _mech("k53")
    n = 4096
    dev = S.generate_cells(mech, n, S.distribution("k53", seed=1)).cpu().numpy()
    host = synthetic.generate_cells(m.K, n, "k53", seed=1)
    assert np.allclose(dev[2], host.temperature, rtol=1e-14, atol=0)
    assert np.allclose(dev[0], host.pressure_R, rtol=1e-12, atol=0)
    assert np.array_equal(dev[3], host.volume)
    rel = np.abs(dev[4:] - host.amounts) / np.maximum(np.abs(host.amounts), 1e-300)
    # CUDA's and glibc's log/cos/exp differ in the last bits; a rejection test can then rarely flip
    assert np.mean(rel < 1e-9) > 0.999, np.mean(rel < 1e-9)


@pytest.mark.parametrize("hidden,rows", [(2, 512), (4, 1024)])
def test_forward_backward_against_restatement(hidden, rows):
    from combustion_gb300 import surrogate as S
    mech = _mech("k10")
    s = S.Surrogate(mech, width=256, hidden_layers=hidden, batch=1024, seed=11)
    info = s.info
    rng = np.random.default_rng(hidden)
    p = s.params()
    # random weights with realistic scale everywhere a gradient flows (padding stays zero)
    layers = s.layers(p)
    nf = info.n_features
    for l, (W, b) in enumerate(layers):
        fan_in = nf if l == 0 else W.shape[1]
        rows_l = nf if l == len(layers) - 1 else W.shape[0]
        cols_l = nf if l == 0 else W.shape[1]
        W[:rows_l, :cols_l] = rng.normal(0, 1.2 / np.sqrt(fan_in), (rows_l, cols_l))
        b[:rows_l] = rng.normal(0, 0.1, rows_l)
    s.set_params(p)
    X = np.zeros((rows, info.n_in), np.float32)
    X[:, :nf] = rng.normal(size=(rows, nf))
    T = np.zeros((rows, info.n_out), np.float32)
    T[:, :nf] = rng.normal(size=(rows, nf))
    loss, g, Y = s.evaluate(X, T)
    layers = s.layers(s.params().astype(np.float64))
    lb, gb, Yb = mlp.loss_and_grads(layers, X, T, nf, bf=True)
    l64, g64, Y64 = mlp.loss_and_grads(layers, X, T, nf, bf=False)
    e_out = _nrel(Y[:, :nf], Yb[:, :nf])
    print(f"hidden {hidden}: outputs {e_out:.2e} (vs FP64 {_nrel(Y[:, :nf], Y64[:, :nf]):.2e}); loss {loss:.6f} "
          f"restatement {lb:.6f}")
    assert e_out < 2e-3
    assert _nrel(Y[:, :nf], Y64[:, :nf]) < 3e-2
    assert abs(loss - lb) <= 2e-3 * lb
    gl = s.layers(g.astype(np.float64))
    for l in range(len(layers)):
        for k, name in ((0, "W"), (1, "b")):
            e_b, e_64 = _nrel(gl[l][k], gb[l][k]), _nrel(gl[l][k], g64[l][k])
            print(f"  layer {l} d{name}: {e_b:.2e} (vs FP64 {e_64:.2e})")
            assert e_b < 1e-2, (l, name, e_b)
            assert e_64 < 6e-2, (l, name, e_64)


def _plain_transport(mech, cells):
    import torch
    K, A, n = mech.K, mech.A, cells.shape[1]
    rates = torch.empty((A + 2, n), dtype=torch.float64, device="cuda")
    tr = torch.empty((K + 2, n), dtype=torch.float64, device="cuda")
    mech.rates_transport(cells, rates, tr)
    torch.cuda.synchronize()
    return tr


def _trained(config, n_train, steps, batch, width=256, seed=3):
    from combustion_gb300 import surrogate as S
    mech = _mech(config)
    s = S.Surrogate(mech, width=width, hidden_layers=4, batch=batch, lr=2e-3, lr_final=1e-4, seed=seed)
    s.generate(n_train, S.distribution(config, seed=2))
    untrained = s.params()
    losses = s.train(steps)
    return mech, s, untrained, losses


def test_training_gate_and_audit():
    import torch
    from combustion_gb300 import surrogate as S
    mech, s, untrained, losses = _trained("k10", 1 << 17, 400, 8192)
    print("loss", losses[0], "->", losses[-1])
    assert np.all(np.isfinite(losses)) and losses[-1] < losses[0] / 20
    n = 1 << 16
    cells = S.generate_cells(mech, n, S.distribution("k10", seed=7))
    plain = _plain_transport(mech, cells)
    out = torch.empty_like(plain)
    st = s.transport(cells, out, gate=False)
    assert st["fallback_cells"] == 0
    err = (out - plain).abs() / plain.abs()
    trained_rms = float(err.pow(2).mean().sqrt())
    s2 = S.Surrogate(mech, width=256, hidden_layers=4, batch=8192, seed=3)
    s2.generate(1 << 14, S.distribution("k10", seed=2))
    s2.set_params(untrained)
    out2 = torch.empty_like(plain)
    s2.transport(cells, out2, gate=False)
    untrained_rms = float(((out2 - plain).abs() / plain.abs()).pow(2).mean().sqrt())
    print(f"rms rel error: trained {trained_rms:.2e}, untrained {untrained_rms:.2e}; max {float(err.max()):.2e}")
    assert trained_rms < untrained_rms / 10
    # gate: cells outside the training temperatures go to the plain kernel, bit for bit
    cells[2, : n // 4] = 3500.0
    plain = _plain_transport(mech, cells)
    out = torch.empty_like(plain)
    st = s.transport(cells, out, audit_stride=64)
    print(st)
    assert st["fallback_cells"] >= n // 4
    assert torch.equal(out[:, : n // 4], plain[:, : n // 4])
    assert st["audited_cells"] > 0
    assert st["audit_max_rel_err"][2] <= float(err.max()) * 4 + 1e-3
    # every cell is either the network's or the plain kernel's value
    same = (out == plain).all(dim=0)
    assert int(same.sum()) >= st["fallback_cells"] + st["audited_cells"]


@pytest.mark.parametrize("config,width", [("k53", 256), ("k250", 512)])
def test_gate_fallback_warp_per_cell_matches_plain_kernel(config, width):
    """Above 16 species the gate's few fallback and audit cells run one cell per warp; those cells equal
    the one-cell-per-thread kernel's outputs bit for bit, and so do the plain values of audited cells."""
    import torch
    from combustion_gb300 import surrogate as S
    mech = _mech(config)
    s = S.Surrogate(mech, width=width, hidden_layers=2, batch=1024, seed=3)
    s.generate(1 << 13, S.distribution(config, seed=2))
    n = 4096
    cells = S.generate_cells(mech, n, S.distribution(config, seed=7))
    cells[2, : n // 8] = 3500.0  # above the training temperatures
    cells[2, n // 8 : n // 8 + 3] = 250.0  # below them
    plain = _plain_transport(mech, cells)  # not gathered: one cell per thread
    out = torch.empty_like(plain)
    st = s.transport(cells, out, audit_stride=16)
    print(config, st)
    assert n // 8 + 3 <= st["fallback_cells"] <= n // 4  # a small gathered launch: warp per cell
    assert torch.equal(out[:, : n // 8 + 3], plain[:, : n // 8 + 3])
    # audited cells get their plain values from the warp-per-cell kernel in compact order: equal too
    same = (out == plain).all(dim=0)
    assert st["audited_cells"] > 0
    assert int(same.sum()) >= st["fallback_cells"] + st["audited_cells"]
    # the audit's error is the network's against those values: bounded by the error over every cell
    # that holds a plain value outside the forced fallbacks (the audited ones and any natural fallback)
    net = torch.empty_like(plain)
    s.transport(cells, net, gate=False)
    idx = torch.nonzero(same[n // 8 + 3 :]).squeeze(1) + n // 8 + 3
    err = (net[:, idx] - plain[:, idx]).abs() / plain[:, idx].abs()
    assert st["audit_max_rel_err"][2] <= float(err[2:].max()) * (1 + 1e-6)


def _timed(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(reps):
        fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t) / reps


def test_trained_network_gain_over_plain_and_mixed_kernels():
    """What the trained network gains: transport cells/s through the gated surrogate against the plain
    FP64 kernel and the mixed-precision kernel on the same cells (53 species), with its error against the
    plain kernel over every cell. The single-network gate (training range only) bounds nothing: the
    error is reported, and test_ensemble_gate_calibrated_bound states a bound."""
    import torch
    from combustion_gb300 import surrogate as S
    mech, s, _, losses = _trained("k53", 1 << 18, 300, 16384)
    n = 1 << 20
    cells = S.generate_cells(mech, n, S.distribution("k53", seed=9))
    out = torch.empty((mech.K + 2, n), dtype=torch.float64, device="cuda")
    K = mech.K
    tin = torch.empty((K + 1, n), dtype=torch.float64, device="cuda")
    T0 = mech.info.T0
    tin[0] = cells[0] * cells[3] / cells[2]
    tin[1] = cells[2] / T0
    tin[2:] = cells[4:]
    plain, mixed = torch.empty_like(out), torch.empty_like(out)
    t_plain = _timed(lambda: mech.transport(tin, plain))
    t_mixed = _timed(lambda: mech.transport(tin, mixed, mixed=True))
    stats = {}
    t_sur = _timed(lambda: stats.update(s.transport(cells, out, audit_stride=1024)))
    err = (out - plain).abs() / plain.abs()
    err_mixed = float(((mixed - plain).abs() / plain.abs()).max())
    print(f"plain {n / t_plain:.3e} cells/s, mixed {n / t_mixed:.3e} cells/s (max rel err {err_mixed:.1e}), "
          f"surrogate {n / t_sur:.3e} cells/s ({t_plain / t_sur:.1f}x plain, {t_mixed / t_sur:.2f}x mixed); "
          f"rms rel err {float(err.pow(2).mean().sqrt()):.2e}, max {float(err.max()):.2e}, audit {stats}")
    assert t_sur < t_plain
    assert err_mixed < 1e-5
    assert stats["audited_cells"] > 0


def test_ensemble_gate_calibrated_bound():
    """Two networks trained from different initial weights; their disagreement is each cell's error
    estimate. A threshold calibrated on 2^20 cells for half the stated error (0.2 here, for networks
    trained 1,500 steps) keeps every one of 2^18 fresh cells within the stated error: the cells above it
    go to the mixed-precision kernel. At 1e-4 (the mixed form's bar) no calibration cell of these
    networks is accurate enough: every cell falls back, the networks are skipped, and the outputs are the
    mixed kernel's, bit for bit."""
    import torch
    from combustion_gb300 import surrogate as S
    mech, a, _, _ = _trained("k53", 1 << 20, 1500, 16384, seed=3)
    b = S.Surrogate(mech, width=256, hidden_layers=4, batch=16384, lr=2e-3, lr_final=1e-4, seed=4)  # same mechanism
    b.generate(1 << 20, S.distribution("k53", seed=2))
    b.train(1500)
    K = mech.K

    def reference(cells, mixed):
        tr = torch.empty((K + 2, cells.shape[1]), dtype=torch.float64, device="cuda")
        rr = torch.empty((mech.A + 2, cells.shape[1]), dtype=torch.float64, device="cuda")
        mech.rates_transport(cells, rr, tr, mixed=mixed)
        return tr

    cal = S.generate_cells(mech, 1 << 20, S.distribution("k53", seed=11))
    out = torch.empty((K + 2, cal.shape[1]), dtype=torch.float64, device="cuda")
    d = torch.empty(cal.shape[1], dtype=torch.float32, device="cuda")
    st = S.transport_pair(a, b, cal, out, float("inf"), audit_stride=0, disagreement=d)
    err = S.max_rel_err_per_cell(out, reference(cal, False))
    assert bool(err.isfinite().all()) and bool(d.isfinite().all())
    print(f"calibration: median max rel err {float(err.median()):.2e}, disagreement median {float(d.median()):.2e}, "
          f"correlation of logs {float(torch.corrcoef(torch.stack([d.double().log(), err.log()]))[0, 1]):.2f}, "
          f"range fallbacks {st['fallback_cells']}")
    test = S.generate_cells(mech, 1 << 18, S.distribution("k53", seed=13))
    plain = reference(test, False)
    for tol in (0.2, 1e-4):
        t = S.calibrate_threshold(d, err, tol / 2)
        res = torch.empty_like(plain)
        st = S.transport_pair(a, b, test, res, t, audit_stride=256)
        e = S.max_rel_err_per_cell(res, plain)
        frac = st["fallback_cells"] / test.shape[1]
        print(f"stated {tol:g}: threshold {t:.3e}, fallback {100 * frac:.3f}%, max rel err {float(e.max()):.2e}, "
              f"audit {st['audit_max_rel_err']}")
        assert float(e.max()) <= tol
        if tol == 1e-4:
            assert t == float("-inf") and st["fallback_cells"] == test.shape[1]
            assert torch.equal(res, reference(test, True))
        else:
            assert 0.0 < frac < 1.0


def test_ensemble_rejects_bad_arguments():
    """cb_surrogate_transport_pair refuses one network twice, networks of two mechanisms, a NaN
    threshold and an unknown fallback kernel, with CB_ERR_INVALID and a message; nothing is launched."""
    import ctypes as C
    import torch
    import combustion_gb300 as cb
    from combustion_gb300 import surrogate as S
    mech = _mech("k10")
    a = S.Surrogate(mech, width=256, hidden_layers=2, batch=1024, seed=3)
    a.generate(1 << 12, S.distribution("k10", seed=2))
    b = S.Surrogate(mech, width=256, hidden_layers=2, batch=1024, seed=4)
    b.generate(1 << 12, S.distribution("k10", seed=2))
    other = S.Surrogate(_mech("k10"), width=256, hidden_layers=2, batch=1024, seed=5)
    other.generate(1 << 12, S.distribution("k10", seed=2))
    cells = S.generate_cells(mech, 256, S.distribution("k10", seed=7))
    out = torch.zeros((mech.K + 2, 256), dtype=torch.float64, device="cuda")
    for x, y, thr, fb in ((a, a, 1.0, "mixed"), (a, other, 1.0, "mixed"), (a, b, float("nan"), "mixed")):
        with pytest.raises(cb.CombustionError) as e:
            S.transport_pair(x, y, cells, out, thr, fallback=fb)
        assert e.value.code == cb.CB_ERR_INVALID, str(e.value)
    L = S._bind()
    ins, _ = cb.Mechanism._rows(cells)
    outs, n = cb.Mechanism._rows(out)
    g = S.cb_surrogate_gate(1.0, 0, 7, None)  # no such fallback kernel
    rc = L.cb_surrogate_transport_pair(a.h, b.h, n, cb._ptr_array(ins), cb._ptr_array(outs), 0, C.byref(g), None,
                                       None)
    assert rc == cb.CB_ERR_INVALID and b"fallback" in L.cb_last_error()
    assert bool((out == 0).all())
