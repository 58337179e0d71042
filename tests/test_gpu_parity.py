"""GPU parity of the plain FP64 path against the FP64 oracle, through the C ABI.

Plain FP64 must match the oracle to a relative error of 1e-12 per output (util.PLAIN_TOL), measured
against each output's condition scale. Every case runs the same seeded cells through the GPU and through
the oracle on the host cores.
"""
import os

import numpy as np
import pytest

import util
from mechanisms import branch_mechanism, cells_for, sri_mechanism

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 4


def _torch():
    import torch
    return torch


def _mech(m):
    import combustion_gb300 as cb
    mech = cb.Mechanism(m)
    from combustion_gb300 import synthetic
    mech.transport_setup(*synthetic.transport_scales(m))
    return mech


def _oracle_for(m, mech):
    import oracle
    from combustion_gb300 import synthetic
    o = oracle.Oracle(m)
    o.set_transport(*synthetic.transport_scales(m), *mech.transport_coefficients())
    return o


def _dev(rows):
    torch = _torch()
    return torch.tensor(np.array(rows), dtype=torch.float64, device="cuda")


def _run_rates(mech, o, cells):
    torch = _torch()
    ins = o.rates_inputs(cells)
    out = torch.empty((mech.A + 2, cells.n), dtype=torch.float64, device="cuda")
    mech.rates(_dev(ins), out)
    torch.cuda.synchronize()
    mech.synchronize()
    ref, scale = o.rates(ins, nthreads=NTHREADS, scale=True)
    return out.cpu().numpy(), ref, scale


def _run_transport(mech, o, cells):
    torch = _torch()
    ins = o.transport_inputs(cells)
    out = torch.empty((mech.K + 2, cells.n), dtype=torch.float64, device="cuda")
    mech.transport(_dev(ins), out)
    torch.cuda.synchronize()
    mech.synchronize()
    ref, scale = o.transport(ins, nthreads=NTHREADS, scale=True)
    return out.cpu().numpy(), ref, scale


def _report(name, x, ref, scale):
    """Prints condition-scaled and pure relative errors per output group, asserts the pure relative
    error on the well-conditioned outputs (on every output for transport), and returns the
    condition-scaled errors."""
    ce = util.cond_err(x, ref, scale)
    transport = name.split()[0] in ("transport", "fused") and "transport" in name
    groups = util.TRANSPORT_GROUPS if transport else util.RATES_GROUPS
    if "reaction rates" in name:
        groups = (("reactions", slice(None)),)
    util.print_groups(name, util.error_groups(x, ref, scale, groups, floored_species=not transport))
    well = util.well_conditioned(ref, scale)
    re = util.rel_err(x, ref)
    print(f"{name}: {100 * well.mean():.2f}% of outputs well conditioned, their rel max "
          f"{re[well].max() if well.any() else 0.0:.2e}; finite {np.isfinite(x).all()}")
    assert re[well].max(initial=0.0) <= util.PLAIN_TOL
    if transport:  # transport outputs barely cancel: the pure relative bar holds on every one of them
        assert re.max() <= util.PLAIN_TOL
    return ce


@pytest.mark.parametrize("config,n", [("k10", 65536), ("k53", 8192), ("k250", 2048)])
def test_rates_parity(config, n):
    from combustion_gb300 import synthetic
    m = util.mechanism(config)
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, n, config)
    x, ref, scale = _run_rates(mech, o, cells)
    ce = _report(f"rates {config}", x, ref, scale)
    assert np.isfinite(x).all()
    assert ce.max() <= util.PLAIN_TOL


@pytest.mark.parametrize("config,n", [("k10", 65536), ("k53", 8192), ("k250", 2048)])
def test_transport_parity(config, n):
    from combustion_gb300 import synthetic
    m = util.mechanism(config)
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, n, config)
    x, ref, scale = _run_transport(mech, o, cells)
    ce = _report(f"transport {config}", x, ref, scale)
    assert np.isfinite(x).all()
    assert ce.max() <= util.PLAIN_TOL


@pytest.mark.parametrize("K", [11, 15])
def test_transport_species_count_3_mod_4(K, monkeypatch):
    """Wilke's mixing rows run in passes of 4, then one of 2 and one of 1: a species count of 3 mod 4 takes
    both remainder passes (10 and 250 take the 2-row pass, 53 the 1-row pass)."""
    from combustion_gb300 import synthetic
    monkeypatch.setitem(synthetic.CONFIGS, f"k{K}", dict(K=K, elementary=2 * K, three_body=4, troe=2))
    m = synthetic.generate_mechanism(f"k{K}")
    assert m.K == K
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(K, 4096, "k10")
    x, ref, scale = _run_transport(mech, o, cells)
    assert _report(f"transport k{K}", x, ref, scale).max() <= util.PLAIN_TOL


def test_branch_mechanism_parity():
    m = branch_mechanism()
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = cells_for(m, 4096)
    x, ref, scale = _run_rates(mech, o, cells)
    assert _report("rates branches", x, ref, scale).max() <= util.PLAIN_TOL
    x, ref, scale = _run_transport(mech, o, cells)
    assert _report("transport branches", x, ref, scale).max() <= util.PLAIN_TOL


def test_sri_mechanism_parity():
    # SRI falloff: the reference's commented formula (reaction.rs:194-203), restated by the oracle
    m = sri_mechanism()
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = cells_for(m, 4096)
    x, ref, scale = _run_rates(mech, o, cells)
    assert _report("rates sri", x, ref, scale).max() <= util.PLAIN_TOL


@pytest.mark.parametrize("n", [0, 1, 31, 127, 129, 1000])
def test_ragged_sizes(n):
    from combustion_gb300 import synthetic
    torch = _torch()
    m = util.mechanism("k10")
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, max(n, 1), "k10", offset=12345)
    ins = [a[:n] for a in o.rates_inputs(cells)]
    guard = 4
    out = torch.full((mech.A + 2, n + guard), 7.0, dtype=torch.float64, device="cuda")
    mech.rates(_dev(ins) if n else [torch.empty(0, dtype=torch.float64, device="cuda")] * (m.K + 3),
               [out[q, :n] for q in range(mech.A + 2)] if n else [out[q, :0] for q in range(mech.A + 2)])
    torch.cuda.synchronize()
    mech.synchronize()
    res = out.cpu().numpy()
    assert (res[:, n:] == 7.0).all(), "kernel wrote past the end of its outputs"
    if n:
        ref, scale = o.rates(ins, scale=True)
        assert util.cond_err(res[:, :n], ref, scale).max() <= util.PLAIN_TOL


def test_host_memory_path_and_uniform_pressure():
    """CB_HOST_MEMORY with more cells than one staging chunk (first and last chunks of one wave, standard
    chunks between, one of them the remainder), and the uniform-pressure constants."""
    from combustion_gb300 import synthetic
    m = util.mechanism("k10")
    mech = _mech(m)
    o = _oracle_for(m, mech)
    n = (1 << 20) + 4321
    cells = synthetic.generate_cells(m.K, n, "k10")  # fixed 1 atm: P/R is uniform
    ins = o.rates_inputs(cells)
    out = np.zeros((mech.A + 2, n))
    mech.rates(np.array(ins), out)
    ref, scale = o.rates(ins, nthreads=NTHREADS, scale=True)
    assert util.cond_err(out, ref, scale).max() <= util.PLAIN_TOL
    uni = [np.array([ins[0][0]]), np.array([ins[1][0]])] + [np.ascontiguousarray(a) for a in ins[2:]]
    assert (ins[0] == ins[0][0]).all()
    out2 = np.zeros_like(out)
    mech.rates(uni, list(out2), uniform_pressure=True)
    assert np.array_equal(out2, out)
    tin = o.transport_inputs(cells)
    tout = np.zeros((mech.K + 2, n))
    mech.transport(np.array(tin), tout)
    tref, tscale = o.transport(tin, nthreads=NTHREADS, scale=True)
    assert util.cond_err(tout, tref, tscale).max() <= util.PLAIN_TOL
    # the fused call on host arrays equals the device call bit for bit
    torch = _torch()
    ro = torch.empty((mech.A + 2, n), dtype=torch.float64, device="cuda")
    to = torch.empty((mech.K + 2, n), dtype=torch.float64, device="cuda")
    mech.rates_transport(_dev(ins), ro, to)
    torch.cuda.synchronize()
    mech.synchronize()
    hro, hto = np.zeros((mech.A + 2, n)), np.zeros((mech.K + 2, n))
    mech.rates_transport(np.array(ins), hro, hto)
    assert np.array_equal(hro, ro.cpu().numpy()) and np.array_equal(hto, to.cpu().numpy())
    assert np.array_equal(hro, out)


def test_errors_are_reported_not_raised_on_device():
    import combustion_gb300 as cb
    m = util.mechanism("k10")
    mech = cb.Mechanism(m)
    torch = _torch()
    ins = torch.zeros((m.K + 1, 4), dtype=torch.float64, device="cuda")
    out = torch.zeros((m.K + 2, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(cb.CombustionError) as e:
        mech.transport(ins, out)
    assert e.value.code == cb.CB_ERR_NOT_READY


@pytest.mark.parametrize("config,n", [("k10", 16384), ("k53", 4096), ("k250", 1024)])
def test_reaction_rates_parity(config, n):
    from combustion_gb300 import synthetic
    torch = _torch()
    m = util.mechanism(config)
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, n, config)
    ins = o.reaction_rates_inputs(cells)
    out = torch.empty((mech.R, n), dtype=torch.float64, device="cuda")
    mech.reaction_rates(_dev(ins), out)
    torch.cuda.synchronize()
    mech.synchronize()
    ref, scale = o.reaction_rates(ins, nthreads=NTHREADS, scale=True)
    assert _report(f"reaction rates {config}", out.cpu().numpy(), ref, scale).max() <= util.PLAIN_TOL


@pytest.mark.parametrize("config,n", [("k10", 16384), ("k53", 4096), ("k250", 2048)])
def test_fused_parity(config, n):
    """cb_rates_transport_f64: rates plus transport at sum n = (P/R V)/T, T/T0, device and host memory."""
    from combustion_gb300 import synthetic
    torch = _torch()
    m = util.mechanism(config)
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, n, config)
    ins = o.rates_inputs(cells)
    ro = torch.empty((mech.A + 2, n), dtype=torch.float64, device="cuda")
    to = torch.empty((mech.K + 2, n), dtype=torch.float64, device="cuda")
    mech.rates_transport(_dev(ins), ro, to)
    torch.cuda.synchronize()
    mech.synchronize()
    rref, tref = o.fused(ins, nthreads=NTHREADS)
    # condition scales from the separate oracle paths on the same derived inputs
    _, rsc = o.rates(ins, nthreads=NTHREADS, scale=True)
    tin = [(ins[0] * ins[3]) / ins[2], ins[2] / o.T0] + ins[4:]
    tref2, tsc = o.transport(tin, nthreads=NTHREADS, scale=True)
    assert np.array_equal(tref, tref2)
    assert _report(f"fused rates {config}", ro.cpu().numpy(), rref, rsc).max() <= util.PLAIN_TOL
    assert _report(f"fused transport {config}", to.cpu().numpy(), tref, tsc).max() <= util.PLAIN_TOL
    hro, hto = np.zeros((mech.A + 2, n)), np.zeros((mech.K + 2, n))
    mech.rates_transport(np.array(ins), hro, hto)
    assert np.array_equal(hro, ro.cpu().numpy()) and np.array_equal(hto, to.cpu().numpy())


def test_count_nonfinite():
    """cb_count_nonfinite (the reference's finite-output assertion, plot.rs:41-46, as a count the caller
    reads): zero on a rates call's outputs; the planted NaN and infinities exactly, on device arrays
    (more arrays than one launch takes) and on host arrays."""
    torch = _torch()
    from combustion_gb300 import synthetic
    m = util.mechanism("k10")
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, 5000, "k10")
    out, _, _ = _run_rates(mech, o, cells)
    dev = torch.tensor(out, device="cuda")
    assert mech.count_nonfinite(dev) == 0
    dev[0, 7] = float("nan")
    dev[3, 4999] = float("inf")
    dev[5, 0] = float("-inf")
    assert mech.count_nonfinite(dev) == 3
    many = torch.zeros((1100, 33), dtype=torch.float64, device="cuda")
    many[1099, 32] = float("nan")
    many[0, 0] = float("nan")
    many[600, 5] = float("inf")
    assert mech.count_nonfinite(many) == 3
    host = dev.cpu().numpy()
    assert mech.count_nonfinite(host) == 3


def test_staging_timeout_is_reported_and_cleared():
    """The bounded wait on the table staging copy, made to run out (cb_debug_stage_wait_polls(0)):
    the kernels return without computing, the call reports CB_ERR_DEVICE, and once the wait is back to
    its default the next call on the same mechanism and context succeeds with the oracle's values. The
    copy itself always lands (the second wait keeps the full limit), so no block exits with a copy in
    flight."""
    import combustion_gb300 as cb
    from combustion_gb300 import synthetic
    torch = _torch()
    m = util.mechanism("k10")
    mech = _mech(m)
    o = _oracle_for(m, mech)
    cells = synthetic.generate_cells(m.K, 4096, "k10")
    ins = _dev(o.rates_inputs(cells))
    out = torch.full((mech.A + 2, cells.n), 7.0, dtype=torch.float64, device="cuda")
    try:
        cb.debug_stage_wait_polls(0)
        mech.rates(ins, out)
        with pytest.raises(cb.CombustionError) as e:
            mech.synchronize()
        assert e.value.code == cb.CB_ERR_DEVICE and "staging" in str(e.value)
        assert (out.cpu().numpy() == 7.0).all()  # nothing was computed
    finally:
        cb.debug_stage_wait_polls(-1)
    mech.rates(ins, out)
    mech.synchronize()
    ref, scale = o.rates(o.rates_inputs(cells), scale=True)
    assert util.cond_err(out.cpu().numpy(), ref, scale).max() <= util.PLAIN_TOL
