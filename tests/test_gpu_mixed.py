"""The mixed-precision form against the FP64 oracle, through the C ABI.

Stated error bar: 1e-4 per output, relative to the output's condition scale (the metric of the plain
form's 1e-12 bar). Max and RMS errors per output group are printed: condition-scaled, pure relative,
and for species rates the reference's floored metric |x - r| / max(r, 1e3) (cantera.rs:147). Transport
outputs barely cancel, so their pure relative error is asserted at the same 1e-4 bar.
"""
import os

import numpy as np
import pytest

import util
from mechanisms import branch_mechanism, cells_for, sri_mechanism

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 4
MIXED_TOL = util.MIXED_TOL


def _setup(m):
    import combustion_gb300 as cb
    import oracle
    from combustion_gb300 import synthetic
    mech = cb.Mechanism(m)
    scales = synthetic.transport_scales(m)
    mech.transport_setup(*scales)
    o = oracle.Oracle(m)
    o.set_transport(*scales, *mech.transport_coefficients())
    return mech, o


def _dev(rows):
    import torch
    return torch.tensor(np.array(rows), dtype=torch.float64, device="cuda")


def _report(name, x, ref, scale):
    """Condition-scaled error, pure relative error (max and RMS, unclipped) and, for species rates, the
    reference's floored metric; returns the condition-scaled errors."""
    ce = util.cond_err(x, ref, scale)
    re = util.rel_err(x, ref)
    line = (f"{name}: cond err max {ce.max():.2e} rms {np.sqrt((ce ** 2).mean()):.2e}; "
            f"rel err max {re.max():.2e} rms {np.sqrt((re ** 2).mean()):.2e}")
    if "species" in name:
        fe, fa = util.floored_err(x, ref), util.floored_abs_err(x, ref)
        line += (f"; floored max {fe.max():.2e} rms {np.sqrt((fe ** 2).mean()):.2e}"
                 f" (on |r|: max {fa.max():.2e} rms {np.sqrt((fa ** 2).mean()):.2e})")
    print(line)
    return ce


@pytest.mark.parametrize("config,n", [("k10", 65536), ("k53", 16384), ("k250", 2048)])
def test_mixed_rates_and_transport(config, n):
    import torch
    from combustion_gb300 import synthetic
    m = util.mechanism(config)
    mech, o = _setup(m)
    cells = synthetic.generate_cells(m.K, n, config)
    rin, tin = o.rates_inputs(cells), o.transport_inputs(cells)
    r = torch.empty((mech.A + 2, n), dtype=torch.float64, device="cuda")
    t = torch.empty((mech.K + 2, n), dtype=torch.float64, device="cuda")
    mech.rates(_dev(rin), r, mixed=True)
    mech.transport(_dev(tin), t, mixed=True)
    torch.cuda.synchronize()
    mech.synchronize()
    rref, rsc = o.rates(rin, nthreads=NTHREADS, scale=True)
    tref, tsc = o.transport(tin, nthreads=NTHREADS, scale=True)
    rr, tt = r.cpu().numpy(), t.cpu().numpy()
    assert np.isfinite(rr).all() and np.isfinite(tt).all()
    assert _report(f"mixed rates {config} dT/dt, dV/dt", rr[:2], rref[:2], rsc[:2]).max() <= MIXED_TOL
    assert _report(f"mixed rates {config} species", rr[2:], rref[2:], rsc[2:]).max() <= MIXED_TOL
    assert _report(f"mixed transport {config} lambda", tt[:1], tref[:1], tsc[:1]).max() <= MIXED_TOL
    assert _report(f"mixed transport {config} mu", tt[1:2], tref[1:2], tsc[1:2]).max() <= MIXED_TOL
    assert _report(f"mixed transport {config} rhoD", tt[2:], tref[2:], tsc[2:]).max() <= MIXED_TOL
    assert util.rel_err(tt, tref).max() <= MIXED_TOL


@pytest.mark.parametrize("name", ["branches", "sri"])
def test_mixed_branch_mechanism_and_fused_host_path(name):
    import torch
    m = branch_mechanism() if name == "branches" else sri_mechanism()
    mech, o = _setup(m)
    cells = cells_for(m, 4096)
    rin = o.rates_inputs(cells)
    ro, to = np.zeros((mech.A + 2, cells.n)), np.zeros((mech.K + 2, cells.n))
    mech.rates_transport(np.array(rin), ro, to, mixed=True)
    rref, rsc = o.rates(rin, scale=True)
    tin = [(rin[0] * rin[3]) / rin[2], rin[2] / o.T0] + rin[4:]
    tref, tsc = o.transport(tin, scale=True)
    assert _report(f"mixed fused rates {name}", ro, rref, rsc).max() <= MIXED_TOL
    assert _report(f"mixed fused transport {name}", to, tref, tsc).max() <= MIXED_TOL
    d_r = torch.empty((mech.A + 2, cells.n), dtype=torch.float64, device="cuda")
    d_t = torch.empty((mech.K + 2, cells.n), dtype=torch.float64, device="cuda")
    mech.rates_transport(_dev(rin), d_r, d_t, mixed=True)
    torch.cuda.synchronize()
    assert np.array_equal(d_r.cpu().numpy(), ro) and np.array_equal(d_t.cpu().numpy(), to)
