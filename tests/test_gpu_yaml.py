"""A Cantera-YAML mechanism through the GPU kernels (the role of yaml.rs:54-171 and lib.rs:127-140):
a hand-written file is read by cb_yaml_load, its arrays go to cb_mech_create, and the plain and mixed
rates, per-reaction rates and transport are compared with the FP64 oracle built from the same arrays.

The file (tests/test_yaml.py's HANDWRITTEN, plus a Troe reaction with a T2 term and an SRI reaction)
covers: activation energies in cal/mol (and, in the second case, the same file in K), an inert species
listed before the active ones (moved after them, yaml.rs:159-162), a species whose two NASA-7 pieces
are equal (merged into one, yaml.rs:64-77), a species with a single temperature range, an irreversible
reaction, a three-body reaction with efficiencies, Lindemann falloff (no Troe block, yaml.rs:147),
Troe with and without T2, a pressure-dependent-Arrhenius reaction with one rate (yaml.rs:148-153), a
duplicate reaction, and SRI falloff.
"""
import os
import re

import numpy as np
import pytest

import util
from combustion_gb300 import synthetic
from test_yaml import HANDWRITTEN, SRI_REACTION

NTHREADS = os.cpu_count() or 4

TROE_T2 = """\
- equation: O + OH (+M) <=> HO2 (+M)
  type: falloff
  low-P-rate-constant: {A: 1.2e+19, b: -1.2, Ea: 0.0}
  high-P-rate-constant: {A: 3.1e+12, b: 0.2, Ea: 350.0}
  Troe: {A: 0.7, T3: 120.0, T1: 1800.0, T2: 5200.0}
  efficiencies: {AR: 0.6, H2O: 11.0}
"""

FILE_CAL = HANDWRITTEN + TROE_T2 + SRI_REACTION


def in_kelvin(text):
    """The same file with activation energies in K (Ea / R)."""
    text = text.replace("activation-energy: cal/mol", "activation-energy: K")
    return re.sub(r"Ea: (-?[0-9.e+-]+)", lambda m: f"Ea: {float(m.group(1)) * 4.184 / synthetic.R!r}", text)


def _load(text):
    from combustion_gb300 import build, cantera_yaml
    build.build()
    return cantera_yaml.load(text)


def test_yaml_file_is_complete():
    """CPU: the file holds every model the GPU cases run (irreversible, elementary, three-body, Troe,
    Lindemann, SRI) and validates; K units give the same arrays as cal/mol up to the last bits."""
    import combustion_gb300 as cb
    m = _load(FILE_CAL)
    assert set(m.model.tolist()) == {0, 1, 2, 3, 4, 5}
    assert np.isfinite(m.troe[m.model == 4, 3]).sum() == 1  # one Troe with T2, one without
    assert cb.validate(m).n_active == 7
    mk = _load(in_kelvin(FILE_CAL))
    assert np.allclose(mk.rate, m.rate, rtol=1e-14, atol=0) and np.allclose(mk.k0, m.k0, rtol=1e-14, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("units", ["cal/mol", "K"])
def test_yaml_mechanism_on_gpu(units):
    import torch
    import combustion_gb300 as cb
    import oracle
    m = _load(FILE_CAL if units == "cal/mol" else in_kelvin(FILE_CAL))
    mech = cb.Mechanism(m)
    scales = synthetic.transport_scales(m)  # fuel H2, oxidiser O2, diluent N2 (the last species)
    mech.transport_setup(*scales)
    o = oracle.Oracle(m)
    o.set_transport(*scales, *mech.transport_coefficients())
    cells = synthetic.generate_cells(m.K, 8192, "k10", seed=9)
    dev = lambda rows: torch.tensor(np.array(rows), dtype=torch.float64, device="cuda")

    rin, tin, qin = o.rates_inputs(cells), o.transport_inputs(cells), o.reaction_rates_inputs(cells)
    rref, rsc = o.rates(rin, nthreads=NTHREADS, scale=True)
    tref, tsc = o.transport(tin, nthreads=NTHREADS, scale=True)
    qref, qsc = o.reaction_rates(qin, nthreads=NTHREADS, scale=True)
    for mixed, tol in ((False, util.PLAIN_TOL), (True, util.MIXED_TOL)):
        r = torch.empty((mech.A + 2, cells.n), dtype=torch.float64, device="cuda")
        t = torch.empty((mech.K + 2, cells.n), dtype=torch.float64, device="cuda")
        mech.rates(dev(rin), r, mixed=mixed)
        mech.transport(dev(tin), t, mixed=mixed)
        torch.cuda.synchronize()
        mech.synchronize()
        r, t = r.cpu().numpy(), t.cpu().numpy()
        name = f"yaml ({units}) {'mixed' if mixed else 'plain'}"
        util.print_groups(name + " rates", util.error_groups(r, rref, rsc, util.RATES_GROUPS, floored_species=True))
        util.print_groups(name + " transport", util.error_groups(t, tref, tsc, util.TRANSPORT_GROUPS))
        assert np.isfinite(r).all() and np.isfinite(t).all()
        assert util.cond_err(r, rref, rsc).max() <= tol
        assert util.cond_err(t, tref, tsc).max() <= tol
    q = torch.empty((mech.R, cells.n), dtype=torch.float64, device="cuda")
    mech.reaction_rates(dev(qin), q)
    torch.cuda.synchronize()
    assert util.cond_err(q.cpu().numpy(), qref, qsc).max() <= util.PLAIN_TOL
