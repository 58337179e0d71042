"""Edge-case inputs of the reference program through the GPU kernels, against the FP64 oracle.

The seeded generator only draws T in [300, 3000] K and strictly positive Dirichlet amounts. These cells
reach the places where the reference clamps or selects, which the kernels implement with integer
compares on bit patterns:
  - T exactly at the NASA-7 split and one ulp either side (piece 0 for T <= split: lib.rs:15,
    interpret.rs:75-76);
  - negative and zero amounts (max(0, n): reaction.rs:339,366), all amounts zero but the bulk species,
    and a negative bulk concentration (C_bulk = C - sum C_k: reaction.rs:372);
  - T outside the transport fit range [300, 3000] K (transport.rs:127), and at its ends;
  - a subnormal amount;
  - rate constants that saturate at f32::MAX (reaction.rs:138), including the no-exponential form and
    a low-pressure falloff coefficient, and Gibbs exponentials clamped at M3 and cbrt(f32::MAX)
    (reaction.rs:244-262; reached at 250 K).
Each runs through both table placements: K = 10 and 53 (tables staged in shared memory, KMAX 16 and
64) and K = 250 (tables read through L1, KMAX 256), in the plain and the mixed form.
"""
import copy
import os

import numpy as np
import pytest

import util
from combustion_gb300 import synthetic

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 4
F32_MAX = float(np.finfo(np.float32).max)
SPLIT = 1000.0  # the generator's NASA-7 split


def edge_cells(K, config):
    """About 30 cells, each one edge case, in the generator's input layout; returns (cells, labels)."""
    base = synthetic.generate_cells(K, 3, config, seed=21)
    X = np.vstack([base.amounts, base.total_amount - base.amounts.sum(0)]) / base.total_amount  # [K, 3]
    rows, labels = [], []

    def add(label, T, pR, amounts=None, x=None, total=None):
        tot = pR / T if total is None else total  # V = 1 m^3
        a = (x[:K - 1] * tot) if amounts is None else amounts
        rows.append((pR, T, 1.0, np.array(a, dtype=np.float64), tot))
        labels.append(label)

    pR = base.pressure_R
    lo, hi = np.nextafter(SPLIT, 0.0), np.nextafter(SPLIT, np.inf)
    for c in range(2):
        for T, name in ((SPLIT, "T = split"), (lo, "T = split - 1 ulp"), (hi, "T = split + 1 ulp")):
            add(f"{name} #{c}", T, pR[c], x=X[:, c])
    for T in (250.0, 300.0, 3000.0, 3200.0):
        add(f"T = {T:g} K", T, pR[2], x=X[:, 2])
    for k in (0, K // 3, K - 2):
        a = X[:K - 1, 0] * (pR[0] / 1500.0)
        neg, zero = a.copy(), a.copy()
        neg[k] = -0.3 * pR[0] / 1500.0
        zero[k] = 0.0
        add(f"n_{k} < 0", 1500.0, pR[0], amounts=neg)
        add(f"n_{k} = 0", 1500.0, pR[0], amounts=zero)
    for T in (1500.0, 250.0):
        add(f"only bulk, T = {T:g}", T, pR[1], amounts=np.zeros(K - 1))
    for T in (900.0, 2400.0):
        a = X[:K - 1, 1] / X[:K - 1, 1].sum() * (1.2 * pR[1] / T)  # sum n_k = 1.2 n: bulk at -0.2 n
        add(f"negative bulk, T = {T:g}", T, pR[1], amounts=a)
    a = X[:K - 1, 2] * (pR[2] / 1800.0)
    a[1] = 5e-320
    add("subnormal amount", 1800.0, pR[2], amounts=a)
    cells = synthetic.Cells(pressure_R=np.array([r[0] for r in rows]), temperature=np.array([r[1] for r in rows]),
                            volume=np.array([r[2] for r in rows]),
                            amounts=np.ascontiguousarray(np.array([r[3] for r in rows]).T),
                            total_amount=np.array([r[4] for r in rows]))
    return cells, labels


def saturating_mechanism(config):
    """The generator's mechanism with rate constants that saturate at f32::MAX: an irreversible reaction
    with A = 1e40 and no exponential (k = min(f32::MAX, A)), a reversible one with A = 1e36, b = 1 (the
    exponential form, saturated above about 1,300 K), a three-body reaction with A = 1e43 / T, and a
    Troe reaction whose low-pressure A is 1e45."""
    m = copy.deepcopy(util.mechanism(config))
    model = np.asarray(m.model)
    # the irreversible one first: an elementary reaction whose reactants do not include the bulk species
    elem = sorted(np.flatnonzero(model == synthetic.ELEMENTARY), key=lambda r: m.reactants[r, m.K - 1] != 0)
    tb = np.flatnonzero(model == synthetic.THREE_BODY)
    troe = np.flatnonzero(model == synthetic.TROE)
    m.model[elem[0]] = synthetic.IRREVERSIBLE
    m.rate[elem[0]] = (1e40, 0.0, 0.0)
    m.rate[elem[1]] = (1e36, 1.0, 1000.0)
    m.rate[tb[0]] = (1e43, -1.0, 0.0)
    m.k0[troe[0]] = (1e45, 0.0, 0.0)
    m.meta = {"config": config + "-saturating"}
    return m, int(elem[0])


def _setup(m, transport=True):
    import combustion_gb300 as cb
    import oracle
    mech = cb.Mechanism(m)
    o = oracle.Oracle(m)
    if transport:
        scales = synthetic.transport_scales(m)
        mech.transport_setup(*scales)
        o.set_transport(*scales, *mech.transport_coefficients())
    return mech, o


def _dev(rows):
    import torch
    return torch.tensor(np.array(rows), dtype=torch.float64, device="cuda")


def _rates(mech, ins, mixed=False):
    import torch
    out = torch.empty((mech.A + 2, len(ins[0])), dtype=torch.float64, device="cuda")
    mech.rates(_dev(ins), out, mixed=mixed)
    torch.cuda.synchronize()
    mech.synchronize()
    return out.cpu().numpy()


def _transport(mech, ins, mixed=False):
    import torch
    out = torch.empty((mech.K + 2, len(ins[0])), dtype=torch.float64, device="cuda")
    mech.transport(_dev(ins), out, mixed=mixed)
    torch.cuda.synchronize()
    mech.synchronize()
    return out.cpu().numpy()


def _check(name, x, ref, scale, labels, tol):
    """Non-finite values exactly where the oracle has them, the condition-scaled bar on the rest; the
    worst cell is named. (Only the bulk species' diffusion of a cell whose other amounts are all zero is
    non-finite: the reference's formula divides by its empty mixing sum. Its sign or NaN-ness depends on
    the last bit of a cancelling numerator, so only its non-finiteness is compared.)"""
    assert np.array_equal(np.isfinite(x), np.isfinite(ref)), name
    bad = ~np.isfinite(ref)
    e = np.where(bad, 0.0, util.cond_err(np.where(bad, 0.0, x), np.where(bad, 0.0, ref), scale))
    worst = np.unravel_index(np.argmax(e), e.shape)
    print(f"{name}: max cond err {e.max():.2e} (output {worst[0]}, cell '{labels[worst[1]]}'), "
          f"{int(bad.sum())} non-finite in the oracle")
    assert e.max() <= tol, (name, labels[worst[1]])


@pytest.mark.parametrize("config", ["k10", "k53", "k250"])
@pytest.mark.parametrize("mixed", [False, True], ids=["plain", "mixed"])
def test_edge_inputs(config, mixed):
    m = util.mechanism(config)
    mech, o = _setup(m)
    cells, labels = edge_cells(m.K, config)
    tol = util.MIXED_TOL if mixed else util.PLAIN_TOL
    rin, tin = o.rates_inputs(cells), o.transport_inputs(cells)
    r = _rates(mech, rin, mixed)
    rref, rsc = o.rates(rin, nthreads=NTHREADS, scale=True)
    _check(f"{'mixed' if mixed else 'plain'} rates {config}", r, rref, rsc, labels, tol)
    t = _transport(mech, tin, mixed)
    tref, tsc = o.transport(tin, nthreads=NTHREADS, scale=True)
    _check(f"{'mixed' if mixed else 'plain'} transport {config}", t, tref, tsc, labels, tol)

    # The piece select is exercised: the oracle's outputs one ulp either side of the split differ far
    # beyond the bar, and the kernels agree with the oracle on both sides (above).
    i_lo, i_hi = labels.index("T = split - 1 ulp #0"), labels.index("T = split + 1 ulp #0")
    assert util.rel_err(rref[:, i_lo], rref[:, i_hi]).max() > 1e-8
    # max(0, n): a negative amount gives exactly the outputs of a zero amount.
    for k in (0, m.K // 3, m.K - 2):
        a, b = labels.index(f"n_{k} < 0"), labels.index(f"n_{k} = 0")
        assert np.array_equal(r[:, a], r[:, b]), k
        assert np.array_equal(rref[:, a], rref[:, b]), k
    # Clamped Gibbs exponentials are reached at 250 K (|g/RT| above ln M3) by the generator's enthalpies.
    assert np.isfinite(r[:, labels.index("T = 250 K")]).all()


@pytest.mark.parametrize("config", ["k10", "k53", "k250"])
@pytest.mark.parametrize("mixed", [False, True], ids=["plain", "mixed"])
def test_saturated_rate_constants(config, mixed):
    """k = min(f32::MAX, k) in every Arrhenius form, on generator cells and the edge cells; per-reaction
    rates (plain form) of the irreversible A = 1e40 reaction are f32::MAX times its concentration
    product, exactly."""
    import torch
    m, r_irr = saturating_mechanism(config)
    mech, o = _setup(m, transport=False)
    cells, labels = edge_cells(m.K, config)
    gen = synthetic.generate_cells(m.K, 512, config, seed=5)
    for c in (cells, gen):
        rin = o.rates_inputs(c)
        lab = labels if c is cells else [f"generator cell {i}" for i in range(c.n)]
        r = _rates(mech, rin, mixed)
        rref, rsc = o.rates(rin, nthreads=NTHREADS, scale=True)
        _check(f"{'mixed' if mixed else 'plain'} saturated rates {config}", r, rref, rsc, lab,
               util.MIXED_TOL if mixed else util.PLAIN_TOL)
    if mixed:
        return
    ins = o.reaction_rates_inputs(gen)
    out = torch.empty((mech.R, gen.n), dtype=torch.float64, device="cuda")
    mech.reaction_rates(_dev(ins), out)
    torch.cuda.synchronize()
    rr = out.cpu().numpy()
    ref, sc = o.reaction_rates(ins, nthreads=NTHREADS, scale=True)
    _check(f"saturated reaction rates {config}", rr, ref, sc, [str(i) for i in range(gen.n)], util.PLAIN_TOL)
    # the irreversible reaction (no bulk reactant): cR = f32::MAX * prod C_k^nu_k in species order,
    # C_k = max(0, n_k) / V with V = 1
    ks = np.flatnonzero(m.reactants[r_irr])
    assert m.K - 1 not in ks
    C = np.maximum(gen.amounts, 0.0)
    p = None
    for k in ks:
        for _ in range(int(m.reactants[r_irr, k])):
            p = C[k].copy() if p is None else p * C[k]
    assert np.array_equal(rr[r_irr], F32_MAX * p)
    assert np.array_equal(ref[r_irr], F32_MAX * p)
