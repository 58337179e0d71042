"""The FP64 oracle against its golden fixtures, an independent numpy restatement and physics known answers.

The reference has no golden vectors for this path (no tests, and its Rust sources cannot be built here), so
parity is unpinned: these tests pin the oracle to itself across machines (fixtures written by
tests/golden/make_golden.py), to a second independent transcription of the same formulas, and to
closed-form physics.
"""
import math
import os

import numpy as np
import pytest

import numpy_restatement as nr
import oracle
import util
from combustion_gb300 import synthetic
from mechanisms import branch_mechanism, cells_for, sri_mechanism

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# Fixtures were written on x86-64 glibc; another libm (e.g. aarch64) may differ by an ulp in exp/log.
FIXTURE_TOL = 1e-13


def _golden(name):
    m = synthetic.Mechanism.load(os.path.join(GOLDEN, f"mech_{name}.npz"))
    g = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    o = oracle.Oracle(m)
    T0, mu0, l0 = g["scales"]
    o.set_transport(T0, mu0, l0, g["cond"], g["visc"], g["diff"])
    return m, g, o


@pytest.mark.parametrize("name", ["k10", "k53", "branches"])
def test_oracle_matches_golden_fixtures(name):
    m, g, o = _golden(name)
    r = o.rates(list(g["rates_in"]))
    t = o.transport(list(g["transport_in"]))
    q = o.reaction_rates(list(g["reaction_in"]))
    assert util.cond_err(r, g["rates_out"], g["rates_scale"]).max() <= FIXTURE_TOL
    assert util.cond_err(t, g["transport_out"], g["transport_scale"]).max() <= FIXTURE_TOL
    assert util.cond_err(q, g["reaction_out"], g["reaction_scale"]).max() <= FIXTURE_TOL


@pytest.mark.parametrize("name", ["k10", "branches", "sri"])
def test_oracle_matches_numpy_restatement(name):
    m = {"branches": branch_mechanism, "sri": sri_mechanism}.get(name, lambda: util.mechanism(name))()
    cells = synthetic.generate_cells(m.K, 1024, name, offset=777) if name == "k10" else cells_for(m, 1024)
    o = oracle.Oracle(m)
    T0, mu0, l0 = synthetic.transport_scales(m)
    coefs = o.fit(T0)
    o.set_transport(T0, mu0, l0, *coefs)
    rin, tin = o.rates_inputs(cells), o.transport_inputs(cells)
    r, rs = o.rates(rin, scale=True)
    t, ts = o.transport(tin, scale=True)
    rn = nr.rates(m, rin[0], rin[1], rin[2], rin[3], np.array(rin[4:]))
    tn = nr.transport(m, (T0, mu0, l0), coefs, tin[0], tin[1], np.array(tin[2:]))
    assert util.cond_err(r, rn, rs).max() <= 1e-14
    assert util.cond_err(t, tn, ts).max() <= 1e-14
    # most outputs agree to the last bit: only libm vs numpy exp/log roundings differ
    assert (t == tn).mean() > 0.9


def test_oracle_threads_are_deterministic():
    o = util.loaded_oracle("k10")
    cells = synthetic.generate_cells(10, 3000, "k10")
    ins = o.rates_inputs(cells)
    assert np.array_equal(o.rates(ins, nthreads=1), o.rates(ins, nthreads=7))


def _one_species_mech():
    """A two-species mechanism (A <=> bulk is not allowed: the bulk is inert), A + A <=> B with a bulk."""
    m = synthetic.generate_mechanism("k10")
    return m


def test_equilibrium_gives_zero_net_rate():
    """At a state where Rf == Rr/K for the only reaction touching a pair, its cR vanishes: build cells
    at which the reverse and forward progress balance by solving for the product concentration."""
    m = util.mechanism("k10")
    o = oracle.Oracle(m)
    r = next(i for i in range(m.R) if m.model[i] == synthetic.ELEMENTARY and m.reactants[i].sum() == 1
             and m.products[i].sum() == 1)
    a, b = int(np.argmax(m.reactants[r])), int(np.argmax(m.products[r]))
    T, P_R = 1500.0, 101325.0 / synthetic.R
    # K_c = exp(-(g_b - g_a)) for a unimolecular reaction (no C0 factor).
    def g(k):
        c = m.nasa7[k, 0 if T <= m.nasa7_split[k] else 1]
        return (c[0] - c[6] - c[0] * math.log(T) - c[1] / 2 * T + (1 / 3 - 1 / 2) * c[2] * T * T
                + (1 / 4 - 1 / 3) * c[3] * T ** 3 + (1 / 5 - 1 / 4) * c[4] * T ** 4 + c[5] / T)
    ga, gb = g(a), g(b)
    if not (abs(ga) < 25 and abs(gb) < 25):
        pytest.skip("Gibbs factors saturate at this temperature")
    Kc = math.exp(ga - gb)
    total = P_R / T
    n = np.zeros(m.K - 1)
    n[a] = 0.01 * total
    n[b] = Kc * n[a]
    if n.sum() >= total:
        pytest.skip("equilibrium state exceeds the total amount")
    inp = [np.array([x]) for x in [P_R, 1 / P_R, T, 1.0, *n]]
    q, qs = o.reaction_rates([inp[0], inp[2], inp[3]] + inp[4:], scale=True)
    assert abs(q[r, 0]) <= 1e-10 * qs[r, 0]


@pytest.mark.parametrize("tstar,omega", [(1.0, 1.5929), (2.0, 1.1757), (5.0, 0.92676), (0.5, 2.2837)])
def test_collision_integral_on_table_nodes(tstar, omega):
    """With zero dipole and T* on a table node, the quadratic interpolation returns the tabulated
    Omega(2,2)* of column 0 (transport.rs:92-93)."""
    m = util.mechanism("k10")
    o = oracle.Oracle(m)
    T = tstar * m.well_depth[0] / synthetic.kB
    assert o.omega22(0, 0, T) == pytest.approx(omega, rel=1e-12)


def test_one_species_mixture_gives_the_species_properties():
    """A mixture of the bulk species alone: Wilke phi_kk = 1, so mu_mix = mu_k and the conductivity
    mixing rule gives lambda_k, each to the accuracy of the degree-4 fits (transport.rs:119-158)."""
    m = util.mechanism("k10")
    o = util.loaded_oracle("k10")
    T0, mu0, l0 = synthetic.transport_scales(m)
    b = m.K - 1
    for T in (400.0, 1000.0, 2500.0):
        N = 40.0
        inp = [np.array([N]), np.array([T / T0])] + [np.zeros(1) for _ in range(m.K - 1)]
        out = o.transport(inp)
        assert out[1, 0] * mu0 == pytest.approx(o.viscosity(b, T), rel=2e-3)
        assert out[0, 0] * l0 == pytest.approx(o.conductivity(b, T), rel=1e-2)


def test_species_physics_magnitudes():
    """Chapman-Enskog magnitudes for a nitrogen-like species (W = 28 g/mol, sigma = 3.621 A, eps/k = 97.53 K):
    viscosity about 1.8e-5 Pa s at 300 K and P*D_self about 2.0 Pa m^2/s."""
    m = util.mechanism("k10")
    m2 = synthetic.Mechanism(**{**m.__dict__})
    m2.molar_mass = m.molar_mass.copy(); m2.molar_mass[0] = 0.028
    m2.diameter = m.diameter.copy(); m2.diameter[0] = 3.621e-10
    m2.well_depth = m.well_depth.copy(); m2.well_depth[0] = 97.53 * synthetic.kB
    o = oracle.Oracle(m2)
    assert o.viscosity(0, 300.0) == pytest.approx(1.78e-5, rel=0.03)
    assert o.diffusivity(0, 0, 300.0) == pytest.approx(2.0, rel=0.1)
