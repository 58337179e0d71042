"""The Cantera-YAML reader (cb_yaml_load, the role of yaml.rs:54-171 + lib.rs:20-140), on the CPU: a
hand-written file exercising every construct the reference reads, and round trips of the synthetic
mechanisms written as Cantera YAML (same arrays, same rates through the FP64 oracle)."""
import math

import numpy as np
import pytest

import oracle
import util
from cantera_yaml_writer import compositions, molar_mass, write
from combustion_gb300 import synthetic

R = synthetic.R
CAL = 4.184 / R

HANDWRITTEN = """\
description: |-
  A small hand-written mechanism: every construct the reader accepts.
  # not a comment inside a block scalar
generator: tests
units: {length: cm, time: s, quantity: mol, activation-energy: cal/mol}

phases:
- name: gas
  species: [AR, H2, O2, H, O, OH, H2O, HO2, N2]

species:
- name: AR   # inert, listed first: goes after the active species
  composition: {Ar: 1}
  thermo:
    model: NASA7
    temperature-ranges: [300.0, 1000.0, 5000.0]
    data:
    - [2.5, 0.0, 0.0, 0.0, 0.0, -745.375, 4.366]
    - [2.5, 0.0, 0.0, 0.0, 0.0, -745.375, 4.366]
  transport: {model: gas, geometry: atom, well-depth: 136.5, diameter: 3.33}
- name: H2
  composition: {H: 2}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [2.3, 0.008, -1.9e-05, 2.0e-08, -7.4e-12,
       -917.9, 0.68]
    - [3.3, -4.9e-05, 4.99e-07, -1.8e-10, 2.0e-14, -950.1, -3.2]
  transport:
    model: gas
    geometry: linear
    well-depth: 38.0
    diameter: 2.92
    polarizability: 0.79
    rotational-relaxation: 280.0
    dipole: 1.5  # ignored for linear molecules (lib.rs:41-42)
- name: O2
  composition: {O: 2}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [3.8, -0.003, 9.8e-06, -9.7e-09, 3.2e-12, -1063.9, 3.66]
    - [3.3, 0.0013, -5.3e-07, 9.6e-11, -6.4e-15, -1088.5, 5.45]
  transport: {model: gas, geometry: linear, well-depth: 107.4, diameter: 3.46, polarizability: 1.6, rotational-relaxation: 3.8}
- name: H
  composition: {H: 1}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 3500.0]
    data:
    - [2.5, 0.0, 0.0, 0.0, 0.0, 25473.6, -0.447]
  transport: {model: gas, geometry: atom, well-depth: 145.0, diameter: 2.05}
- name: O
  composition: {O: 1}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [3.2, -0.0033, 6.5e-06, -5.7e-09, 1.9e-12, 29122.3, 2.05]
    - [2.6, -8.6e-05, 4.2e-08, -1.0e-11, 1.2e-15, 29217.6, 4.78]
  transport: {model: gas, geometry: atom, well-depth: 80.0, diameter: 2.75}
- name: OH
  composition: {O: 1, H: 1}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [4.1, -0.0032, 6.5e-06, -5.9e-09, 2.1e-12, 3381.5, -0.69]
    - [2.9, 0.001, -2.6e-07, 3.7e-11, -2.3e-15, 3718.9, 5.7]
  transport: {model: gas, geometry: linear, well-depth: 80.0, diameter: 2.75}
- name: H2O
  composition: {H: 2, O: 1}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [4.2, -0.0020, 6.5e-06, -5.5e-09, 1.8e-12, -30293.7, -0.85]
    - [3.0, 0.0021, -1.6e-07, -9.7e-11, 1.7e-14, -30004.3, 4.97]
  transport: {model: gas, geometry: nonlinear, well-depth: 572.4, diameter: 2.605, dipole: 1.844, rotational-relaxation: 4.0}
- name: HO2
  composition: {H: 1, O: 2}
  thermo:
    model: NASA7
    temperature-ranges: [200.0, 1000.0, 3500.0]
    data:
    - [4.3, -0.0047, 2.1e-05, -2.4e-08, 9.3e-12, 294.8, 3.72]
    - [4.0, 0.0022, -6.3e-07, 1.1e-10, -9.2e-15, 111.9, 3.79]
  transport: {model: gas, geometry: nonlinear, well-depth: 107.4, diameter: 3.458, rotational-relaxation: 1.0}
- name: N2
  composition: {N: 2}
  thermo:
    model: NASA7
    temperature-ranges: [300.0, 1000.0, 5000.0]
    data:
    - [3.3, 0.0014, -4.0e-06, 5.6e-09, -2.4e-12, -1020.9, 3.95]
    - [2.9, 0.0015, -5.7e-07, 1.0e-10, -6.8e-15, -922.8, 5.98]
  transport: {model: gas, geometry: linear, well-depth: 97.53, diameter: 3.621, polarizability: 1.76, rotational-relaxation: 4.0}

reactions:
- equation: H + O2 <=> O + OH  # elementary
  rate-constant: {A: 3.5e+15, b: -0.4, Ea: 16600.0}
- equation: H2 + O => H + OH
  rate-constant: {A: 50000.0, b: 2.7, Ea: 6290.0}
- equation: 2 O + M <=> O2 + M
  type: three-body
  rate-constant: {A: 6.2e+15, b: -0.5, Ea: 0.0}
  efficiencies: {AR: 0.8, H2: 2.5}
- equation: H + O2 (+M) <=> HO2 (+M)
  type: falloff
  low-P-rate-constant: {A: 6.4e+20, b: -1.7, Ea: 520.0}
  high-P-rate-constant: {A: 4.7e+12, b: 0.44, Ea: 0.0}
  Troe: {A: 0.5, T3: 1.0e-30, T1: 1.0e+30}
  efficiencies: {H2: 2.0, H2O: 14.0}
- equation: 2 OH (+M) <=> H2O + O (+M)
  type: falloff
  low-P-rate-constant: {A: 2.3e+18, b: -0.9, Ea: -1700.0}
  high-P-rate-constant: {A: 7.4e+13, b: -0.37, Ea: 0.0}
- equation: HO2 + H <=> 2 OH
  type: pressure-dependent-Arrhenius
  rate-constants:
  - {P: 1.0 atm, A: 7.1e+13, b: 0.0, Ea: 300.0}
- equation: H2O + H <=> H2 + OH
  duplicate: true
  rate-constant: {A: 2.3e+09, b: 1.5, Ea: 18500.0}
"""

SRI_REACTION = """\
- equation: H + OH (+M) <=> H2O (+M)
  type: falloff
  low-P-rate-constant: {A: 4.0e+22, b: -2.0, Ea: 0.0}
  high-P-rate-constant: {A: 2.5e+13, b: 0.23, Ea: -114.0}
  SRI: {A: 0.45, B: 797.0, C: 979.0}
"""


def _load(text):
    from combustion_gb300 import build, cantera_yaml
    build.build()
    return cantera_yaml.load(text)


def test_handwritten_file():
    m = _load(HANDWRITTEN)
    assert m.names == ["H2", "O2", "H", "O", "OH", "H2O", "HO2", "AR", "N2"]
    K = m.K
    idx = {n: k for k, n in enumerate(m.names)}
    W = {"H2": 2 * 1.008, "O2": 2 * 15.999, "H": 1.008, "O": 15.999, "OH": 17.007, "H2O": 2 * 1.008 + 15.999,
         "HO2": 1.008 + 2 * 15.999, "AR": 39.95, "N2": 2 * 14.007}
    for n, w in W.items():
        assert m.molar_mass[idx[n]] == pytest.approx(w / 1e3, rel=1e-15)
    # one piece for H (two ranges) and for AR (duplicate pieces merged), split 1000 K otherwise
    assert math.isnan(m.nasa7_split[idx["H"]]) and math.isnan(m.nasa7_split[idx["AR"]])
    assert m.nasa7_split[idx["O2"]] == 1000.0
    assert (m.nasa7[idx["H"], 0] == m.nasa7[idx["H"], 1]).all()
    assert m.nasa7[idx["H2"], 0, 0] == 2.3 and m.nasa7[idx["H2"], 0, 5] == -917.9  # flow list over two lines
    assert list(m.geometry[[idx["AR"], idx["H2"], idx["H2O"]]]) == [0, 1, 2]
    assert m.dipole[idx["H2"]] == 0.0  # linear: dipole ignored
    assert m.dipole[idx["H2O"]] == pytest.approx(1.844 * 1e-21 / 299792458.0, rel=1e-15)
    assert m.well_depth[idx["H2O"]] == pytest.approx(572.4 * synthetic.kB, rel=1e-15)
    assert m.diameter[idx["N2"]] == pytest.approx(3.621e-10, rel=1e-15)
    assert m.polarizability[idx["AR"]] == 0.0 and m.rotational_relaxation[idx["AR"]] == 0.0
    assert m.polarizability[idx["O2"]] == pytest.approx(1.6e-30, rel=1e-15)
    assert list(m.model) == [0, 1, 2, 4, 3, 0, 0]
    r = m.rate
    assert r[0] == pytest.approx([3.5e15 * 1e-6, -0.4, 16600.0 * 4.184 / R], rel=1e-15)
    assert r[2][0] == pytest.approx(6.2e15 * 1e-12, rel=1e-15)  # three-body: M counts in the order
    assert r[3][0] == pytest.approx(4.7e12 * 1e-6, rel=1e-15) and m.k0[3][0] == pytest.approx(6.4e20 * 1e-12, rel=1e-15)
    assert m.k0[4][2] == pytest.approx(-1700.0 * 4.184 / R, rel=1e-15)
    assert r[5][0] == pytest.approx(7.1e13 * 1e-6, rel=1e-15)
    assert list(m.troe[3][:3]) == [0.5, 1.0e-30, 1.0e30] and math.isinf(m.troe[3][3])
    assert m.efficiencies[2][idx["AR"]] == 0.8 and m.efficiencies[2][idx["H2"]] == 2.5
    assert m.efficiencies[2][idx["O"]] == 1.0
    assert m.efficiencies[3][idx["H2O"]] == 14.0
    # stoichiometry: "2 O + M" and "2 OH (+M)"
    assert m.reactants[2][idx["O"]] == 2 and m.products[2][idx["O2"]] == 1 and m.reactants[2].sum() == 2
    assert m.reactants[4][idx["OH"]] == 2 and m.products[4][idx["H2O"]] == 1 and m.products[4][idx["O"]] == 1
    assert m.products[5][idx["OH"]] == 2
    import combustion_gb300 as cb
    info = cb.validate(m)
    assert (info.n_species, info.n_active, info.n_reactions) == (9, 7, 7)
    assert m.active() == 7


def test_sri_is_read():
    import combustion_gb300 as cb
    m = _load(HANDWRITTEN + SRI_REACTION)
    assert m.model[-1] == synthetic.SRI
    assert list(m.sri[-1]) == [0.45, 797.0, 979.0, 1.0, 0.0]
    assert m.k0[-1][0] == pytest.approx(4.0e22 * 1e-12, rel=1e-15)
    assert cb.validate(m).n_reactions == 8


@pytest.mark.parametrize("bad,code", [
    ("units: {length: m, time: s, quantity: mol, activation-energy: K}\nspecies: []\nreactions: []\n", 2),
    (HANDWRITTEN.replace("2 O + M <=> O2 + M", "2 O + M <=> O3 + M"), 2),
    (HANDWRITTEN.replace("type: three-body", "type: chemically-activated"), 5),
])
def test_rejections(bad, code):
    import combustion_gb300 as cb
    with pytest.raises(cb.CombustionError) as e:
        _load(bad)
    assert e.value.code == code


@pytest.mark.parametrize("config,unit", [("k10", "cal/mol"), ("k53", "K")])
def test_round_trip_of_synthetic_mechanisms(config, unit):
    src = util.mechanism(config)
    comps = compositions(src.K)
    m = _load(write(src, comps, unit))
    assert m.names == src.names
    assert np.array_equal(m.nasa7, src.nasa7) and np.array_equal(m.nasa7_split, src.nasa7_split)
    assert np.allclose(m.molar_mass, [molar_mass(c) for c in comps], rtol=1e-15, atol=0)
    assert np.array_equal(m.reactants, src.reactants) and np.array_equal(m.products, src.products)
    assert np.array_equal(m.model, src.model) and np.array_equal(m.efficiencies, src.efficiencies)
    assert np.allclose(m.rate, src.rate, rtol=1e-14, atol=0)
    assert np.allclose(m.k0, src.k0, rtol=1e-14, atol=0)
    assert np.array_equal(m.troe[:, :3], src.troe[:, :3]) and np.all(np.isinf(m.troe[src.model == 4, 3]))
    for a in ("diameter", "well_depth", "polarizability", "rotational_relaxation"):
        assert np.allclose(getattr(m, a), getattr(src, a), rtol=1e-14, atol=0), a
    # the same rates through the oracle, up to the last bits of the converted constants
    expect = util.mechanism(config)
    import copy
    expect = copy.deepcopy(expect)
    expect.molar_mass = m.molar_mass.copy()
    cells = synthetic.generate_cells(src.K, 256, config)
    o1, o2 = oracle.Oracle(m), oracle.Oracle(expect)
    ins = o1.rates_inputs(cells)
    a, sa = o1.rates(ins, scale=True)
    b = o2.rates(ins)
    assert (np.abs(a - b) / np.maximum(sa, 1e-300)).max() < 1e-12
