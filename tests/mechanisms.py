"""Test mechanisms that exercise every branch of the reference's rate builder (reaction.rs:113-309).

The benchmark mechanisms only contain elementary reversible, three-body and two-term Troe reactions.
``branch_mechanism`` starts from the seeded 10-species mechanism and rewrites a few reactions and species so
that one mechanism covers: irreversible reactions, Lindemann falloff, Troe with a T2 term, Troe with a
constant k_inf (b = Ea = 0), Troe without the T1 term (T1 >= 1e30), three-body reactions without
efficiencies and with an efficiency of exactly 2, stoichiometric coefficients of 2, every temperature
factor bucket of arrhenius() including the no-exponential case, and a single-piece (NaN split) species.
"""
import copy
import math

import numpy as np

from combustion_gb300 import synthetic as s


def branch_mechanism():
    m = copy.deepcopy(s.generate_mechanism("k10"))
    K = m.K
    E, IRR, TB, LIN, TROE = s.ELEMENTARY, s.IRREVERSIBLE, s.THREE_BODY, s.LINDEMANN, s.TROE
    rows = {r: int(m.model[r]) for r in range(m.R)}
    elem = [r for r, k in rows.items() if k == E]
    troe = [r for r, k in rows.items() if k == TROE]
    tb = [r for r, k in rows.items() if k == TB]
    # irreversible
    m.model[elem[0]] = IRR
    # Lindemann with dense efficiencies
    r = elem[1]
    m.model[r] = LIN
    m.k0[r] = (m.rate[r, 0] * 1e3 * 1e-6, m.rate[r, 1] - 0.3, m.rate[r, 2] * 0.7)
    m.efficiencies[r] = np.linspace(0.5, 4.0, K)
    # Troe variants
    m.troe[troe[0], 3] = 3000.0                       # T2 term present
    m.rate[troe[1], 1] = 0.0                          # k_inf constant: b = Ea = 0
    m.rate[troe[1], 2] = 0.0
    m.troe[troe[1], 2] = 1e31                         # no T1 exponential: constant A term
    # three-body without efficiencies, and with an efficiency of exactly 2
    m.efficiencies[tb[0]] = 1.0
    m.efficiencies[tb[1], 2] = 2.0
    # stoichiometric coefficient 2 on the reactant side of a reversible reaction: 2 S_a -> S_b
    r = elem[2]
    a, b = 0, 5
    m.reactants[r] = 0
    m.products[r] = 0
    m.reactants[r, a] = 2
    m.products[r, b] = 1
    # and 2 on the product side: S_c -> 2 S_d
    r = elem[3]
    m.reactants[r] = 0
    m.products[r] = 0
    m.reactants[r, 3] = 1
    m.products[r, 4] = 2
    # temperature factor buckets of arrhenius() (reaction.rs:117-125)
    for r, (bb, ea) in zip(elem[4:], [(-2.0, 0.0), (-1.0, 5000.0), (4.0, 0.0), (3.0, 8000.0), (2.0, 0.0),
                                       (1.0, 0.0), (0.0, 0.0), (0.25, 0.0), (0.5, 12000.0)]):
        m.rate[r, 1] = bb
        m.rate[r, 2] = ea
    # a single-piece species (NaN split; both pieces equal)
    m.nasa7_split[3] = math.nan
    m.nasa7[3, 1] = m.nasa7[3, 0]
    m.meta = {"config": "branches"}
    assert m.active() == K - 1
    return m


def cells_for(m, n, seed=7):
    return s.generate_cells(m.K, n, "k10", seed=seed)


def sri_mechanism():
    """The seeded 10-species mechanism with SRI falloff reactions (the reference leaves SRI unimplemented;
    the library follows its commented formula, reaction.rs:194-203): its two Troe reactions become SRI
    (one with A = 0, D != 1, E != 0) and one elementary reaction becomes SRI with the typical defaults."""
    m = copy.deepcopy(s.generate_mechanism("k10"))
    K = m.K
    rows = {r: int(m.model[r]) for r in range(m.R)}
    elem = [r for r, k in rows.items() if k == s.ELEMENTARY]
    troe = [r for r, k in rows.items() if k == s.TROE]
    for r, p in zip(troe + [elem[0]], [(0.45, 797.0, 979.0, 1.0, 0.0), (0.0, 0.0, 1500.0, 1.3, 0.2),
                                       (1.2, 350.0, 2200.0, 0.8, -0.3)]):
        m.model[r] = s.SRI
        m.sri[r] = p
        if not m.k0[r].any():
            m.k0[r] = (m.rate[r, 0] * 1e3 * 1e-6, m.rate[r, 1] - 0.5, m.rate[r, 2] * 0.8)
            m.efficiencies[r] = np.linspace(0.7, 3.0, K)
    m.meta = {"config": "sri"}
    assert m.active() == K - 1
    return m
