"""Writes the golden fixtures of the oracle (run from the repository root: python tests/golden/make_golden.py).

The reference has no tests, fixtures or published vectors for this path and cannot be built here, so the
fixtures pin this project's FP64 oracle: the seeded mechanisms, small batches of seeded cells, the
oracle's outputs and condition scales, and the library's fitted transport coefficients. Each set is
cross-checked against the independent numpy restatement before it is written.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy_restatement as nr  # noqa: E402
import oracle  # noqa: E402

import combustion_gb300 as cb  # noqa: E402
from combustion_gb300 import synthetic  # noqa: E402
from mechanisms import branch_mechanism, cells_for  # noqa: E402

SETS = [("k10", 256), ("k53", 64), ("branches", 128)]


def make(name, n):
    m = branch_mechanism() if name == "branches" else synthetic.generate_mechanism(name)
    cells = cells_for(m, n) if name == "branches" else synthetic.generate_cells(m.K, n, name)
    T0, mu0, l0 = synthetic.transport_scales(m)
    cond, visc, diff = cb.transport_fit(m, T0)
    o = oracle.Oracle(m)
    o.set_transport(T0, mu0, l0, cond, visc, diff)
    rin = o.rates_inputs(cells)
    tin = o.transport_inputs(cells)
    qin = o.reaction_rates_inputs(cells)
    rout, rsc = o.rates(rin, scale=True)
    tout, tsc = o.transport(tin, scale=True)
    qout, qsc = o.reaction_rates(qin, scale=True)
    rnp = nr.rates(m, rin[0], rin[1], rin[2], rin[3], np.array(rin[4:]))
    tnp = nr.transport(m, (T0, mu0, l0), (cond, visc, diff), tin[0], tin[1], np.array(tin[2:]))
    assert (np.abs(rout - rnp) / rsc).max() < 1e-14, name
    assert (np.abs(tout - tnp) / tsc).max() < 1e-14, name
    path = os.path.join(HERE, f"golden_{name}.npz")
    m.save(os.path.join(HERE, f"mech_{name}.npz"))
    np.savez_compressed(path, rates_in=np.array(rin), rates_out=rout, rates_scale=rsc, transport_in=np.array(tin),
                        transport_out=tout, transport_scale=tsc, reaction_in=np.array(qin), reaction_out=qout,
                        reaction_scale=qsc, cond=cond, visc=visc, diff=diff, scales=np.array([T0, mu0, l0]))
    print("wrote", path)


if __name__ == "__main__":
    for name, n in SETS:
        make(name, n)
