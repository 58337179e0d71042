"""Writes a synthetic mechanism as a Cantera YAML file (the tests' source of reader inputs)."""
import numpy as np

from combustion_gb300 import synthetic

WEIGHTS = {"H": 1.008, "C": 12.011, "N": 14.007, "O": 15.999}  # g/mol, the reader's table
GEOMETRY = {0: "atom", 1: "linear", 2: "nonlinear"}


def compositions(K, seed=7):
    rng = np.random.default_rng(seed)
    return [{"C": int(rng.integers(0, 3)), "H": int(rng.integers(1, 6)), "O": int(rng.integers(0, 3))} for _ in range(K)]


def molar_mass(comp):
    return sum(n * WEIGHTS[e] for e, n in comp.items()) / 1e3


def order(mech, r):
    n = int(mech.reactants[r].sum())
    return n + (1 if mech.model[r] == synthetic.THREE_BODY else 0)


def write(mech, comps, ea_unit="cal/mol"):
    names = mech.names
    out = ["description: |-", "  Synthetic mechanism written by the tests.", "  Second line of the description.", "",
           f"units: {{length: cm, time: s, quantity: mol, activation-energy: {ea_unit}}}", "",
           "phases:", "- name: gas", "  thermo: ideal-gas", "  elements: [H, C, O]",
           "  species: [" + ", ".join(names) + "]", "", "species:"]
    for k in range(mech.K):
        comp = ", ".join(f"{e}: {n}" for e, n in comps[k].items() if n)
        split = mech.nasa7_split[k]
        out += [f"- name: {names[k]}", f"  composition: {{{comp}}}", "  thermo:", "    model: NASA7",
                f"    temperature-ranges: [200.0, {float(split)!r}, 3500.0]", "    data:"]
        for q in range(2):
            out.append("    - [" + ", ".join(repr(float(c)) for c in mech.nasa7[k, q]) + "]")
        g = GEOMETRY[int(mech.geometry[k])]
        out += ["  transport:", "    model: gas", f"    geometry: {g}",
                f"    well-depth: {float(mech.well_depth[k] / synthetic.kB)!r}",
                f"    diameter: {float(mech.diameter[k] * 1e10)!r}"]
        if g != "atom":
            out += [f"    polarizability: {float(mech.polarizability[k] * 1e30)!r}",
                    f"    rotational-relaxation: {float(mech.rotational_relaxation[k])!r}"]
    out += ["", "reactions:"]
    for r in range(mech.R):
        def side(v):
            return " + ".join((f"{n} {names[k]}" if n > 1 else names[k]) for k, n in enumerate(v) if n)
        m = int(mech.model[r])
        lhs, rhs = side(mech.reactants[r]), side(mech.products[r])
        arrow = " => " if m == synthetic.IRREVERSIBLE else " <=> "
        if m == synthetic.THREE_BODY:
            eq = f"{lhs} + M{arrow}{rhs} + M"
        elif m in (synthetic.TROE, synthetic.LINDEMANN, synthetic.SRI):
            eq = f"{lhs} (+M){arrow}{rhs} (+M)"
        else:
            eq = lhs + arrow + rhs

        def rate(row, exponent):
            A = float(row[0]) / 1e-6 ** exponent
            Ea = float(row[2]) if ea_unit == "K" else float(row[2]) * synthetic.R / 4.184
            return f"{{A: {A!r}, b: {float(row[1])!r}, Ea: {Ea!r}}}"
        n = int(mech.reactants[r].sum())
        out.append(f"- equation: {eq}  # reaction {r + 1}")
        if m == synthetic.THREE_BODY:
            out += ["  type: three-body", f"  rate-constant: {rate(mech.rate[r], order(mech, r) - 1)}"]
        elif m in (synthetic.TROE, synthetic.LINDEMANN):
            out += ["  type: falloff", f"  low-P-rate-constant: {rate(mech.k0[r], n)}",
                    f"  high-P-rate-constant: {rate(mech.rate[r], n - 1)}"]
            if m == synthetic.TROE:
                a, T3, T1, T2 = mech.troe[r]
                t2 = "" if not np.isfinite(T2) else f", T2: {float(T2)!r}"
                out.append(f"  Troe: {{A: {float(a)!r}, T3: {float(T3)!r}, T1: {float(T1)!r}{t2}}}")
        else:
            out.append(f"  rate-constant: {rate(mech.rate[r], n - 1)}")
        if m in (synthetic.THREE_BODY, synthetic.TROE, synthetic.LINDEMANN):
            eff = ", ".join(f"{names[k]}: {float(e)!r}" for k, e in enumerate(mech.efficiencies[r]) if e != 1.0)
            out.append(f"  efficiencies: {{{eff}}}")
    return "\n".join(out) + "\n"
