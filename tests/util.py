"""Shared helpers of the tests: workloads, the oracle, and the parity metrics."""
import functools

import numpy as np

import oracle
from combustion_gb300 import synthetic

# Parity bar of the plain FP64 path against the FP64 oracle: relative error per output of 1e-12,
# measured against the output's condition scale (the sum of magnitudes of the terms it accumulates,
# computed by the oracle). Outputs that cancel to near zero cannot be reproduced more closely by any
# evaluation order that differs from the oracle's in the last bit of one term.
PLAIN_TOL = 1e-12
# Bar of the mixed-precision form, same metric.
MIXED_TOL = 1e-4
# Pure relative error |x - r| / |r| is asserted at PLAIN_TOL on every output whose condition scale is
# at most this multiple of its magnitude (an output that cancels less than 30-fold): with the plain
# path's condition-scaled error of a few 1e-14, such outputs are within 1e-12 relative.
WELL_CONDITIONED = 30.0


@functools.lru_cache(maxsize=None)
def mechanism(config):
    return synthetic.generate_mechanism(config)


@functools.lru_cache(maxsize=None)
def loaded_oracle(config):
    m = mechanism(config)
    o = oracle.Oracle(m)
    T0, mu0, l0 = synthetic.transport_scales(m)
    import combustion_gb300 as cb
    coefs = cb.transport_fit(m, T0)  # per-cell parity on the library's own fitted tables
    o.set_transport(T0, mu0, l0, *coefs)
    return o


def cond_err(x, ref, scale):
    """Per-element |x - ref| / scale (scale floored at the tiniest normal to avoid 0/0)."""
    return np.abs(x - ref) / np.maximum(scale, 1e-300)


def rel_err(x, ref):
    return np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)


def floored_err(x, ref):
    """The reference's own comparison metric for species rates, |x - r| / max(r, 1e3) (cantera.rs:147),
    rates in mol/m^3/s; r enters signed, as written there, so that a negative rate is compared in
    absolute terms (its error divided by 1e3)."""
    return np.abs(x - ref) / np.maximum(ref, 1e3)


def floored_abs_err(x, ref):
    """The same floor on |r|: |x - r| / max(|r|, 1e3)."""
    return np.abs(x - ref) / np.maximum(np.abs(ref), 1e3)


def _mr(e):
    e = np.asarray(e, dtype=np.float64).ravel()
    if e.size == 0:
        return {"max": 0.0, "rms": 0.0}
    return {"max": float(e.max()), "rms": float(np.sqrt(np.mean(e * e)))}


RATES_GROUPS = (("dTdt", slice(0, 1)), ("dVdt", slice(1, 2)), ("species", slice(2, None)))
TRANSPORT_GROUPS = (("conductivity", slice(0, 1)), ("viscosity", slice(1, 2)), ("diffusion", slice(2, None)))


def error_groups(x, ref, scale, groups, floored_species=False):
    """Per output group: condition-scaled and pure relative error (max, RMS), the fraction of outputs
    above PLAIN_TOL pure relative, and for species rates the reference's floored metric."""
    out = {}
    for name, rows in groups:
        g = {"cond": _mr(cond_err(x[rows], ref[rows], scale[rows])), "rel": _mr(rel_err(x[rows], ref[rows])),
             "frac_rel_above_1e-12": float((rel_err(x[rows], ref[rows]) > PLAIN_TOL).mean())}
        if floored_species and name == "species":
            g["floored"] = _mr(floored_err(x[rows], ref[rows]))
            g["floored_abs"] = _mr(floored_abs_err(x[rows], ref[rows]))
        out[name] = g
    return out


def well_conditioned(ref, scale):
    """Mask of the outputs whose condition scale is at most WELL_CONDITIONED times their magnitude."""
    return scale <= WELL_CONDITIONED * np.abs(ref)


def print_groups(name, groups):
    for g, v in groups.items():
        extra = (f", floored max {v['floored']['max']:.2e} (on |r|: {v['floored_abs']['max']:.2e})"
                 if "floored" in v else "")
        print(f"{name} {g}: cond max {v['cond']['max']:.2e} rms {v['cond']['rms']:.2e}; rel max {v['rel']['max']:.2e} "
              f"rms {v['rel']['rms']:.2e}; {100 * v['frac_rel_above_1e-12']:.3f}% above 1e-12 rel{extra}")
