"""Shared helpers of the tests: workloads, the oracle, and the parity metric."""
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
