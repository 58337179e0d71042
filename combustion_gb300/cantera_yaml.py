"""Cantera-YAML mechanisms through the C ABI (cb_yaml_* in include/combustion_gb300.h): the role of the
reference's yaml.rs:54-171 loader and of combustion::new (lib.rs:127-140)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _check, cb_mech_desc, lib
from .synthetic import Mechanism

_bound = False


def _bind():
    global _bound
    L = lib()
    if not _bound:
        vp = C.c_void_p
        L.cb_yaml_load.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(vp)]
        L.cb_yaml_desc.argtypes = [vp, C.POINTER(cb_mech_desc)]
        L.cb_yaml_species_name.argtypes = [vp, C.c_int32]
        L.cb_yaml_species_name.restype = C.c_char_p
        L.cb_yaml_free.argtypes = [vp]
        _bound = True
    return L


def _arr(ptr, shape, ctype, dtype):
    n = int(np.prod(shape))
    if not ptr or n == 0:
        return np.zeros(shape, dtype=dtype)
    buf = C.cast(ptr, C.POINTER(ctype * n)).contents
    return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape).copy()


def load(text: str) -> Mechanism:
    """A Mechanism (SI arrays, active species first) from the text of a Cantera YAML file."""
    L = _bind()
    raw = text.encode()
    h = C.c_void_p()
    _check(L.cb_yaml_load(raw, len(raw), C.byref(h)))
    try:
        d = cb_mech_desc()
        _check(L.cb_yaml_desc(h, C.byref(d)))
        K, R = d.n_species, d.n_reactions
        f8, i4, u1 = C.c_double, C.c_int32, C.c_uint8
        m = Mechanism(
            names=[L.cb_yaml_species_name(h, k).decode() for k in range(K)],
            molar_mass=_arr(d.molar_mass, (K,), f8, np.float64),
            nasa7_split=_arr(d.nasa7_split, (K,), f8, np.float64),
            nasa7=_arr(d.nasa7, (K, 2, 7), f8, np.float64),
            geometry=_arr(d.geometry, (K,), i4, np.int32),
            diameter=_arr(d.diameter, (K,), f8, np.float64),
            well_depth=_arr(d.well_depth, (K,), f8, np.float64),
            polarizability=_arr(d.polarizability, (K,), f8, np.float64),
            dipole=_arr(d.dipole, (K,), f8, np.float64),
            rotational_relaxation=_arr(d.rotational_relaxation, (K,), f8, np.float64),
            reactants=_arr(d.reactants, (R, K), u1, np.uint8),
            products=_arr(d.products, (R, K), u1, np.uint8),
            model=_arr(d.model, (R,), i4, np.int32),
            rate=_arr(d.rate, (R, 3), f8, np.float64),
            k0=_arr(d.k0, (R, 3), f8, np.float64),
            troe=_arr(d.troe, (R, 4), f8, np.float64),
            sri=_arr(d.sri, (R, 5), f8, np.float64),
            efficiencies=_arr(d.efficiencies, (R, K), f8, np.float64),
            meta={"source": "cantera-yaml"})
    finally:
        L.cb_yaml_free(h)
    return m
