"""ctypes binding of the FP64 CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU
baseline leg, as the checker and the timed CPU baseline. The product library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
# No FMA contraction and no fast-math: every operation rounds once, like the reference interpreter.
CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fno-fast-math",
          "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    hdrs = [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "combustion_gb300", "csrc", "collision_integrals.h")]
    newest = max(os.path.getmtime(p) for p in [src] + hdrs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run(["gcc", *CFLAGS, src, "-o", tmp, "-lm", "-lpthread"], check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None
_dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.or_mech_new.restype = vp
        L.or_mech_new.argtypes = [C.c_int, C.c_int] + [vp] * 17
        L.or_mech_free.argtypes = [vp]
        L.or_active.argtypes = [vp]
        L.or_check.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.or_transport_samples.argtypes = [vp, C.c_double, vp, vp, vp, vp]
        L.or_transport_fit.argtypes = [vp, C.c_double, vp, vp, vp]
        for f in ("or_viscosity", "or_conductivity"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [vp, C.c_int, C.c_double]
        for f in ("or_diffusivity", "or_omega22"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [vp, C.c_int, C.c_int, C.c_double]
        L.or_set_transport.argtypes = [vp, C.c_double, C.c_double, C.c_double, vp, vp, vp]
        L.or_rates.argtypes = [vp, vp, vp, vp]
        L.or_reaction_rates.argtypes = [vp, vp, vp]
        L.or_transport.argtypes = [vp, vp, vp, vp]
        L.or_rates_batch.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_int]
        L.or_reaction_rates_batch.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_int]
        L.or_transport_batch.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_int]
        L.or_fused_batch.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _ptrs(rows):
    arr = (C.c_void_p * len(rows))(*[r.ctypes.data for r in rows])
    return arr


class Oracle:
    """A mechanism loaded into the oracle. ``mech`` is a combustion_gb300.synthetic.Mechanism."""

    def __init__(self, mech, transport=None):
        self.mech = mech
        self._keep = []
        K, R = mech.K, mech.R

        def f64(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            self._keep.append(a)
            return _p(a)

        def i32(a):
            a = np.ascontiguousarray(a, dtype=np.int32)
            self._keep.append(a)
            return _p(a)

        def u8(a):
            a = np.ascontiguousarray(a, dtype=np.uint8)
            self._keep.append(a)
            return _p(a)

        self.h = lib().or_mech_new(K, R, f64(mech.molar_mass), f64(mech.nasa7_split), f64(mech.nasa7),
                                   i32(mech.geometry), f64(mech.diameter), f64(mech.well_depth),
                                   f64(mech.polarizability), f64(mech.dipole), f64(mech.rotational_relaxation),
                                   u8(mech.reactants), u8(mech.products), i32(mech.model), f64(mech.rate),
                                   f64(mech.k0), f64(mech.troe), f64(mech.sri), f64(mech.efficiencies))
        buf = C.create_string_buffer(256)
        if lib().or_check(self.h, buf, 256):
            raise ValueError("oracle rejected the mechanism: " + buf.value.decode())
        self.K, self.R = K, R
        self.A = lib().or_active(self.h)
        self.T0 = None
        if transport is not None:
            self.set_transport(*transport)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_mech_free(self.h)
            self.h = None

    # -- transport set-up ------------------------------------------------------------------
    def samples(self, T0):
        K = self.K
        x = np.zeros(50)
        yc, yv, yd = np.zeros((K, 50)), np.zeros((K, 50)), np.zeros((K * K, 50))
        lib().or_transport_samples(self.h, T0, _p(x), _p(yc), _p(yv), _p(yd))
        return x, yc, yv, yd

    def fit(self, T0):
        K = self.K
        c, v, d = np.zeros((K, 5)), np.zeros((K, 5)), np.zeros((K * K, 5))
        lib().or_transport_fit(self.h, T0, _p(c), _p(v), _p(d))
        return c, v, d

    def set_transport(self, T0, mu0, lambda0, cond, visc, diff):
        cond, visc, diff = (np.ascontiguousarray(a, dtype=np.float64) for a in (cond, visc, diff))
        lib().or_set_transport(self.h, T0, mu0, lambda0, _p(cond), _p(visc), _p(diff))
        self.T0 = T0

    def viscosity(self, k, T):
        return lib().or_viscosity(self.h, k, T)

    def conductivity(self, k, T):
        return lib().or_conductivity(self.h, k, T)

    def diffusivity(self, a, b, T):
        return lib().or_diffusivity(self.h, a, b, T)

    def omega22(self, a, b, T):
        return lib().or_omega22(self.h, a, b, T)

    # -- batches (struct of arrays) ---------------------------------------------------------
    @staticmethod
    def rates_inputs(cells):
        n = cells.n
        rows = [cells.pressure_R, 1.0 / cells.pressure_R, cells.temperature, cells.volume] + list(cells.amounts)
        return [np.ascontiguousarray(r, dtype=np.float64) for r in rows]

    def transport_inputs(self, cells):
        rows = [cells.total_amount, cells.temperature / self.T0] + list(cells.amounts)
        return [np.ascontiguousarray(r, dtype=np.float64) for r in rows]

    def rates(self, inputs, nthreads=1, scale=False):
        n = len(inputs[0])
        out = np.zeros((self.A + 2, n))
        sc = np.zeros((self.A + 2, n)) if scale else None
        rc = lib().or_rates_batch(self.h, n, _ptrs(inputs), _ptrs(list(out)), _ptrs(list(sc)) if scale else None,
                                  nthreads)
        assert rc == 0, rc
        return (out, sc) if scale else out

    @staticmethod
    def reaction_rates_inputs(cells):
        rows = [cells.pressure_R, cells.temperature, cells.volume] + list(cells.amounts)
        return [np.ascontiguousarray(r, dtype=np.float64) for r in rows]

    def fused_inputs(self, cells):
        return self.rates_inputs(cells)

    def reaction_rates(self, inputs, nthreads=1, scale=False):
        n = len(inputs[0])
        out = np.zeros((self.R, n))
        sc = np.zeros((self.R, n)) if scale else None
        assert lib().or_reaction_rates_batch(self.h, n, _ptrs(inputs), _ptrs(list(out)),
                                             _ptrs(list(sc)) if scale else None, nthreads) == 0
        return (out, sc) if scale else out

    def transport(self, inputs, nthreads=1, scale=False):
        n = len(inputs[0])
        out = np.zeros((self.K + 2, n))
        sc = np.zeros((self.K + 2, n)) if scale else None
        rc = lib().or_transport_batch(self.h, n, _ptrs(inputs), _ptrs(list(out)), _ptrs(list(sc)) if scale else None,
                                      nthreads)
        assert rc == 0, rc
        return (out, sc) if scale else out

    def fused(self, inputs, nthreads=1):
        n = len(inputs[0])
        o1, o2 = np.zeros((self.A + 2, n)), np.zeros((self.K + 2, n))
        assert lib().or_fused_batch(self.h, n, _ptrs(inputs), _ptrs(list(o1)), _ptrs(list(o2)), nthreads) == 0
        return o1, o2
