"""Batched constant-pressure reactors over the C ABI (cb_reactors_* in include/combustion_gb300.h).

Role of the reference's reactor loop (plot.rs:32-118) and cvode crate (cvode/lib.rs:17-47): the state
u = [T, V, n_0 .. n_{A-1}] evolves at fixed pressure with du/dt = the rates function's outputs
(reaction.rs:356-391); here thousands of reactors advance together on the GPU (variable-order BDF).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import Mechanism, _check, lib
from .synthetic import R, uniform


class cb_bdf_options(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("t_end", C.c_double), ("max_steps", C.c_int32),
                ("slice_steps", C.c_int32), ("warps_per_block", C.c_int32), ("tables_in_shared", C.c_int32),
                ("flags", C.c_int32)]


MIXED_RHS = 1  # CB_BDF_MIXED_RHS: first Newton iteration per step on the mixed-precision f; the rest FP64
REUSE_LU = 2   # CB_BDF_REUSE_LU: keep the factorisation while h / gamma_q changes by at most 30 %
GLOBAL_MEMORY = 4  # CB_BDF_GLOBAL_MEMORY: workspaces in global memory even when they fit in shared memory
LU32 = 8  # CB_BDF_LU32: FP32 factorisation (global-memory workspaces); residuals and corrections FP64


class cb_reactor_stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("steps", "rhs_evals", "jacobians", "factorizations", "newton_failures",
                                           "error_failures", "finished", "failed")] + [
        ("ms", C.c_double), ("warps_per_block", C.c_int32), ("tables_in_shared", C.c_int32),
        ("graph_replays", C.c_int32), ("slices", C.c_int32), ("global_memory", C.c_int32), ("register_cap", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class _cand(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("tables_in_shared", C.c_int32), ("global_memory", C.c_int32),
                ("register_cap", C.c_int32), ("ms", C.c_double)]


class cb_reactor_tuning(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("tables_in_shared", C.c_int32), ("n_candidates", C.c_int32),
                ("calib_reactors", C.c_int32), ("global_memory", C.c_int32), ("register_cap", C.c_int32),
                ("candidates", _cand * 32)]

    def as_dict(self):
        return {"warps_per_block": self.warps_per_block, "tables_in_shared": self.tables_in_shared,
                "global_memory": self.global_memory, "register_cap": self.register_cap,
                "calib_reactors": self.calib_reactors,
                "candidates": [{"warps_per_block": c.warps_per_block, "tables_in_shared": c.tables_in_shared,
                                "global_memory": c.global_memory, "register_cap": c.register_cap, "ms": c.ms}
                               for c in self.candidates[:self.n_candidates]]}


STATUS = {0: "new", 1: "unfinished", 2: "done", 3: "step size underflow", 4: "step limit", 5: "singular"}
_bound = False


def _bind():
    global _bound
    L = lib()
    if not _bound:
        vp, sz = C.c_void_p, C.c_size_t
        L.cb_reactors_create.argtypes = [vp, sz, C.POINTER(cb_bdf_options), C.POINTER(vp)]
        L.cb_reactors_destroy.argtypes = [vp]
        L.cb_reactors_set_state.argtypes = [vp, vp, vp, vp, vp]
        L.cb_reactors_autotune.argtypes = [vp, C.c_int32, C.POINTER(cb_reactor_tuning)]
        L.cb_reactors_integrate.argtypes = [vp, C.POINTER(cb_reactor_stats)]
        L.cb_reactors_results.argtypes = [vp, vp, vp, vp, vp]
        L.cb_reactors_eval.argtypes = [vp, C.c_int32, vp, vp, vp, vp]
        L.cb_reactors_set_outputs.argtypes = [vp, C.c_int32, C.c_int32]
        L.cb_reactors_outputs.argtypes = [vp, vp, vp, vp, vp, vp]
        _bound = True
    return L


def initial_states(K: int, n: int, seed: int = 4, T=(1000.0, 1600.0), P_atm=(1.0, 40.0), phi=(0.5, 2.0),
                   diluent=0.79):
    """Seeded reactor inlets: fuel species 0 and oxidiser species 1 at equivalence ratio phi (fuel :
    oxidiser = phi : 2, a methane-like stoichiometry) in `diluent` mole fraction of the bulk species,
    T and P (log-uniform) drawn per reactor, V = 1 m^3. Returns (pressure_R [n], T [n], V [n],
    amounts [K-1, n])."""
    idx = np.arange(n, dtype=np.uint64)
    Tn = T[0] + (T[1] - T[0]) * uniform(seed, 1, idx)
    lo, hi = math.log(P_atm[0]), math.log(P_atm[1])
    P = 101325.0 * np.exp(lo + (hi - lo) * uniform(seed, 2, idx))
    ph = phi[0] + (phi[1] - phi[0]) * uniform(seed, 3, idx)
    reac = 1.0 - diluent
    X = np.zeros((K, n))
    X[0] = reac * ph / (ph + 2.0)
    X[1] = reac * 2.0 / (ph + 2.0)
    X[K - 1] = diluent
    pressure_R = P / R
    V = np.ones(n)
    total = pressure_R * V / Tn
    return pressure_R, Tn, V, np.ascontiguousarray(X[:K - 1] * total)


class Reactors:
    """A batch of reactors on the current CUDA device."""

    def __init__(self, mech: Mechanism, n: int, rtol=1e-6, atol=1e-12, t_end=1e-3, max_steps=200000,
                 slice_steps=0, warps_per_block=0, tables_in_shared=-1, flags=0):
        L = _bind()
        self.mech, self.n = mech, n
        self.N = mech.A + 2
        o = cb_bdf_options(rtol, atol, t_end, max_steps, slice_steps, warps_per_block, tables_in_shared, flags)
        h = C.c_void_p()
        _check(L.cb_reactors_create(mech.h, n, C.byref(o), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().cb_reactors_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, pressure_R, T, V, amounts):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (pressure_R, T, V, amounts)]
        assert arrs[3].shape == (self.N - 2, self.n)
        _check(lib().cb_reactors_set_state(self.h, *[a.ctypes.data for a in arrs]))

    def autotune(self, calib_reactors=0):
        t = cb_reactor_tuning()
        _check(lib().cb_reactors_autotune(self.h, calib_reactors, C.byref(t)))
        return t.as_dict()

    def integrate(self):
        st = cb_reactor_stats()
        _check(lib().cb_reactors_integrate(self.h, C.byref(st)))
        return st.as_dict()

    def results(self):
        ign = np.zeros(self.n)
        state = np.zeros((self.N, self.n))
        status = np.zeros(self.n, dtype=np.int32)
        steps = np.zeros(self.n, dtype=np.int32)
        _check(lib().cb_reactors_results(self.h, ign.ctypes.data, state.ctypes.data, status.ctypes.data,
                                         steps.ctypes.data))
        return {"ignition_delay": ign, "state": state, "status": status, "steps": steps}

    def set_outputs(self, n_points=0, peak_species=-1):
        """Trajectory points (uniform times over [0, t_end]) and the peak of one active species' mole
        fraction, recorded by the following integrations (the role of plot.rs:76-138)."""
        _check(lib().cb_reactors_set_outputs(self.h, n_points, peak_species))
        self.n_points, self.peak_species = n_points, peak_species

    def outputs(self):
        """{times [P], trajectory [P, N, n], peak_time [n], peak_fraction [n], peak_state [N, n]} (the
        entries that were requested)."""
        P, n, N = getattr(self, "n_points", 0), self.n, self.N
        out = {}
        t = traj = pt = pf = ps = None
        if P:
            t, traj = np.zeros(P), np.zeros((P, N, n))
            out.update(times=t, trajectory=traj)
        if getattr(self, "peak_species", -1) >= 0:
            pt, pf, ps = np.zeros(n), np.zeros(n), np.zeros((N, n))
            out.update(peak_time=pt, peak_fraction=pf, peak_state=ps)
        ptr = lambda a: None if a is None else a.ctypes.data
        _check(lib().cb_reactors_outputs(self.h, ptr(t), ptr(traj), ptr(pt), ptr(pf), ptr(ps)))
        return out

    def eval(self, pressure_R, states):
        """(f [m, N], J [m, N, N]) of the integrator at the given states [m, N]."""
        y = np.ascontiguousarray(states, dtype=np.float64)
        m = y.shape[0]
        p = np.ascontiguousarray(pressure_R, dtype=np.float64)
        f = np.zeros((m, self.N))
        J = np.zeros((m, self.N, self.N))
        _check(lib().cb_reactors_eval(self.h, m, p.ctypes.data, y.ctypes.data, f.ctypes.data, J.ctypes.data))
        return f, J
