"""Learned transport surrogate over the C ABI (cb_surrogate_* in include/combustion_gb300.h).

No reference counterpart: the network is trained on the plain FP64 transport kernel's outputs
(transport.rs:179-214 restated on the GPU) and its trust gate sends cells back to that kernel.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import CombustionError, Mechanism, _check, _ptr_array, lib

CB_UNIFORM_PRESSURE = 2
CB_SURROGATE_NO_GATE = 8
CB_SURROGATE_TIMING = 16


class cb_cell_distribution(C.Structure):
    _fields_ = [("T_min", C.c_double), ("T_max", C.c_double), ("P_min", C.c_double), ("P_max", C.c_double),
                ("alpha", C.c_double), ("seed", C.c_uint64)]


class cb_surrogate_desc(C.Structure):
    _fields_ = [("width", C.c_int32), ("hidden_layers", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("lr_final", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint64)]


class cb_surrogate_info(C.Structure):
    _fields_ = [("n_features", C.c_int32), ("n_in", C.c_int32), ("n_out", C.c_int32), ("width", C.c_int32),
                ("hidden_layers", C.c_int32), ("batch", C.c_int32), ("n_params", C.c_int64),
                ("n_weights", C.c_int64), ("n_train", C.c_int64), ("steps_done", C.c_int64),
                ("weight_offset", C.c_int64 * 8), ("bias_offset", C.c_int64 * 8), ("dims", C.c_int32 * 9)]


class cb_surrogate_stats(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("fallback_cells", C.c_uint64), ("audited_cells", C.c_uint64),
                ("audit_max_rel_err", C.c_double * 3), ("audit_rms_rel_err", C.c_double * 3),
                ("ms_features", C.c_double), ("ms_network", C.c_double), ("ms_outputs", C.c_double),
                ("ms_gate", C.c_double)]

    def as_dict(self):
        return {"cells": self.cells, "fallback_cells": self.fallback_cells, "audited_cells": self.audited_cells,
                "audit_max_rel_err": list(self.audit_max_rel_err), "audit_rms_rel_err": list(self.audit_rms_rel_err),
                "ms": {"features": self.ms_features, "network": self.ms_network, "outputs": self.ms_outputs,
                       "gate": self.ms_gate}}


class cb_surrogate_gate(C.Structure):
    _fields_ = [("threshold", C.c_double), ("audit_stride", C.c_uint32), ("fallback", C.c_uint32),
                ("disagreement", C.c_void_p)]


CB_FALLBACK_MIXED, CB_FALLBACK_PLAIN = 0, 1


# Cell distributions of the named workloads (T in K, P in atm, Dirichlet alpha).
DISTRIBUTIONS = {
    "k10": dict(T_min=800.0, T_max=2800.0, P_min=1.0, P_max=1.0, alpha=0.5),
    "k53": dict(T_min=300.0, T_max=3000.0, P_min=0.1, P_max=40.0, alpha=0.3),
    "k250": dict(T_min=300.0, T_max=3000.0, P_min=0.1, P_max=40.0, alpha=0.3),
}

_bound = False


def _bind():
    global _bound
    if _bound:
        return lib()
    L = lib()
    vp, sz = C.c_void_p, C.c_size_t
    L.cb_generate_cells.argtypes = [vp, sz, sz, C.POINTER(cb_cell_distribution), vp, vp]
    L.cb_surrogate_create.argtypes = [vp, C.POINTER(cb_surrogate_desc), C.POINTER(vp)]
    L.cb_surrogate_destroy.argtypes = [vp]
    L.cb_surrogate_query.argtypes = [vp, C.POINTER(cb_surrogate_info)]
    L.cb_surrogate_generate.argtypes = [vp, sz, C.POINTER(cb_cell_distribution)]
    L.cb_surrogate_train.argtypes = [vp, C.c_int32, vp]
    L.cb_surrogate_transport.argtypes = [vp, sz, vp, vp, C.c_uint32, C.c_uint32, C.POINTER(cb_surrogate_stats), vp]
    L.cb_surrogate_get_params.argtypes = [vp, vp]
    L.cb_surrogate_set_params.argtypes = [vp, vp]
    L.cb_surrogate_normalisation.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.cb_surrogate_evaluate.argtypes = [vp, C.c_int32, vp, vp, vp, vp, vp]
    L.cb_surrogate_transport_pair.argtypes = [vp, vp, sz, vp, vp, C.c_uint32, C.POINTER(cb_surrogate_gate),
                                              C.POINTER(cb_surrogate_stats), vp]
    _bound = True
    return L


def distribution(name: str = "k53", seed: int = 2, **over) -> cb_cell_distribution:
    d = dict(DISTRIBUTIONS[name])
    d.update(over)
    return cb_cell_distribution(d["T_min"], d["T_max"], d["P_min"], d["P_max"], d["alpha"], seed)


def generate_cells(mech: Mechanism, n: int, dist: cb_cell_distribution, offset: int = 0, stream=None):
    """Seeded rates-layout cells [K+3, n] on the current CUDA device (torch float64)."""
    import torch
    L = _bind()
    out = torch.empty((mech.K + 3, n), dtype=torch.float64, device="cuda")
    rows, _ = Mechanism._rows(out)
    _check(L.cb_generate_cells(mech.h, n, offset, C.byref(dist), _ptr_array(rows), Mechanism._stream(stream)))
    return out


class Surrogate:
    """MLP transport surrogate bound to a Mechanism whose transport is set up."""

    def __init__(self, mech: Mechanism, width=256, hidden_layers=4, batch=65536, lr=1e-3, lr_final=1e-3,
                 beta1=0.9, beta2=0.999, eps=1e-8, seed=3):
        L = _bind()
        self.mech = mech
        d = cb_surrogate_desc(width, hidden_layers, batch, lr, lr_final, beta1, beta2, eps, seed)
        h = C.c_void_p()
        _check(L.cb_surrogate_create(mech.h, C.byref(d), C.byref(h)))
        self.h = h
        self.info = self.query()

    def close(self):
        if getattr(self, "h", None):
            lib().cb_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def query(self) -> cb_surrogate_info:
        info = cb_surrogate_info()
        _check(lib().cb_surrogate_query(self.h, C.byref(info)))
        return info

    @property
    def dims(self):
        i = self.info
        return [i.dims[l] for l in range(i.hidden_layers + 2)]

    def layers(self, flat):
        """Split a flat parameter vector into [(W [out, in], b [out])] per layer."""
        i, d, out = self.info, self.dims, []
        for l in range(i.hidden_layers + 1):
            w0, b0 = i.weight_offset[l], i.bias_offset[l]
            out.append((flat[w0:w0 + d[l + 1] * d[l]].reshape(d[l + 1], d[l]), flat[b0:b0 + d[l + 1]]))
        return out

    def generate(self, n_train: int, dist: cb_cell_distribution):
        _check(lib().cb_surrogate_generate(self.h, n_train, C.byref(dist)))
        self.info = self.query()

    def train(self, steps: int) -> np.ndarray:
        losses = np.zeros(steps, dtype=np.float32)
        _check(lib().cb_surrogate_train(self.h, steps, losses.ctypes.data))
        self.info = self.query()
        return losses

    def params(self) -> np.ndarray:
        p = np.zeros(self.info.n_params, dtype=np.float32)
        _check(lib().cb_surrogate_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.info.n_params
        _check(lib().cb_surrogate_set_params(self.h, p.ctypes.data))
        self.info = self.query()

    def normalisation(self):
        nf = self.info.n_features
        a = [np.zeros(nf, dtype=np.float32) for _ in range(6)]
        _check(lib().cb_surrogate_normalisation(self.h, *[x.ctypes.data for x in a]))
        return dict(zip(("in_mean", "in_rstd", "out_mean", "out_std", "in_lo", "in_hi"), a))

    def evaluate(self, features: np.ndarray, targets: np.ndarray, outputs=True):
        """One forward + backward pass on host rows: (loss, grads [n_params], outputs [rows, n_out])."""
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        rows = f.shape[0]
        assert f.shape == (rows, self.info.n_in) and t.shape == (rows, self.info.n_out)
        loss = C.c_float()
        g = np.zeros(self.info.n_params, dtype=np.float32)
        y = np.zeros((rows, self.info.n_out), dtype=np.float32) if outputs else None
        _check(lib().cb_surrogate_evaluate(self.h, rows, f.ctypes.data, t.ctypes.data, C.byref(loss), g.ctypes.data,
                                           y.ctypes.data if outputs else None))
        return loss.value, g, y

    def transport(self, inputs, outputs, audit_stride=1024, gate=True, uniform_pressure=False, stream=None,
                  timing=False):
        """Rates-layout inputs [K+3, n] -> transport outputs [K+2, n] (torch CUDA float64). Returns stats."""
        ins, _ = Mechanism._rows(inputs)
        outs, n = Mechanism._rows(outputs)
        flags = (0 if gate else CB_SURROGATE_NO_GATE) | (CB_UNIFORM_PRESSURE if uniform_pressure else 0)
        flags |= CB_SURROGATE_TIMING if timing else 0
        st = cb_surrogate_stats()
        _check(lib().cb_surrogate_transport(self.h, n, _ptr_array(ins), _ptr_array(outs), flags, audit_stride,
                                            C.byref(st), Mechanism._stream(stream)))
        return st.as_dict()


def transport_pair(a: Surrogate, b: Surrogate, inputs, outputs, threshold: float, audit_stride=1024,
                   fallback="mixed", disagreement=None, uniform_pressure=False, stream=None, timing=False):
    """Ensemble-gated transport (cb_surrogate_transport_pair): rates-layout inputs [K+3, n] -> outputs
    [K+2, n] (torch CUDA float64); cells whose networks disagree by more than `threshold` (or outside
    the training range) go to the mixed ("mixed") or plain ("plain") kernel. `disagreement` (torch CUDA
    float32 [n]) receives each cell's estimate. Returns the stats."""
    L = _bind()
    ins, _ = Mechanism._rows(inputs)
    outs, n = Mechanism._rows(outputs)
    flags = (CB_UNIFORM_PRESSURE if uniform_pressure else 0) | (CB_SURROGATE_TIMING if timing else 0)
    d_ptr = None
    if disagreement is not None:
        import torch
        assert disagreement.dtype == torch.float32 and disagreement.is_contiguous() and disagreement.numel() >= n
        d_ptr = disagreement.data_ptr()
    g = cb_surrogate_gate(float(threshold), int(audit_stride),
                          {"mixed": CB_FALLBACK_MIXED, "plain": CB_FALLBACK_PLAIN}[fallback], d_ptr)
    st = cb_surrogate_stats()
    _check(L.cb_surrogate_transport_pair(a.h, b.h, n, _ptr_array(ins), _ptr_array(outs), flags, C.byref(g),
                                         C.byref(st), Mechanism._stream(stream)))
    return st.as_dict()


def max_rel_err_per_cell(x, ref):
    """max_j |x_j - r_j| / |r_j| per cell (column) of two [K+2, n] torch tensors."""
    return ((x - ref).abs() / ref.abs()).amax(dim=0)


def calibrate_threshold(disagreement, err, tol: float) -> float:
    """The largest disagreement threshold t such that every calibration cell with disagreement <= t has
    a max relative error <= tol (cells sorted by disagreement; the longest prefix whose running maximum
    of the error stays within tol). Returns -inf when even the most confident cell misses tol (every
    cell then falls back)."""
    import torch
    d = disagreement.double()
    order = torch.argsort(d)
    run = torch.cummax(err.double()[order], dim=0).values
    ok = int((run <= tol).sum())  # running maximum is monotone: the prefix length
    if ok == 0:
        return float("-inf")
    t = float(d[order[ok - 1]])
    if ok < len(order) and float(d[order[ok]]) == t:  # ties at the boundary: step below the tied value
        t = float(np.nextafter(np.float32(t), np.float32(-np.inf)))
    return t


__all__ = ["Surrogate", "generate_cells", "distribution", "DISTRIBUTIONS", "CombustionError", "transport_pair",
           "calibrate_threshold", "max_rel_err_per_cell"]
