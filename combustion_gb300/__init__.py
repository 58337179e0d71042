"""combustion_gb300: GB300 per-cell chemistry (species rates + mixture-averaged transport).

Python host mirror of the reference's interface for this path, over the C ABI of
libcombustion_gb300.so (include/combustion_gb300.h):

  reference                                        here
  combustion::new(&model)             lib.rs:127    Mechanism(mech)                (tables on the GPU)
  transport::properties::<5>(...)   transport.rs:212 Mechanism.transport_setup(T0, mu0, lambda0)
  device::assemble(reaction::rates(..), _)(c, in)    Mechanism.rates(inputs, outputs, ...)
  device::assemble(transport::properties(..))(c, in) Mechanism.transport(inputs, outputs, ...)
  reaction::reactions_rates          reaction.rs:329 Mechanism.reaction_rates(...)

Inputs and outputs are struct-of-arrays, one array per input/output in the reference's order.
Device arrays are torch CUDA tensors (2-D, one row per array, or a list of 1-D tensors); host arrays
are numpy arrays and go through the CB_HOST_MEMORY path. There is no CPU fallback: without the
built library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import synthetic  # noqa: F401  (seeded workloads)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcombustion_gb300.so")

CB_OK, CB_ERR_INVALID, CB_ERR_MECHANISM, CB_ERR_CUDA, CB_ERR_NOT_READY, CB_ERR_UNSUPPORTED, CB_ERR_DEVICE = range(7)
CB_HOST_MEMORY = 1
CB_UNIFORM_PRESSURE = 2

EXPORTS = ["cb_mech_create", "cb_mech_validate", "cb_mech_destroy", "cb_mech_query", "cb_transport_setup",
           "cb_transport_fit", "cb_transport_coefficients", "cb_rates_f64", "cb_reaction_rates_f64",
           "cb_transport_f64", "cb_rates_transport_f64", "cb_work_model", "cb_synchronize", "cb_last_error",
           "cb_version", "cb_device_fp64_peak", "cb_fp64_math", "cb_rates_mixed", "cb_transport_mixed",
           "cb_rates_transport_mixed", "cb_generate_cells", "cb_surrogate_create", "cb_surrogate_destroy",
           "cb_surrogate_query", "cb_surrogate_generate", "cb_surrogate_train", "cb_surrogate_transport",
           "cb_surrogate_get_params", "cb_surrogate_set_params", "cb_surrogate_normalisation",
           "cb_surrogate_evaluate", "cb_reactors_create", "cb_reactors_destroy", "cb_reactors_set_state",
           "cb_reactors_autotune", "cb_reactors_integrate", "cb_reactors_results", "cb_reactors_eval",
           "cb_reactors_eval_noalloc", "cb_yaml_load", "cb_yaml_desc", "cb_yaml_free", "cb_debug_stage_wait_polls",
           "cb_surrogate_transport_pair"]


class CombustionError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[code {code}] {msg}")
        self.code = code


class cb_mech_desc(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_reactions", C.c_int32)] + [
        (name, C.c_void_p) for name in ("molar_mass", "nasa7_split", "nasa7", "geometry", "diameter", "well_depth",
                                        "polarizability", "dipole", "rotational_relaxation", "reactants", "products",
                                        "model", "rate", "k0", "troe", "sri", "efficiencies")]


class cb_mech_info(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_active", C.c_int32), ("n_reactions", C.c_int32),
                ("transport_ready", C.c_int32), ("T0", C.c_double), ("viscosity0", C.c_double),
                ("conductivity0", C.c_double), ("rates_inputs", C.c_int32), ("rates_outputs", C.c_int32),
                ("transport_inputs", C.c_int32), ("transport_outputs", C.c_int32),
                ("device_table_bytes", C.c_size_t)]


class cb_work(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("flops", "exps", "logs", "divs", "sqrts", "bytes_in", "bytes_out")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def lib():
    """The loaded C library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CombustionError(CB_ERR_UNSUPPORTED, f"{LIB_PATH} is missing: run combustion_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, sz = C.c_void_p, C.c_size_t
        L.cb_mech_create.argtypes = [C.POINTER(cb_mech_desc), C.POINTER(vp)]
        L.cb_mech_validate.argtypes = [C.POINTER(cb_mech_desc), C.POINTER(cb_mech_info)]
        L.cb_mech_destroy.argtypes = [vp]
        L.cb_mech_query.argtypes = [vp, C.POINTER(cb_mech_info)]
        L.cb_transport_setup.argtypes = [vp, C.c_double, C.c_double, C.c_double]
        L.cb_transport_fit.argtypes = [C.POINTER(cb_mech_desc), C.c_double, vp, vp, vp]
        L.cb_transport_coefficients.argtypes = [vp, vp, vp, vp]
        for f in ("cb_rates_f64", "cb_reaction_rates_f64", "cb_transport_f64", "cb_rates_mixed", "cb_transport_mixed"):
            getattr(L, f).argtypes = [vp, sz, vp, vp, C.c_uint32, vp]
        L.cb_rates_transport_f64.argtypes = [vp, sz, vp, vp, vp, C.c_uint32, vp]
        L.cb_rates_transport_mixed.argtypes = [vp, sz, vp, vp, vp, C.c_uint32, vp]
        L.cb_work_model.argtypes = [vp, C.POINTER(cb_work), C.POINTER(cb_work)]
        L.cb_count_nonfinite.argtypes = [vp, sz, C.c_int32, vp, C.POINTER(C.c_uint64), C.c_uint32, vp]
        L.cb_synchronize.argtypes = [vp, vp]
        L.cb_last_error.restype = C.c_char_p
        L.cb_version.restype = C.c_char_p
        L.cb_device_fp64_peak.argtypes = [C.POINTER(C.c_double)]
        L.cb_fp64_math.argtypes = [C.c_int, vp, vp, sz, vp]
        L.cb_debug_stage_wait_polls.argtypes = [C.c_int64]
        _lib = L
    return _lib


def _check(rc):
    if rc != CB_OK:
        raise CombustionError(rc, lib().cb_last_error().decode())


class _Desc:
    """A cb_mech_desc over numpy copies of a synthetic.Mechanism (kept alive with the struct)."""

    def __init__(self, mech):
        self.keep = []

        def p(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self.keep.append(a)
            return a.ctypes.data

        f8, i4, u1 = np.float64, np.int32, np.uint8
        self.desc = cb_mech_desc(
            mech.K, mech.R, p(mech.molar_mass, f8), p(mech.nasa7_split, f8), p(mech.nasa7, f8), p(mech.geometry, i4),
            p(mech.diameter, f8), p(mech.well_depth, f8), p(mech.polarizability, f8), p(mech.dipole, f8),
            p(mech.rotational_relaxation, f8), p(mech.reactants, u1), p(mech.products, u1), p(mech.model, i4),
            p(mech.rate, f8), p(mech.k0, f8), p(mech.troe, f8), p(mech.sri, f8), p(mech.efficiencies, f8))


def validate(mech) -> cb_mech_info:
    """combustion::new without a device: the checks the reference's builder makes, and the sizes."""
    d = _Desc(mech)
    info = cb_mech_info()
    _check(lib().cb_mech_validate(C.byref(d.desc), C.byref(info)))
    return info


def transport_fit(mech, T0: float):
    """transport::Polynomials::new on the host: raw fits (cond [K,5], visc [K,5], diff [K*K,5])."""
    d = _Desc(mech)
    K = mech.K
    c, v, df = np.zeros((K, 5)), np.zeros((K, 5)), np.zeros((K * K, 5))
    _check(lib().cb_transport_fit(C.byref(d.desc), T0, c.ctypes.data, v.ctypes.data, df.ctypes.data))
    return c, v, df


def _ptr_array(arrays):
    return (C.c_void_p * len(arrays))(*arrays)


class Mechanism:
    """A mechanism uploaded to the current CUDA device (combustion::new + the rates tables)."""

    def __init__(self, mech):
        self.mech = mech
        d = _Desc(mech)
        h = C.c_void_p()
        _check(lib().cb_mech_create(C.byref(d.desc), C.byref(h)))
        self.h = h
        self.info = self.query()
        self.K, self.A, self.R = self.info.n_species, self.info.n_active, self.info.n_reactions

    def close(self):
        if getattr(self, "h", None):
            lib().cb_mech_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def query(self) -> cb_mech_info:
        info = cb_mech_info()
        _check(lib().cb_mech_query(self.h, C.byref(info)))
        return info

    def transport_setup(self, T0, viscosity0, conductivity0):
        _check(lib().cb_transport_setup(self.h, T0, viscosity0, conductivity0))
        self.info = self.query()

    def transport_coefficients(self):
        K = self.K
        c, v, d = np.zeros((K, 5)), np.zeros((K, 5)), np.zeros((K * K, 5))
        _check(lib().cb_transport_coefficients(self.h, c.ctypes.data, v.ctypes.data, d.ctypes.data))
        return c, v, d

    def work_model(self):
        r, t = cb_work(), cb_work()
        _check(lib().cb_work_model(self.h, C.byref(r), C.byref(t)))
        return r.as_dict(), t.as_dict()

    def synchronize(self, stream=None):
        _check(lib().cb_synchronize(self.h, stream))

    # ---- calls -------------------------------------------------------------------------------
    @staticmethod
    def _rows(x):
        """Per-array base addresses of a 2-D tensor/array (one row per array) or a list of 1-D ones."""
        if isinstance(x, (list, tuple)):
            return [Mechanism._addr(a) for a in x], len(x[0]) if len(x) else 0
        import torch
        if isinstance(x, torch.Tensor):
            assert x.dtype == torch.float64 and x.dim() == 2 and x.stride(1) == 1
            base, s = x.data_ptr(), x.stride(0) * 8
            return [base + q * s for q in range(x.shape[0])], x.shape[1]
        assert x.dtype == np.float64 and x.ndim == 2 and x.strides[1] == 8
        base, s = x.ctypes.data, x.strides[0]
        return [base + q * s for q in range(x.shape[0])], x.shape[1]

    @staticmethod
    def _addr(a):
        try:
            import torch
            if isinstance(a, torch.Tensor):
                assert a.dtype == torch.float64 and a.is_contiguous()
                return a.data_ptr()
        except ImportError:
            pass
        assert a.dtype == np.float64 and a.flags.c_contiguous
        return a.ctypes.data

    @staticmethod
    def _is_host(x):
        first = x[0] if isinstance(x, (list, tuple)) else x
        return isinstance(first, np.ndarray)

    @staticmethod
    def _stream(stream):
        if stream is None:
            try:
                import torch
                if torch.cuda.is_available():
                    return torch.cuda.current_stream().cuda_stream
            except ImportError:
                pass
            return None
        return getattr(stream, "cuda_stream", stream)

    def _call(self, fn, inputs, outputs, flags, stream, n=None):
        ins, n_in = self._rows(inputs)
        outs, n_out = self._rows(outputs)
        n = n if n is not None else n_out
        if self._is_host(outputs):
            flags |= CB_HOST_MEMORY
        _check(fn(self.h, n, _ptr_array(ins), _ptr_array(outs), flags, None if flags & CB_HOST_MEMORY else self._stream(stream)))
        return outputs

    def rates(self, inputs, outputs, uniform_pressure=False, stream=None, mixed=False):
        """inputs [K+3]: P/R, R/P, T, V, n_0..n_{K-2}; outputs [A+2]: dT/dt, dV/dt, wdot_0..wdot_{A-1}.
        mixed=True: the mixed-precision form (cb_rates_mixed)."""
        fn = lib().cb_rates_mixed if mixed else lib().cb_rates_f64
        return self._call(fn, inputs, outputs, CB_UNIFORM_PRESSURE if uniform_pressure else 0, stream)

    def reaction_rates(self, inputs, outputs, stream=None):
        """inputs [K+2]: P/R, T, V, n_0..n_{K-2}; outputs [R]: rate of progress of each reaction."""
        return self._call(lib().cb_reaction_rates_f64, inputs, outputs, 0, stream)

    def transport(self, inputs, outputs, stream=None, mixed=False):
        """inputs [K+1]: sum n, T/T0, n_0..n_{K-2}; outputs [K+2]: lambda/lambda0, mu/mu0, rhoD_k/mu0."""
        fn = lib().cb_transport_mixed if mixed else lib().cb_transport_f64
        return self._call(fn, inputs, outputs, 0, stream)

    def count_nonfinite(self, arrays, stream=None):
        """Number of NaN or infinite values in the rows of `arrays` (device tensors or host arrays)."""
        rows, n = self._rows(arrays)
        flags = CB_HOST_MEMORY if self._is_host(arrays) else 0
        c = C.c_uint64()
        _check(lib().cb_count_nonfinite(self.h, n, len(rows), _ptr_array(rows), C.byref(c), flags,
                                        None if flags else self._stream(stream)))
        return int(c.value)

    def rates_transport(self, inputs, rates_out, transport_out, stream=None, mixed=False):
        """Both paths on the same cells (transport at sum n = P/R V / T, T/T0)."""
        ins, _ = self._rows(inputs)
        ro, n = self._rows(rates_out)
        to, _ = self._rows(transport_out)
        flags = CB_HOST_MEMORY if self._is_host(rates_out) else 0
        fn = lib().cb_rates_transport_mixed if mixed else lib().cb_rates_transport_f64
        _check(fn(self.h, n, _ptr_array(ins), _ptr_array(ro), _ptr_array(to), flags,
                  None if flags else self._stream(stream)))
        return rates_out, transport_out


def device_fp64_peak() -> float:
    """FP64 FMAs per second of the current GPU (measured)."""
    v = C.c_double()
    _check(lib().cb_device_fp64_peak(C.byref(v)))
    return v.value


def fp64_math(which: str, x):
    """The kernels' FP64 exp/log/reciprocal on a CUDA float64 tensor (which: "exp", "log", "rcp")."""
    import torch
    code = {"exp": 0, "log": 1, "rcp": 2}[which]
    x = x.contiguous()
    y = torch.empty_like(x)
    _check(lib().cb_fp64_math(code, x.data_ptr(), y.data_ptr(), x.numel(), torch.cuda.current_stream().cuda_stream))
    return y


def debug_stage_wait_polls(polls: int) -> None:
    """Test hook: polls of the plain FP64 kernels' first table-staging wait (negative: the default)."""
    _check(lib().cb_debug_stage_wait_polls(int(polls)))


def version() -> str:
    return lib().cb_version().decode()
