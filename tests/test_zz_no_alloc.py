"""cb_reactors_eval_noalloc (the no-allocation variant of cb_reactors_eval) through the C ABI: same du/dt
and Jacobians as the allocating entry point on two calls in a row, no change of free device memory
across a call, and a clear error above its fixed size limit. Collected last on purpose; it also passes
alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    import combustion_gb300 as cb
    from combustion_gb300 import reactors as RX
    L = RX._bind()
    vp = C.c_void_p
    L.cb_reactors_eval_noalloc.argtypes = [vp, C.c_int32, vp, vp, vp, vp]
    return cb, RX, L


def _batch(config, m):
    cb, RX, L = _lib()
    from combustion_gb300 import synthetic
    mech = cb.Mechanism(synthetic.generate_reactor_mechanism(config))
    R = RX.Reactors(mech, 4)
    cells = synthetic.generate_cells(mech.K, m, "k53" if config == "k53" else "k10", seed=6)
    Y = np.ascontiguousarray(np.vstack([cells.temperature, cells.volume, cells.amounts]).T)
    return cb, L, mech, R, np.ascontiguousarray(cells.pressure_R), Y


def _noalloc(L, R, pR, Y):
    m, N = Y.shape
    f = np.zeros((m, N))
    J = np.zeros((m, N, N))
    rc = L.cb_reactors_eval_noalloc(R.h, m, pR.ctypes.data, Y.ctypes.data, f.ctypes.data, J.ctypes.data)
    return rc, f, J


@pytest.mark.parametrize("config,m", [("k10", 300), ("k53", 160)])
def test_noalloc_matches_allocating_entry_point(config, m):
    import torch
    cb, L, mech, R, pR, Y = _batch(config, m)
    f_ref, J_ref = R.eval(pR, Y)
    rc, f1, J1 = _noalloc(L, R, pR, Y)
    assert rc == 0, L.cb_last_error().decode()
    free_before = torch.cuda.mem_get_info()[0]
    Y2 = Y.copy()
    Y2[:, 0] *= 1.01  # second call on different states
    f_ref2, J_ref2 = R.eval(pR, Y2)
    free_mid = torch.cuda.mem_get_info()[0]
    rc, f2, J2 = _noalloc(L, R, pR, Y2)
    assert rc == 0, L.cb_last_error().decode()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after >= free_mid  # the no-allocation call took no device memory
    assert np.array_equal(f1, f_ref) and np.array_equal(J1, J_ref)
    assert np.array_equal(f2, f_ref2) and np.array_equal(J2, J_ref2)
    del free_before


def test_noalloc_rejects_more_states_than_its_scratch():
    cb, L, mech, R, pR, Y = _batch("k53", 8)
    N = Y.shape[1]
    limit = (1 << 19) // (N * N + 2 * N + 1)
    big = np.repeat(Y, (limit + 1 + len(Y) - 1) // len(Y), axis=0)[: limit + 1]
    pRb = np.repeat(pR, (limit + 1 + len(pR) - 1) // len(pR))[: limit + 1]
    rc, _, _ = _noalloc(L, R, np.ascontiguousarray(pRb), np.ascontiguousarray(big))
    assert rc == cb.CB_ERR_INVALID
    assert f"at most {limit} states" in L.cb_last_error().decode()
    rc, _, _ = _noalloc(L, R, np.ascontiguousarray(pRb[:limit]), np.ascontiguousarray(big[:limit]))
    assert rc == 0, L.cb_last_error().decode()
