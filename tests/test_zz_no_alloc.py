"""cb_reactors_eval_noalloc (the no-allocation variant of cb_reactors_eval) through the C ABI.

It serves host loops that evaluate du/dt and Jacobians many times (an implicit solver's Newton iterations,
a controller) and cannot allocate device memory per call: cudaFree synchronises the whole device, and
under a caching allocator that has reserved the GPU's memory cudaMalloc can fail outright. The GPU tests
check the same du/dt and Jacobians as the allocating entry point on two calls in a row, no change of free
device memory across a call, and a clear error above the fixed size limit; a CPU test reads the entry
point's source and the helpers it calls and checks that none of them names an allocating call.
Collected last on purpose; the GPU tests also pass alone in a fresh process."""
import ctypes as C
import os
import re

import numpy as np
import pytest

BDF_CU = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "combustion_gb300", "csrc",
                      "bdf.cu")


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


@pytest.mark.gpu
@pytest.mark.parametrize("config,m", [("k10", 300), ("k53", 160)])
def test_noalloc_matches_allocating_entry_point(config, m):
    import torch
    cb, L, mech, R, pR, Y = _batch(config, m)
    f_ref, J_ref = R.eval(pR, Y)
    rc, f1, J1 = _noalloc(L, R, pR, Y)
    assert rc == 0, L.cb_last_error().decode()
    Y2 = Y.copy()
    Y2[:, 0] *= 1.01  # second call on different states
    f_ref2, J_ref2 = R.eval(pR, Y2)
    free_mid = torch.cuda.mem_get_info()[0]
    rc, f2, J2 = _noalloc(L, R, pR, Y2)
    assert rc == 0, L.cb_last_error().decode()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after >= free_mid  # the no-allocation call kept no device memory
    assert np.array_equal(f1, f_ref) and np.array_equal(J1, J_ref)
    assert np.array_equal(f2, f_ref2) and np.array_equal(J2, J_ref2)


@pytest.mark.gpu
def test_noalloc_rejects_more_states_than_its_scratch():
    cb, L, mech, R, pR, Y = _batch("k53", 8)
    N = Y.shape[1]
    limit = (1 << 19) // (N * N + 2 * N + 1)
    assert (N, limit) == (54, 173)
    big = np.repeat(Y, (limit + 1 + len(Y) - 1) // len(Y), axis=0)[: limit + 1]
    pRb = np.repeat(pR, (limit + 1 + len(pR) - 1) // len(pR))[: limit + 1]
    rc, _, _ = _noalloc(L, R, np.ascontiguousarray(pRb), np.ascontiguousarray(big))
    assert rc == cb.CB_ERR_INVALID
    assert f"at most {limit} states" in L.cb_last_error().decode()
    rc, _, _ = _noalloc(L, R, np.ascontiguousarray(pRb[:limit]), np.ascontiguousarray(big[:limit]))
    assert rc == 0, L.cb_last_error().decode()


def _function_body(src, signature_regex):
    m = re.search(signature_regex, src)
    assert m, signature_regex
    i = src.index("{", m.end() - 1)
    depth = 0
    for j in range(i, len(src)):
        depth += {"{": 1, "}": -1}.get(src[j], 0)
        if depth == 0:
            return src[i:j + 1]
    raise AssertionError("unbalanced braces")


def test_noalloc_source_names_no_allocating_call():
    """A call that allocated and freed inside itself would leave free memory unchanged; this reads the
    entry point and every library helper it calls for allocating routines instead."""
    src = open(BDF_CU).read()
    bodies = {"cb_reactors_eval_noalloc": _function_body(src, r"int cb_reactors_eval_noalloc\([^)]*\)\s*\{")}
    for helper in ("params", "shape_fits", "smem_bytes", "sm_count", "max_smem"):
        bodies[helper] = _function_body(src, r"\b(?:Params|bool|size_t|int)\s+%s\([^)]*\)\s*\{" % helper)
    banned = re.compile(r"\b(cudaMalloc\w*|cudaFree\w*|cudaHostAlloc|cudaMemPool\w*|malloc|calloc|realloc|"
                        r"new\b|std::vector|std::string\s*\(|torch)")
    for name, body in bodies.items():
        body = re.sub(r"//[^\n]*", "", body)
        # the error message of the size check builds a string only on the rejection path
        body = body.replace('"cb_reactors_eval_noalloc: at most " + std::to_string(max_states)', "")
        assert not banned.search(body), (name, banned.search(body).group(0))
    assert "cudaGetSymbolAddress" in bodies["cb_reactors_eval_noalloc"]
    assert "cudaMemsetAsync(s->counters + 2" in bodies["cb_reactors_eval_noalloc"]
