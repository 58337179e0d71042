"""CPU reference for the batched reactors (TEST INFRASTRUCTURE ONLY: the checker of the GPU integrator;
the product library never uses it).

One reactor at a time with scipy's BDF (scipy.integrate.solve_ivp, method "BDF", finite-difference
Jacobian): the role of the reference's cvode crate (cvode/lib.rs:17-47: CVODE BDF, dense solver,
difference-quotient Jacobian) on the FP64 rates restatement of the oracle (reaction.rs:356-391). The
ignition delay is the time of the largest dT/dt over the accepted steps, refined by the vertex of the
parabola through the samples around it (the GPU integrator's definition).
"""
from __future__ import annotations

import numpy as np


def rhs(o, pressure_R, y):
    """du/dt for u = [T, V, n_0 .. n_{A-1}] (rows) or a batch of states (columns)."""
    y = np.asarray(y, dtype=np.float64)
    Y = y.reshape(len(y), -1)
    n = Y.shape[1]
    ins = [np.full(n, pressure_R), np.full(n, 1.0 / pressure_R)] + [np.ascontiguousarray(r) for r in Y]
    out = o.rates(ins)
    return out if y.ndim == 2 else out[:, 0]


def ignition_time(t, g):
    """Vertex of the parabola through the largest sample of g and its neighbours (or the sample)."""
    i = int(np.argmax(g))
    if 0 < i < len(t) - 1:
        ta, tb, tc = t[i - 1], t[i], t[i + 1]
        ga, gb, gc = g[i - 1], g[i], g[i + 1]
        d1, d2 = tb - ta, tb - tc
        den = d1 * (gb - gc) - d2 * (gb - ga)
        if den != 0.0:
            v = tb - 0.5 * (d1 * d1 * (gb - gc) - d2 * d2 * (gb - ga)) / den
            if ta < v < tc:
                return float(v)
    return float(t[i])


def trajectory(o, pressure_R, y0, t_end, times, peak_species, rtol=1e-9, atol=1e-14):
    """States at `times` (dense output) and, over the accepted steps, the largest mole fraction among the
    active species of `peak_species` with its time: the CPU check of the GPU integrator's outputs."""
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda t, y: rhs(o, pressure_R, y), (0.0, t_end), np.asarray(y0, dtype=np.float64),
                    method="BDF", rtol=rtol, atol=atol, dense_output=True)
    if sol.status != 0:
        raise RuntimeError(sol.message)
    x = sol.y[2 + peak_species] / sol.y[2:].sum(axis=0)
    i = int(np.argmax(x))
    return sol.sol(np.asarray(times)), float(sol.t[i]), float(x[i])


def integrate(o, pressure_R, y0, t_end, rtol=1e-9, atol=1e-14):
    """(ignition delay, final state, number of steps) of one reactor."""
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda t, y: rhs(o, pressure_R, y), (0.0, t_end), np.asarray(y0, dtype=np.float64),
                    method="BDF", rtol=rtol, atol=atol)
    if sol.status != 0:
        raise RuntimeError(sol.message)
    g = rhs(o, pressure_R, sol.y)[0]
    return ignition_time(sol.t, g), sol.y[:, -1], len(sol.t) - 1


def _integrate_job(args):
    mech, pressure_R, y0, t_end, rtol, atol = args
    import oracle
    return integrate(oracle.Oracle(mech), pressure_R, y0, t_end, rtol=rtol, atol=atol)


def integrate_batch(mech, pressure_R, Y0, t_end, rtol=1e-9, atol=1e-14, workers=0):
    """integrate() of every reactor (pressure_R [n], initial states Y0 [n][N]) over a pool of spawned
    processes (spawned, not forked: the caller may hold a CUDA context). Returns a list of
    (ignition delay, final state, steps)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os
    workers = workers or min(16, os.cpu_count() or 1, len(Y0))
    jobs = [(mech, float(pressure_R[i]), np.asarray(Y0[i], dtype=np.float64), t_end, rtol, atol)
            for i in range(len(Y0))]
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_integrate_job, jobs))
