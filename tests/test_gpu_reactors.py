"""The batched BDF reactors through the C ABI: the integrator's warp-cooperative du/dt against the FP64
oracle, its Jacobian against finite differences of the oracle, ignition delays of 32 reactors
against the CPU reference integration (scipy's BDF on the oracle, oracle/reactor.py, over spawned host
processes), the autotuner and the graph
replays. Stated error bars: du/dt within 1e-12 of the oracle (condition-scaled); ignition delays within
0.1 % of the reference integration at rtol 1e-9 (32 reactors each at K = 53, rtol 1e-6, and K = 10,
rtol 1e-7) and, over 2048
reactors against the same integrator at rtol 1e-10, within 0.1 % at the median and 0.5 % at most (the
difference is the rtol 1e-6 integration error); final temperatures within 1e-5.
"""
import numpy as np
import pytest

import oracle
import util
from oracle import reactor

pytestmark = pytest.mark.gpu


def _setup(config, n, **kw):
    import combustion_gb300 as cb
    from combustion_gb300 import reactors as RX
    from combustion_gb300 import synthetic
    m = synthetic.generate_reactor_mechanism(config)
    mech = cb.Mechanism(m)
    R = RX.Reactors(mech, n, **kw)
    pR, T, V, am = RX.initial_states(m.K, n, seed=4)
    R.set_state(pR, T, V, am)
    return m, mech, R, (pR, T, V, am)


@pytest.mark.parametrize("config", ["k10", "k53"])
def test_rhs_and_jacobian_against_oracle(config):
    from combustion_gb300 import synthetic
    m, mech, R, _ = _setup(config, 4)
    o = oracle.Oracle(m)
    cells = synthetic.generate_cells(m.K, 16, config if config != "k10" else "k10", seed=5)
    pR = cells.pressure_R
    Y = np.vstack([cells.temperature, cells.volume, cells.amounts]).T.copy()
    f, J = R.eval(pR, Y)
    ins = o.rates_inputs(cells)
    ref, sc = o.rates(ins, scale=True)
    err = util.cond_err(f.T, ref, sc)
    print(config, "du/dt max cond err %.2e" % err.max())
    assert err.max() <= util.PLAIN_TOL * 10
    # Jacobian against central differences of the oracle
    worst = 0.0
    for s in range(4):
        y = Y[s]
        Jfd = np.zeros_like(J[s])
        for j in range(len(y)):
            h = 1e-6 * max(abs(y[j]), 1e-3 * (abs(y[0]) if j == 0 else max(1e-30, abs(y[2:]).max())))
            yp, ym = y.copy(), y.copy()
            yp[j] += h
            ym[j] -= h
            Jfd[:, j] = (reactor.rhs(o, pR[s], yp) - reactor.rhs(o, pR[s], ym)) / (yp[j] - ym[j])
        rel = np.linalg.norm(J[s] - Jfd) / np.linalg.norm(Jfd)
        worst = max(worst, rel)
        # the species block without falloff broadening terms is exact up to differencing error
    print(config, "Jacobian rel err (Frobenius) %.2e" % worst)
    assert worst < 2e-2


@pytest.mark.parametrize("config,n,rtol", [("k10", 32, 1e-7), ("k53", 32, 1e-6)])
def test_ignition_delays_against_cpu_bdf(config, n, rtol):
    """32 reactors against scipy's BDF at rtol 1e-9 on the oracle: K = 53 at the benchmark's rtol 1e-6;
    K = 10 at rtol 1e-7, because at 1e-6 its ~400 steps per reactor leave the ignition estimate (the
    vertex of the parabola through the largest dT/dt sample and its neighbours) up to 1.1e-3 off on one
    reactor of 32 (max 8.9e-4 on the rest): discretisation, which the tighter tolerance removes."""
    m, mech, R, (pR, T, V, am) = _setup(config, n, rtol=rtol, atol=1e-12, t_end=1e-3)
    st = R.integrate()
    res = R.results()
    print(config, st)
    assert st["finished"] == n and st["failed"] == 0
    Y0 = [np.concatenate([[T[i], V[i]], am[:, i]]) for i in range(n)]
    cpu = reactor.integrate_batch(m, pR, Y0, 1e-3, rtol=1e-9, atol=1e-15)
    worst = 0.0
    for i in range(n):
        tau, yf, steps = cpu[i]
        g = res["ignition_delay"][i]
        worst = max(worst, abs(g - tau) / tau)
        print(f"  reactor {i}: GPU tau {g:.6e} ({res['steps'][i]} steps), CPU tau {tau:.6e} ({steps} steps), "
              f"T_end {res['state'][0, i]:.4f} / {yf[0]:.4f}")
        assert abs(g - tau) <= 1e-3 * tau
        assert abs(res["state"][0, i] - yf[0]) <= 1e-5 * yf[0]
    print(f"{config}: {n} reactors, ignition delay max rel diff {worst:.2e} against scipy BDF on the oracle")


def test_autotune_graph_replays_and_tolerance_convergence():
    n = 2048
    m, mech, R, state = _setup("k10", n, rtol=1e-6, atol=1e-12, t_end=1e-3, slice_steps=64)
    tune = R.autotune(512)
    print(tune)
    assert tune["candidates"] and tune["warps_per_block"] >= 1
    # one workspace fits in shared memory: both placements are timed
    assert {c["global_memory"] for c in tune["candidates"]} == {0, 1}
    st = R.integrate()
    assert st["global_memory"] == tune["global_memory"]
    print(st)
    assert st["finished"] == n and st["graph_replays"] >= 2  # 64-step slices: several replays
    res = R.results()
    import combustion_gb300 as cb
    from combustion_gb300 import reactors as RX
    tight = RX.Reactors(mech, n, rtol=1e-10, atol=1e-16, t_end=1e-3, warps_per_block=tune["warps_per_block"],
                        tables_in_shared=tune["tables_in_shared"],
                        flags=RX.GLOBAL_MEMORY if tune["global_memory"] else 0)
    tight.set_state(*state)
    st2 = tight.integrate()
    ref = tight.results()
    assert st2["finished"] == n
    rel = np.abs(res["ignition_delay"] - ref["ignition_delay"]) / ref["ignition_delay"]
    print("ignition delay vs rtol 1e-10: max rel diff %.2e, median %.2e" % (rel.max(), np.median(rel)))
    assert np.median(rel) <= 1e-3 and rel.max() <= 5e-3


def test_global_memory_workspaces_match_shared_memory():
    """CB_BDF_GLOBAL_MEMORY, the placement large mechanisms get by themselves: the factorisation by
    panels (the same FMAs in the same order), the solves on its transpose and the workspaces in global
    memory take the shared-memory path's steps (53 species, 64 reactors, 64-step launches); the two
    kernels are compiled apart, so values may differ in the last bits, which can flip a step decision in
    a few reactors."""
    from combustion_gb300 import reactors as RX
    n = 64
    kw = dict(slice_steps=64, warps_per_block=2, tables_in_shared=0)
    m, mech, R, state = _setup("k53", n, **kw)
    st = R.integrate()
    res = R.results()
    Rg = RX.Reactors(mech, n, flags=RX.GLOBAL_MEMORY, **kw)
    Rg.set_state(*state)
    stg = Rg.integrate()
    resg = Rg.results()
    print(st, stg, sep="\n")
    assert st["finished"] == n and stg["finished"] == n and st["slices"] >= 8
    # the same arithmetic, so the same steps, except where a last-bit difference flips a step decision
    for key in ("steps", "rhs_evals", "jacobians", "factorizations"):
        assert abs(st[key] - stg[key]) <= 1e-3 * st[key] + 4, key
    rel = np.abs(res["ignition_delay"] / resg["ignition_delay"] - 1)
    assert np.median(rel) <= 1e-9 and rel.max() <= 1e-3
    same = np.equal(res["steps"], resg["steps"])
    assert same.mean() >= 0.9
    # those reactors' final states within 5 % of the integrator's own error scale atol + rtol |u|
    # (last-bit differences grow in trace species, whose amounts are at the absolute tolerance)
    d = np.abs(res["state"] - resg["state"]) / (1e-12 + 1e-6 * np.abs(res["state"]))
    assert np.max(d[:, same]) <= 5e-2


@pytest.mark.parametrize("flags", ["mixed", "reuse", "mixed+reuse", "lu32"])
def test_mixed_rhs_and_kept_factorisations(flags):
    """Ignition delays with the mixed-precision first Newton iterations, the kept factorisations, both,
    or the FP32 factorisation (global-memory placement), within 0.1 % of the FP64 integration (53
    species, 256 reactors); the mixed f(u) itself within the mixed form's bar of the FP64 oracle
    (condition-scaled)."""
    from combustion_gb300 import reactors as RX
    from combustion_gb300 import synthetic
    bits = {"mixed": RX.MIXED_RHS, "reuse": RX.REUSE_LU, "mixed+reuse": RX.MIXED_RHS | RX.REUSE_LU,
            "lu32": RX.GLOBAL_MEMORY | RX.LU32}[flags]
    n = 256
    m, mech, R, state = _setup("k53", n)
    st = R.integrate()
    ref = R.results()
    Rv = RX.Reactors(mech, n, flags=bits)
    Rv.set_state(*state)
    stv = Rv.integrate()
    res = Rv.results()
    print(st, stv, sep="\n")
    assert stv["finished"] == n
    rel = np.abs(res["ignition_delay"] - ref["ignition_delay"]) / ref["ignition_delay"]
    dT = np.abs(res["state"][0] - ref["state"][0]) / ref["state"][0]
    print(f"{flags}: ignition delay rel diff max {rel.max():.2e} median {np.median(rel):.2e}; final T {dT.max():.2e}; "
          f"factorisations {stv['factorizations']} vs {st['factorizations']}, rhs {stv['rhs_evals']} vs {st['rhs_evals']}")
    assert rel.max() <= 1e-3 and dT.max() <= 1e-5
    if bits & RX.REUSE_LU:
        assert stv["factorizations"] < st["factorizations"]
    if bits & RX.MIXED_RHS:
        o = oracle.Oracle(m)
        cells = synthetic.generate_cells(m.K, 16, "k53", seed=5)
        Y = np.vstack([cells.temperature, cells.volume, cells.amounts]).T.copy()
        f, _ = Rv.eval(cells.pressure_R, Y)
        ref_f, sc = o.rates(o.rates_inputs(cells), scale=True)
        err = util.cond_err(f.T, ref_f, sc)
        print("mixed du/dt max cond err %.2e" % err.max())
        assert err.max() <= util.MIXED_TOL


def test_large_mechanism_reactors():
    """250 species (251 states): the iteration matrix leaves shared memory, so workspaces and
    factorisations go to global memory by themselves; the mixed-precision first Newton iterations with
    kept factorisations, with FP64 or FP32 factors (the large configuration's form), against the FP64
    integration: ignition delays within 0.1 %."""
    from combustion_gb300 import reactors as RX
    n = 32
    m, mech, R, state = _setup("k250", n)
    st = R.integrate()
    ref = R.results()
    assert st["finished"] == n
    for name, bits in (("mixed+reuse", RX.MIXED_RHS | RX.REUSE_LU),
                       ("mixed+reuse+lu32", RX.MIXED_RHS | RX.REUSE_LU | RX.LU32)):
        Rv = RX.Reactors(mech, n, flags=bits)
        Rv.set_state(*state)
        stv = Rv.integrate()
        res = Rv.results()
        print(st, stv, sep="\n")
        assert stv["finished"] == n
        rel = np.abs(res["ignition_delay"] - ref["ignition_delay"]) / ref["ignition_delay"]
        print(f"k250 {name}: ignition delay rel diff max {rel.max():.2e} median {np.median(rel):.2e}")
        assert rel.max() <= 1e-3


def test_trajectory_and_species_peak_against_cpu_bdf():
    """Headless trajectory and species peak (the role of plot.rs:76-138): 21 states per reactor at
    uniform times from the integrator's interpolating polynomial against scipy's BDF dense output on the
    oracle at rtol 1e-9 (temperature within 1e-4, amounts within 1e-3 of each species' largest amount);
    the first and last points equal to the initial and final states; the largest mole fraction of one
    species among the active ones within 1 % of the CPU integration's, the state there consistent with
    it and no trajectory sample above it."""
    n, P, k_peak = 6, 21, 3
    m, mech, R, (pR, T, V, am) = _setup("k10", n, rtol=1e-6, atol=1e-12, t_end=1e-3)
    R.set_outputs(P, k_peak)
    st = R.integrate()
    res = R.results()
    out = R.outputs()
    assert st["finished"] == n
    traj, times = out["trajectory"], out["times"]
    assert traj.shape == (P, m.K + 1, n) and times[0] == 0.0 and times[-1] == 1e-3
    y0 = np.vstack([T, V, am])
    assert np.array_equal(traj[0], y0)
    assert np.array_equal(traj[-1], res["state"])
    ps, pf = out["peak_state"], out["peak_fraction"]
    assert np.allclose(ps[2 + k_peak] / ps[2:].sum(axis=0), pf, rtol=1e-12, atol=0)
    x_samples = traj[:, 2 + k_peak, :] / traj[:, 2:, :].sum(axis=1)
    assert np.all(x_samples.max(axis=0) <= pf * (1 + 1e-3))
    o = oracle.Oracle(m)
    for i in range(n):
        Y, t_pk, x_pk = reactor.trajectory(o, pR[i], y0[:, i], 1e-3, times, k_peak)
        g = traj[:, :, i].T
        relT = float(np.max(np.abs(g[0] - Y[0]) / Y[0]))
        scale = np.abs(Y[2:]).max(axis=1, keepdims=True)
        rel_n = float(np.max(np.abs(g[2:] - Y[2:]) / (1e-3 * scale + 1e-30)))
        print(f"  reactor {i}: T max rel {relT:.1e}, amounts {rel_n * 1e-3:.1e} of max; peak x {pf[i]:.6e} at "
              f"{out['peak_time'][i]:.4e} s, CPU {x_pk:.6e} at {t_pk:.4e} s")
        assert relT <= 1e-4 and rel_n <= 1.0
        assert abs(pf[i] - x_pk) <= 1e-2 * x_pk
