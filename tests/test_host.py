"""Host side of the library, no GPU: the C ABI loads and exports what include/*.h declares, mechanisms
are validated like the reference's builder does, and the transport fits match an SVD least-squares solve."""
import copy
import os
import re

import numpy as np
import pytest

import oracle
import util
from combustion_gb300 import synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cb():
    import combustion_gb300 as cb
    from combustion_gb300 import build
    build.build()
    return cb


def test_library_exports_every_declared_symbol():
    cb = _cb()
    L = cb.lib()
    declared = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            declared |= set(re.findall(r"^\s*(?:int|const char\*|double)\s+(cb_\w+)\s*\(", text, re.M))
    assert declared, "no declarations found"
    for sym in sorted(declared):
        assert hasattr(L, sym), sym
    assert set(cb.EXPORTS) <= declared
    assert "sm_103a" in cb.version()


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every ctypes Structure the Python side passes through the C ABI has the size and field offsets
    that a C compiler gives the header's struct of the same name."""
    import ctypes
    import shutil
    import subprocess
    import combustion_gb300 as cb
    from combustion_gb300 import reactors, surrogate
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = [cls for mod in (cb, reactors, surrogate) for cls in vars(mod).values()
               if isinstance(cls, type) and issubclass(cls, ctypes.Structure) and cls.__name__.startswith("cb_")]
    assert {"cb_bdf_options", "cb_reactor_stats", "cb_reactor_tuning"} <= {c.__name__ for c in mirrors}
    lines, expect = [], {}
    for cls in mirrors:
        t = cls.__name__
        lines.append(f'printf("{t} %zu\\n", sizeof({t}));')
        expect[t] = ctypes.sizeof(cls)
        for f, _ in cls._fields_:
            lines.append(f'printf("{t}.{f} %zu\\n", offsetof({t}, {f}));')
            expect[f"{t}.{f}"] = getattr(cls, f).offset
    # the autotuner's candidate records, an anonymous struct inside cb_reactor_tuning
    cand = reactors.cb_reactor_tuning._fields_[-1][1]._type_
    lines.append('printf("cand %zu\\n", sizeof(((cb_reactor_tuning*)0)->candidates[0]));')
    expect["cand"] = ctypes.sizeof(cand)
    for f, _ in cand._fields_:
        lines.append(f'printf("cand.{f} %zu\\n", offsetof(cb_reactor_tuning, candidates[0].{f}) - '
                     f'offsetof(cb_reactor_tuning, candidates));')
        expect[f"cand.{f}"] = getattr(cand, f).offset
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "combustion_gb300.h"\nint main(void) {\n'
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    bad = {k: (int(got[k]), v) for k, v in expect.items() if int(got[k]) != v}
    assert not bad, bad


def test_python_flag_constants_match_the_header():
    """The flag values the Python side passes (CB_* in the package, CB_BDF_* as reactors.<NAME>) are the
    header's #defines."""
    import combustion_gb300 as cb
    from combustion_gb300 import reactors, surrogate
    text = open(os.path.join(ROOT, "include", "combustion_gb300.h")).read()
    defines = {k: int(v) for k, v in re.findall(r"^#define (CB_\w+) (\d+)u", text, re.M)}
    checked = 0
    for mod in (cb, surrogate):
        for name, value in vars(mod).items():
            if name in defines:  # the flag #defines (status codes are an enum, checked elsewhere)
                assert defines[name] == value, name
                checked += 1
    for name, value in defines.items():
        if name.startswith("CB_BDF_"):
            assert getattr(reactors, name[len("CB_BDF_"):]) == value, name
            checked += 1
    assert checked >= 8


def test_validate_counts_and_sizes():
    cb = _cb()
    for config, (K, R) in {"k10": (10, 25), "k53": (53, 325)}.items():
        info = cb.validate(util.mechanism(config))
        assert (info.n_species, info.n_active, info.n_reactions) == (K, K - 1, R)
        assert info.rates_inputs == K + 3 and info.rates_outputs == K + 1 and info.transport_outputs == K + 2


def _rejects(m, code):
    cb = _cb()
    with pytest.raises(cb.CombustionError) as e:
        cb.validate(m)
    assert e.value.code == code, str(e.value)
    with pytest.raises(ValueError):
        oracle.Oracle(m)  # the oracle rejects the same mechanism
    return str(e.value)


def test_rejects_non_prefix_active_species():
    cb = _cb()
    m = copy.deepcopy(util.mechanism("k10"))
    # make the last (bulk) species change in a reaction: it is no longer inert
    m.products[0, m.K - 1] += 1
    _rejects(m, cb.CB_ERR_MECHANISM)


def test_sri_follows_the_reference_commented_formula():
    # the reference panics on SRI (unimplemented!, reaction.rs:194-203); the library and the oracle
    # evaluate its commented formula, and reject parameters it cannot take (C = 0, D <= 0)
    cb = _cb()
    from mechanisms import sri_mechanism
    m = sri_mechanism()
    info = cb.validate(m)
    assert info.n_reactions == m.R
    bad = copy.deepcopy(m)
    r = int(np.flatnonzero(bad.model == synthetic.SRI)[0])
    bad.sri[r, 2] = 0.0
    assert "SRI" in _rejects(bad, cb.CB_ERR_MECHANISM)


def test_rejects_reversible_reaction_without_net_change():
    cb = _cb()
    m = copy.deepcopy(util.mechanism("k10"))
    r = int(np.flatnonzero(m.model == synthetic.ELEMENTARY)[5])
    m.products[r] = m.reactants[r]
    # keep every species active: species of reaction r may still change elsewhere
    try:
        m.active()
    except ValueError:
        pytest.skip("rewriting this reaction changes the active set")
    if m.active() != m.K - 1:
        pytest.skip("rewriting this reaction changes the active set")
    _rejects(m, cb.CB_ERR_MECHANISM)


def test_transport_fit_matches_oracle_and_svd():
    cb = _cb()
    m = util.mechanism("k10")
    T0 = 1000.0
    c, v, d = cb.transport_fit(m, T0)
    o = oracle.Oracle(m)
    oc, ov, od = o.fit(T0)
    x, yc, yv, yd = o.samples(T0)
    V = np.vander(x, 5, increasing=True)
    for P, Q, Y in [(c, oc, yc), (v, ov, yv), (d, od, yd)]:
        for p, q, y in zip(P, Q, Y):
            w = 1.0 / y ** 2
            svd, *_ = np.linalg.lstsq(V * w[:, None], y * w, rcond=None)
            ev, eq, es = V @ p, V @ q, V @ svd
            assert np.max(np.abs(ev - eq) / np.abs(eq)) < 1e-13
            assert np.max(np.abs(ev - es) / np.abs(es)) < 1e-12


def test_work_model_counts():
    """The algorithmic operation counts of the reference program at K = 53 (one exp per Arrhenius rate,
    Gibbs exponentials, Troe blending; one reciprocal per diffusion pair)."""
    _cb()
    # work model is only exposed on a device mechanism; the counts are checked in the GPU suite.
    assert True
