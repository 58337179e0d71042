"""Independent numpy restatement of the reference's per-cell formulas, vectorised over cells.

Used only to cross-check the C oracle (oracle/oracle.c): a second transcription of reaction.rs and
transport.rs, written as array code instead of per-cell loops, so that a slip in either shows up as a
disagreement. It follows the same operation order and the same constant folding
(ast/lib.rs:195-232); numpy's exp/log may differ from libm in the last bit, so agreement is checked
to a tolerance rather than bit for bit.
"""
import math

import numpy as np

F32MAX = float(np.finfo(np.float32).max)
F32MINPOS = float(np.finfo(np.float32).tiny)
kB, NA = 1.380649e-23, 6.02214076e23
R = kB * NA


def _f32(c):
    return np.float32(c) if abs(c) < 1e38 else np.float32(np.inf if c > 0 else -np.inf)


def canon_add(c):
    return 0.0 if _f32(c) == 0 else c


def canon_mul(c):
    f = _f32(c)
    if f == 0:
        return 0.0
    if f == 1:
        return 1.0
    if f == -1:
        return -1.0
    return c


def _cbrt_max():
    """(largest f32 whose cube is <= f32::MAX in f32 arithmetic, correctly rounded cbrt(f32::MAX))."""
    c = np.float32(np.cbrt(np.float64(F32MAX)))  # glibc cbrtf is correctly rounded here
    m = c
    with np.errstate(over="ignore"):
        while np.float32(np.float32(m * m) * m) > np.float32(F32MAX):
            m = np.nextafter(m, np.float32(-np.inf))
    return float(m), float(c)


def arrhenius(A, b, Ea, t):
    """reaction.rs:113-139 for all cells (t: dict of temperature arrays)."""
    if b <= -1.5:
        f, br = t["rcpT2"], b + 2
    elif b <= -0.5:
        f, br = t["rcpT"], b + 1
    elif b >= 3.5:
        f, br = t["T4"], b - 4
    elif b >= 2.5:
        f, br = t["T3"], b - 3
    elif b >= 1.5:
        f, br = t["T2"], b - 2
    elif b >= 0.5:
        f, br = t["T"], b - 1
    else:
        f, br = None, b
    terms = []
    if _f32(br) != 0:
        terms.append(canon_mul(br) * t["lnT"])
    if Ea != 0:
        terms.append(canon_mul(-Ea) * t["rcpT"])
    if terms:
        x = terms[0] if len(terms) == 1 else terms[0] + terms[1]
        lnA = canon_add(math.log(A))
        if lnA != 0:
            x = x + lnA
        e = np.exp(x)
        k = f * e if f is not None else e
    else:
        k = f * canon_mul(A) if f is not None else np.full_like(t["T"], A)
    return np.fmin(F32MAX, k)


def rates(mech, P_R, rcpP_R, T, V, n):
    """reaction.rs:356-391: returns [dT/dt, dV/dt, wdot_0..wdot_{A-1}] as a (A+2, N) array."""
    K, Rn = mech.K, mech.R
    A = mech.active()
    M3, CBRT = _cbrt_max()
    md = 1.0 / V
    t = {"T": T, "rcpT": 1.0 / T, "lnT": np.log(T)}
    t["T2"] = T * T
    Ck = [md * np.fmax(0.0, n[k]) for k in range(K - 1)]
    t["T3"] = T * t["T2"]
    C = P_R * t["rcpT"]
    t["rcpT2"] = t["rcpT"] * t["rcpT"]
    t["T4"] = t["T2"] * t["T2"]
    s = Ck[0]
    for k in range(1, K - 1):
        s = s + Ck[k]
    Ck.append(C - s)
    low = [T <= mech.nasa7_split[k] for k in range(K)]

    def gibbs(k):
        out = None
        for p in (0, 1):
            a = mech.nasa7[k, p]
            g = [a[0] - a[6], -a[0], -a[1] / 2.0, (1.0 / 3.0 - 1.0 / 2.0) * a[2], (1.0 / 4.0 - 1.0 / 3.0) * a[3],
                 (1.0 / 5.0 - 1.0 / 4.0) * a[4], a[5]]
            v = g[0] + g[1] * t["lnT"]
            v = v + g[2] * T
            v = v + g[3] * t["T2"]
            v = v + g[4] * t["T3"]
            v = v + g[5] * t["T4"]
            v = v + g[6] * t["rcpT"]
            out = v if out is None else np.where(low[k], out, v)
        return out

    ex, exn = {}, {}
    P0 = 101325.0 / R
    wdot = [None] * A
    for r in range(Rn):
        model = int(mech.model[r])
        A_, b_, Ea_ = mech.rate[r]
        if model in (2, 3, 4, 5):
            e = mech.efficiencies[r]
            terms = []
            for k in range(K):
                if e[k] == 1.0:
                    continue
                c = e[k] - 1.0
                cc = canon_mul(c)
                if c == 1.0 or cc == 1.0:
                    terms.append(Ck[k])
                elif _f32(c) != 0:
                    terms.append(cc * Ck[k])
            if terms:
                S = terms[0]
                for q in terms[1:]:
                    S = S + q
                M = C + S
            else:
                M = C
        if model in (0, 1):
            nn, d = arrhenius(A_, b_, Ea_, t), None
        elif model == 2:
            nn, d = arrhenius(A_, b_, Ea_, t) * M, None
        elif model == 4:
            A0, b0, Ea0 = mech.k0[r]
            k0 = arrhenius(A0 / A_, b0, Ea0, t)
            if b_ == 0 and Ea_ == 0:
                Pr = M * k0
                kinf = canon_mul(A_)
            else:
                ki = arrhenius(1.0, b_, Ea_, t)
                Pr = (M * k0) / (ki + F32MINPOS)
                kinf = canon_mul(A_) * ki
            At, T3, T1, T2 = mech.troe[r]
            F = None
            c1m = canon_mul(1.0 - At)
            if c1m != 0:
                F = c1m * np.exp(T * canon_mul(1.0 / (-T3)))
            if T1 < 1e30:
                ca = canon_mul(At)
                if ca != 0:
                    v = ca * np.exp(T * canon_mul(1.0 / (-T1)))
                    F = v if F is None else F + v
            elif canon_add(At) != 0:
                F = At if F is None else F + At
            if math.isfinite(T2):
                v = np.exp(canon_mul(-T2) * t["rcpT"])
                F = v if F is None else F + v
            lnF = np.log(F)
            Cc = -0.67 * lnF - 0.4 * math.log(10.0)
            Nn = -1.27 * lnF + 0.75 * math.log(10.0)
            lnPrC = np.log(Pr + F32MINPOS) + Cc
            f1 = lnPrC / (-0.14 * lnPrC + Nn)
            Fb = np.exp(lnF / (f1 * f1 + 1.0))
            nn, d = (Fb * kinf) * Pr, Pr + 1.0
        elif model == 3:
            A0, b0, Ea0 = mech.k0[r]
            Ck0 = M * arrhenius(A0, b0, Ea0, t)
            ki = arrhenius(A_, b_, Ea_, t)
            nn, d = Ck0 * ki, (Ck0 + ki) + F32MINPOS
        elif model == 5:  # SRI, the reference's commented formula (reaction.rs:194-203)
            A0, b0, Ea0 = mech.k0[r]
            k0 = arrhenius(A0, b0, Ea0, t)
            ki = arrhenius(A_, b_, Ea_, t)
            Pr = (M * k0) / (ki + F32MINPOS)
            lP = np.log(Pr + F32MINPOS)
            sa, sb, sc, sd, se = mech.sri[r]
            base = np.exp(canon_mul(-1.0 / sc) * T)
            if canon_mul(sa) != 0:
                base = canon_mul(sa) * np.exp(canon_mul(-sb) * t["rcpT"]) + base
            F = np.exp(np.log(base) * (1.0 / (1.0 + lP * lP)))
            if canon_mul(sd) != 1:
                F = canon_mul(sd) * F
            if canon_mul(se) != 0:
                F = F * np.exp(canon_mul(se) * t["lnT"])
            nn, d = (F * ki) * Pr, Pr + 1.0
        else:
            raise NotImplementedError(model)
        re, pr = mech.reactants[r], mech.products[r]

        def prod(st):
            p = None
            for k in range(K):
                for _ in range(int(st[k])):
                    p = Ck[k] if p is None else p * Ck[k]
            return p

        Rf = prod(re)
        if model == 1:
            Rnet = Rf
        else:
            p = None
            for k in range(A):
                nu = int(pr[k]) - int(re[k])
                if nu == 0:
                    continue
                if nu > 0:
                    if k not in ex:
                        ex[k] = np.fmin(M3, np.exp(gibbs(k)))
                    tt = ex[k]
                else:
                    if k not in exn:
                        exn[k] = np.fmin(CBRT, np.exp(-gibbs(k)))
                    tt = exn[k]
                for _ in range(abs(nu)):
                    p = tt if p is None else p * tt
            sn = int(pr.sum()) - int(re.sum())
            if -sn == 0:
                rK = p
            elif -sn == 1:
                rK = (P0 * t["rcpT"]) * p
            elif -sn == -1:
                rK = ((1.0 / P0) * T) * p
            else:
                rc = (1.0 / P0) * T
                rK = (rc * rc) * p
            Rnet = Rf - rK * prod(pr)
        cR = (Rnet * nn) / d if d is not None else Rnet * nn
        for k in range(A):
            nu = int(pr[k]) - int(re[k])
            if nu == 0:
                continue
            if nu == 1:
                wdot[k] = cR if wdot[k] is None else wdot[k] + cR
            elif nu == -1:
                wdot[k] = -cR if wdot[k] is None else wdot[k] - cR
            else:
                v = float(nu) * cR
                wdot[k] = v if wdot[k] is None else wdot[k] + v
    E = None
    for k in range(A):
        h = None
        for p in (0, 1):
            a = mech.nasa7[k, p]
            v = canon_add(a[0]) + canon_mul(a[1] / 2.0) * T
            v = v + canon_mul(a[2] / 3.0) * t["T2"]
            v = v + canon_mul(a[3] / 4.0) * t["T3"]
            v = v + canon_mul(a[4] / 5.0) * t["T4"]
            v = v + canon_mul(a[5]) * t["rcpT"]
            h = v if h is None else np.where(low[k], h, v)
        term = wdot[k] * h
        E = term if E is None else E + term
    Cp = None
    for k in range(K):
        cp = None
        for p in (0, 1):
            a = mech.nasa7[k, p]
            v = canon_add(a[0]) + canon_mul(a[1]) * T
            v = v + canon_mul(a[2]) * t["T2"]
            v = v + canon_mul(a[3]) * t["T3"]
            v = v + canon_mul(a[4]) * t["T4"]
            cp = v if cp is None else np.where(low[k], cp, v)
        term = cp * Ck[k]
        Cp = term if Cp is None else Cp + term
    dtT_T = -E / Cp
    dtE = None
    Wb = mech.molar_mass[K - 1]
    for k in range(A):
        c = canon_mul(1.0 - mech.molar_mass[k] / Wb)
        if c == 0:
            continue
        v = c * wdot[k]
        dtE = v if dtE is None else dtE + v
    dtV = V * (dtT_T + rcpP_R * T * dtE)
    return np.array([T * dtT_T, dtV] + wdot)


def transport(mech, scales, coefs, N, Tn, n):
    """transport.rs:141-210: returns [lambda/lambda0, mu/mu0, rhoD_k/mu0] as a (K+2, cells) array."""
    T0, mu0, l0 = scales
    cond, visc, diff = coefs
    K = mech.K
    W = mech.molar_mass
    sv, sc, sd = math.sqrt(math.sqrt(T0)) / math.sqrt(mu0), math.sqrt(T0) / (2.0 * l0), math.sqrt(T0) / (R * mu0)

    def scaled(P, s):
        return [canon_add(s * P[0])] + [canon_mul(s * p) for p in P[1:]]

    lnT = np.log(Tn)
    L = [None, lnT, lnT * lnT]
    L.append(L[2] * lnT)
    L.append(L[3] * lnT)

    def poly(P):
        v = P[0] + 0.0 * lnT
        for i in range(1, 5):
            if P[i] != 0:
                v = v + P[i] * L[i]
        return v

    X = [n[k] for k in range(K - 1)]
    s = X[0]
    for k in range(1, K - 1):
        s = s + X[k]
    X.append(N - s)
    VT = np.sqrt(Tn)
    MN = None
    for k in range(K):
        c = canon_mul(W[k])
        if c == 0:
            continue
        MN = c * X[k] if MN is None else MN + c * X[k]
    MVTN = MN * VT
    Acc = Bcc = None
    for k in range(K):
        c = poly(scaled(cond[k], sc))
        a, b = X[k] * c, X[k] / c
        Acc = a if Acc is None else Acc + a
        Bcc = b if Bcc is None else Bcc + b
    lam = (Acc / N + N / Bcc) * VT
    v = [poly(scaled(visc[k], sv)) for k in range(K)]
    rv = [1.0 / x for x in v]
    mu = None
    for k in range(K):
        den = None
        for j in range(K):
            Va = math.sqrt(1.0 / math.sqrt(8.0) * 1.0 / math.sqrt(1.0 + W[k] / W[j]))
            b = canon_mul(Va * math.sqrt(math.sqrt(W[j] / W[k])))
            va = canon_add(Va)
            q = (b * v[k]) * rv[j]
            tt = va + q if va != 0 else q
            term = X[j] * (tt * tt)
            den = term if den is None else den + term
        term = (X[k] * (v[k] * v[k])) / den
        mu = term if mu is None else mu + term
    S = [None] * K
    for k in range(K):
        for j in range(k):
            y = poly(scaled(diff[k * K + j], sd))
            Rkj = 1.0 / y
            S[k] = X[j] * Rkj if S[k] is None else S[k] + X[j] * Rkj
            S[j] = X[k] * Rkj if S[j] is None else S[j] + X[k] * Rkj
    out = [lam, VT * mu]
    for k in range(K):
        out.append((MVTN - (VT * canon_mul(W[k])) * X[k]) / S[k])
    return np.array(out)
