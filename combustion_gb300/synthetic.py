"""Seeded synthetic mechanisms and cell states.

The reference measures on real Cantera mechanisms (gri30 in ``perf.rs:12``) that are not
available here, so every workload is a seeded synthetic draw with the shapes named for the
benchmark configurations: K species (the last one an inert diluent, the implicit "bulk"
species of ``reaction.rs:372``), R reactions split into elementary reversible, three-body and
Troe falloff reactions, NASA-7 thermodynamics and Lennard-Jones transport data.

The generator produces the mechanism directly in the SI form that the reference's loader
produces (``yaml.rs:54-171`` followed by ``lib.rs:40-140``): pre-exponential factors are drawn
in cm-mol-s and converted with ``yaml.rs:101-103`` (``A * 1e-6**(order-1)``, three-body order
+1 at ``yaml.rs:100``, falloff low-pressure order +1 at ``yaml.rs:134``); activation energies
are drawn in kcal/mol and converted to an activation temperature with ``yaml.rs:104-114``;
transport data go from Angstrom/Kelvin/Debye to SI with ``lib.rs:40-59``.

All randomness comes from SplitMix64 counters so that a (seed, stream, index) triple always
yields the same draw, independent of draw order or vectorisation.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Physical constants of model.rs:6-8 and lib.rs (kB, NA, R = kB*NA).
kB = 1.380649e-23
NA = 6.02214076e23
R = kB * NA
LIGHT_SPEED = 299_792_458.0
CM_PER_DEBYE = 1e-21 / LIGHT_SPEED
J_PER_CAL = 4.184

# Reaction model codes (lib.rs:238-245).
ELEMENTARY, IRREVERSIBLE, THREE_BODY, LINDEMANN, TROE, SRI = 0, 1, 2, 3, 4, 5
# Species geometry codes (model.rs:15-19).
ATOM, LINEAR, NONLINEAR = 0, 1, 2

_M64 = (1 << 64) - 1
_GOLDEN = 0x9E3779B97F4A7C15


def _mix64(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(_GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, stream: int, index) -> np.ndarray:
    """U[0,1) doubles for counter ``index`` of ``stream`` under ``seed`` (SplitMix64)."""
    key = int(_mix64(np.uint64(seed & _M64)))
    base = (key + ((stream & 0xFFFFFF) << 40)) & _M64
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = _mix64(np.uint64(base) + idx * np.uint64(_GOLDEN))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


class _Stream:
    """Sequential scalar draws from one SplitMix64 stream."""

    def __init__(self, seed: int, stream: int):
        self.seed, self.stream, self.n = seed, stream, 0

    def u(self) -> float:
        v = float(uniform(self.seed, self.stream, self.n))
        self.n += 1
        return v

    def range(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.u()

    def log_range(self, lo: float, hi: float) -> float:
        return 10.0 ** (math.log10(lo) + (math.log10(hi) - math.log10(lo)) * self.u())

    def int(self, n: int) -> int:
        return min(int(self.u() * n), n - 1)


@dataclass
class Mechanism:
    """A mechanism in SI units, in the species order of the reference (active first, bulk last)."""

    names: list
    molar_mass: np.ndarray          # [K] kg/mol
    nasa7_split: np.ndarray         # [K] K (NaN: one piece)
    nasa7: np.ndarray               # [K,2,7] low piece (T <= split) then high piece
    geometry: np.ndarray            # [K] ATOM/LINEAR/NONLINEAR
    diameter: np.ndarray            # [K] m
    well_depth: np.ndarray          # [K] J
    polarizability: np.ndarray      # [K] m^3
    dipole: np.ndarray              # [K] C.m
    rotational_relaxation: np.ndarray  # [K]
    reactants: np.ndarray           # [R,K] uint8
    products: np.ndarray            # [R,K] uint8
    model: np.ndarray               # [R] int32
    rate: np.ndarray                # [R,3] A (SI), b, activation temperature (K)
    k0: np.ndarray                  # [R,3] low-pressure rate constant (falloff models)
    troe: np.ndarray                # [R,4] A, T3, T1, T2
    sri: np.ndarray                 # [R,5] A, B, C, D, E
    efficiencies: np.ndarray        # [R,K]
    meta: dict = field(default_factory=dict)

    @property
    def K(self) -> int:
        return len(self.molar_mass)

    @property
    def R(self) -> int:
        return len(self.model)

    @property
    def internal_degrees_of_freedom(self) -> np.ndarray:
        return np.array([0.0, 1.0, 1.5])[self.geometry]

    def active(self) -> int:
        """Number of active species: a prefix of species whose amount some reaction changes (lib.rs:127-140)."""
        changes = (self.reactants != self.products).any(axis=0)
        a = 0
        while a < self.K and changes[a]:
            a += 1
        if changes[a:].any():
            raise ValueError("active species do not form a prefix")
        return a

    def save(self, path: str) -> None:
        arrays = {k: getattr(self, k) for k in _ARRAYS}
        np.savez_compressed(path, names=np.array(self.names), **arrays,
                            meta=np.array([repr(self.meta)]))

    @staticmethod
    def load(path: str) -> "Mechanism":
        z = np.load(path, allow_pickle=False)
        kw = {k: z[k] for k in _ARRAYS}
        meta = eval(str(z["meta"][0]), {"__builtins__": {}}, {"nan": float("nan"), "inf": float("inf")})
        return Mechanism(names=[str(s) for s in z["names"]], meta=meta, **kw)


_ARRAYS = ["molar_mass", "nasa7_split", "nasa7", "geometry", "diameter", "well_depth", "polarizability",
           "dipole", "rotational_relaxation", "reactants", "products", "model", "rate", "k0", "troe", "sri",
           "efficiencies"]


# The five benchmark configurations: mechanism shapes and cell distributions.
CONFIGS = {
    "k10": dict(K=10, elementary=19, three_body=4, troe=2),
    "k53": dict(K=53, elementary=250, three_body=45, troe=30),
    "k250": dict(K=250, elementary=1200, three_body=180, troe=120),
}


def _fit_nasa7(c: float, theta: float, h298_R: float, s298_R: float):
    """Two-range NASA-7 fit of cp/R = 3.5 + c*(1 - exp(-T/theta)) on [200,1000] and [1000,3500] K."""
    pieces = np.zeros((2, 7))
    for i, (lo, hi) in enumerate(((200.0, 1000.0), (1000.0, 3500.0))):
        T = np.linspace(lo, hi, 64)
        cp = 3.5 + c * (1.0 - np.exp(-T / theta))
        scale = np.array([1.0, 1e3, 1e6, 1e9, 1e12])
        A = np.stack([T ** n for n in range(5)], axis=1) / scale
        coef, *_ = np.linalg.lstsq(A, cp, rcond=None)
        pieces[i, :5] = coef / scale

    def H(a, T):  # H/R
        return a[0] * T + a[1] * T**2 / 2 + a[2] * T**3 / 3 + a[3] * T**4 / 4 + a[4] * T**5 / 5 + a[5]

    def S(a, T):  # S/R
        return a[0] * math.log(T) + a[1] * T + a[2] * T**2 / 2 + a[3] * T**3 / 3 + a[4] * T**4 / 4 + a[6]

    lo, hi = pieces
    lo[5] = 0.0
    lo[5] = h298_R - H(lo, 298.15)
    lo[6] = 0.0
    lo[6] = s298_R - S(lo, 298.15)
    hi[5] = 0.0
    hi[5] = H(lo, 1000.0) - H(hi, 1000.0)
    hi[6] = 0.0
    hi[6] = S(lo, 1000.0) - S(hi, 1000.0)
    return pieces


def generate_mechanism(config: str = "k53", seed: int = 0) -> Mechanism:
    """Seeded synthetic mechanism of the named shape (species drawn first, then reactions)."""
    cfg = CONFIGS[config]
    K = cfg["K"]
    s = _Stream(seed, 1)
    names = [f"S{k}" for k in range(K - 1)] + ["DIL"]
    molar_mass = np.array([s.range(1.0, 100.0) for _ in range(K)]) * 1e-3
    nasa7 = np.zeros((K, 2, 7))
    for k in range(K):
        c, theta = s.range(0.0, 8.0), s.range(500.0, 2000.0)
        h298, s298 = s.range(-5e4, 5e4), s.range(20.0, 40.0)
        nasa7[k] = _fit_nasa7(c, theta, h298, s298)
    split = np.full(K, 1000.0)
    geometry = np.array([s.int(3) for _ in range(K)], dtype=np.int32)
    well_depth_K = np.array([s.range(30.0, 600.0) for _ in range(K)])
    diameter_A = np.array([s.range(2.5, 6.0) for _ in range(K)])
    polar_A3 = np.array([s.range(0.0, 3.0) for _ in range(K)])
    zrot = np.array([s.range(0.0, 4.0) for _ in range(K)])
    # lib.rs:40-59: atoms carry no polarizability or rotational relaxation; zero dipole throughout.
    polarizability = np.where(geometry == ATOM, 0.0, polar_A3 * 1e-30)
    rotational_relaxation = np.where(geometry == ATOM, 0.0, zrot)

    kinds = [ELEMENTARY] * cfg["elementary"] + [THREE_BODY] * cfg["three_body"] + [TROE] * cfg["troe"]
    Rn = len(kinds)
    order = sorted(range(Rn), key=lambda i: s.u())  # seeded shuffle of the reaction kinds
    kinds = [kinds[i] for i in order]
    reactants = np.zeros((Rn, K), dtype=np.uint8)
    products = np.zeros((Rn, K), dtype=np.uint8)
    rate = np.zeros((Rn, 3))
    k0 = np.zeros((Rn, 3))
    troe = np.zeros((Rn, 4))
    sri = np.zeros((Rn, 5))
    efficiencies = np.ones((Rn, K))
    model = np.array(kinds, dtype=np.int32)
    ea_K_per_kcal = 1000.0 * J_PER_CAL / R  # yaml.rs:104-114
    for r in range(Rn):
        while True:
            lhs = np.zeros(K, dtype=np.uint8)
            rhs = np.zeros(K, dtype=np.uint8)
            nr, npd = 1 + s.int(2), 1 + s.int(2)
            forced = r if r < K - 1 else None  # every non-diluent species changes in some reaction
            for i in range(nr):
                lhs[forced if (i == 0 and forced is not None) else s.int(K - 1)] += 1
            for _ in range(npd):
                rhs[s.int(K - 1)] += 1
            net = rhs.astype(int) - lhs.astype(int)
            if forced is not None and net[forced] == 0:
                continue
            if (net != 0).any():
                break
        reactants[r], products[r] = lhs, rhs
        n_react = int(lhs.sum())
        A_cgs = s.log_range(1e6, 1e16)
        b = s.range(-2.0, 3.0)
        Ea = s.range(0.0, 50.0) * ea_K_per_kcal
        kind = kinds[r]
        order_ = n_react + (1 if kind == THREE_BODY else 0)
        rate[r] = (A_cgs * 1e-6 ** (order_ - 1), b, Ea)
        if kind in (THREE_BODY, TROE):
            efficiencies[r] = [s.range(0.5, 12.0) for _ in range(K)]
        if kind == TROE:
            A0_cgs = A_cgs * s.log_range(1e3, 1e5)
            b0 = s.range(-2.0, 3.0)
            Ea0 = s.range(0.0, 50.0) * ea_K_per_kcal
            k0[r] = (A0_cgs * 1e-6 ** n_react, b0, Ea0)
            troe[r] = (s.range(0.3, 0.9), s.range(50.0, 500.0), s.range(500.0, 3000.0), math.inf)
    mech = Mechanism(names=names, molar_mass=molar_mass, nasa7_split=split, nasa7=nasa7, geometry=geometry,
                     diameter=diameter_A * 1e-10, well_depth=well_depth_K * kB, polarizability=polarizability,
                     dipole=np.zeros(K), rotational_relaxation=rotational_relaxation, reactants=reactants,
                     products=products, model=model, rate=rate, k0=k0, troe=troe, sri=sri,
                     efficiencies=efficiencies, meta={"config": config, "seed": seed})
    assert mech.active() == K - 1
    return mech


def generate_reactor_mechanism(config: str = "k53", seed: int = 0) -> Mechanism:
    """A well-posed variant of the named mechanism shape for constant-pressure reactors.

    The rates workload's kinetics (A up to 1e16 cm-mol-s with b up to 3, enthalpies of formation spread
    over +-5e4 K so that equilibrium constants reach e^+-70, random molar masses without element balance)
    drive a constant-pressure reactor (plot.rs:32-118 formulation) to runaway within picoseconds: reverse
    rates of 1e20 mol/m^3/s, volumes growing or collapsing without bound; no integrator, the reference's
    included, reaches 1 ms. This variant keeps the species (heat capacities, entropies, transport), the
    reaction counts per model and the reacting species of every reaction, and changes:
      - products are added or removed so that each reaction conserves moles;
      - every species gets the bulk species' molar mass (the volume then follows n R T / P);
      - enthalpies of formation are scaled by 0.1, and species 0 (fuel) and 1 (oxidiser) get 1.5e4 K
        (h/R) more, so that consuming them releases heat;
      - A log-uniform on [1e11, 1e13] cm-mol-s, b = 0, activation energy U[30, 45] kcal/mol plus the
        reaction enthalpy when that is positive (both directions keep a barrier; falloff k0: A times
        log-uniform [1e3, 1e5]).
    Heat release then accelerates the reactions: an induction time, then ignition.
    """
    m = generate_mechanism(config, seed)
    K, Rn = m.K, m.R
    s = _Stream(seed, 2)
    m.molar_mass = np.full(K, m.molar_mass[K - 1])

    def H_R(k, T):  # h/R of species k at T
        a = m.nasa7[k, 0 if T <= m.nasa7_split[k] else 1]
        return a[0] * T + a[1] * T**2 / 2 + a[2] * T**3 / 3 + a[3] * T**4 / 4 + a[4] * T**5 / 5 + a[5]

    for k in range(K):
        h298 = H_R(k, 298.15)
        target = 0.1 * h298 + (1.5e4 if k in (0, 1) else 0.0)
        m.nasa7[k, :, 5] += target - h298
    ea_K_per_kcal = 1000.0 * J_PER_CAL / R
    for r in range(Rn):
        lhs, rhs = m.reactants[r].astype(int), m.products[r].astype(int)
        forced = r if r < K - 1 else None
        while rhs.sum() < lhs.sum():
            k = s.int(K - 1)
            if k != forced:
                rhs[k] += 1
        while rhs.sum() > lhs.sum():
            nz = [k for k in range(K) if rhs[k] > 0]
            rhs[nz[s.int(len(nz))]] -= 1
        if (rhs == lhs).all() or (forced is not None and rhs[forced] == lhs[forced]):
            # keep the reaction changing its forced species: swap one product for another species
            nz = [k for k in range(K) if rhs[k] > 0]
            rhs[nz[0]] -= 1
            k = s.int(K - 1)
            while k == forced or k == nz[0]:
                k = s.int(K - 1)
            rhs[k] += 1
        m.reactants[r], m.products[r] = lhs.astype(np.uint8), rhs.astype(np.uint8)
        dH = sum(rhs[k] * H_R(k, 1200.0) for k in range(K)) - sum(lhs[k] * H_R(k, 1200.0) for k in range(K))
        n_react = int(lhs.sum())
        A_cgs = s.log_range(1e11, 1e13)
        Ea = s.range(30.0, 45.0) * ea_K_per_kcal + max(0.0, dH)
        order_ = n_react + (1 if m.model[r] == THREE_BODY else 0)
        m.rate[r] = (A_cgs * 1e-6 ** (order_ - 1), 0.0, Ea)
        if m.model[r] == TROE:
            A0_cgs = A_cgs * s.log_range(1e3, 1e5)
            m.k0[r] = (A0_cgs * 1e-6 ** n_react, 0.0, Ea)
    m.meta = {"config": config, "seed": seed, "variant": "reactor"}
    assert m.active() == K - 1
    return m


def transport_scales(mech: Mechanism, T0: float = 1000.0, equivalence_ratio: float = 1.0):
    """(T0, viscosity0, conductivity0) of cantera.rs:60-76: fuel = species 0, oxidiser = species 1,
    diluent = last species, 1 atm, unit diffusivity."""
    K = mech.K
    amounts = np.zeros(K)
    amounts[0] = 1.0
    amounts[1] = 1.0 / (2.0 * equivalence_ratio)
    amounts[K - 1] = 1.0 / (2.0 * equivalence_ratio) * 79.0 / 21.0
    total = sum(amounts)
    X = [a / total for a in amounts]
    pressure_R = 101325.0 / R
    concentration = pressure_R / T0
    mean_molar_mass = sum(m * x for m, x in zip(mech.molar_mass, X))
    density = concentration * mean_molar_mass
    viscosity = density * 1.0
    cp = 0.0
    for k in range(K):
        a = mech.nasa7[k, 0 if T0 <= mech.nasa7_split[k] else 1]
        cpk = a[0] + a[1] * T0 + a[2] * T0 * T0 + a[3] * T0 * T0 * T0 + a[4] * T0 * T0 * T0 * T0
        cp += cpk * X[k]
    conductivity = cp * R / mean_molar_mass * viscosity
    return T0, viscosity, conductivity


@dataclass
class Cells:
    """Struct-of-arrays cell states in the reference's input order (reaction.rs:358, transport.rs:185)."""

    pressure_R: np.ndarray   # [N] P/R
    temperature: np.ndarray  # [N] K
    volume: np.ndarray       # [N] m^3
    amounts: np.ndarray      # [K-1, N] mol (non-bulk species)
    total_amount: np.ndarray  # [N] mol (all species, bulk included)

    @property
    def n(self) -> int:
        return len(self.temperature)


def _normal(seed, stream, idx):
    u1 = uniform(seed, stream, 2 * idx)
    u2 = uniform(seed, stream, 2 * idx + 1)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


def _gamma(alpha: float, seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    """Marsaglia-Tsang Gamma(alpha) draws, boosted by U**(1/alpha) for alpha < 1."""
    a = alpha + 1.0 if alpha < 1.0 else alpha
    d = a - 1.0 / 3.0
    c = 1.0 / math.sqrt(9.0 * d)
    out = np.zeros(idx.shape)
    todo = np.ones(idx.shape, dtype=bool)
    for rnd in range(64):
        sub = idx[todo] * np.uint64(64) + np.uint64(rnd)
        x = _normal(seed, stream, sub)
        u = uniform(seed, stream + 1, sub)
        v = (1.0 + c * x) ** 3
        ok = (v > 0) & (np.log(np.maximum(u, 1e-300)) < 0.5 * x * x + d - d * v + d * np.log(np.where(v > 0, v, 1.0)))
        vals = out[todo]
        vals[ok] = d * v[ok]
        out[todo] = vals
        t = np.flatnonzero(todo)
        todo[t[ok]] = False
        if not todo.any():
            break
    if alpha < 1.0:
        out *= uniform(seed, stream + 2, idx) ** (1.0 / alpha)
    return out


CELL_CONFIGS = {
    # (T range K, pressure: fixed Pa or (lo, hi) atm log-uniform, Dirichlet alpha)
    "k10": dict(T=(800.0, 2800.0), P=101325.0, alpha=0.5),
    "k53": dict(T=(300.0, 3000.0), P=(0.1, 40.0), alpha=0.3),
    "k250": dict(T=(300.0, 3000.0), P=(0.1, 40.0), alpha=0.3),
}


def generate_cells(K: int, n: int, config: str = "k53", seed: int = 1, offset: int = 0) -> Cells:
    """Seeded cells: T uniform, P fixed or log-uniform, mole fractions Dirichlet(alpha) over all K species,
    V = 1 m^3, n_k = X_k * P V / (R T). ``offset`` selects a window of the same infinite cell sequence."""
    cfg = CELL_CONFIGS[config]
    idx = np.arange(offset, offset + n, dtype=np.uint64)
    T = cfg["T"][0] + (cfg["T"][1] - cfg["T"][0]) * uniform(seed, 1, idx)
    if isinstance(cfg["P"], tuple):
        lo, hi = math.log(cfg["P"][0]), math.log(cfg["P"][1])
        P = 101325.0 * np.exp(lo + (hi - lo) * uniform(seed, 2, idx))
    else:
        P = np.full(n, cfg["P"])
    pressure_R = P / R
    V = np.ones(n)
    g = np.empty((K, n))
    for k in range(K):
        g[k] = _gamma(cfg["alpha"], seed, 16 + 4 * k, idx)
    g = np.maximum(g, 1e-300)
    X = g / g.sum(axis=0)
    total = pressure_R * V / T
    amounts = X[:K - 1] * total
    return Cells(pressure_R=pressure_R, temperature=T, volume=V, amounts=np.ascontiguousarray(amounts),
                 total_amount=total)


def _cells_window(args):
    K, n, config, seed, offset = args
    c = generate_cells(K, n, config, seed, offset)
    return c.pressure_R, c.temperature, c.volume, c.amounts, c.total_amount


def generate_cells_parallel(K: int, n: int, config: str = "k53", seed: int = 1, workers: int = 0,
                            out_amounts: np.ndarray = None) -> Cells:
    """generate_cells over ``workers`` spawned processes (identical result: draws are counter-based).
    ``out_amounts`` ([K-1, n] float64, e.g. pinned host memory) receives the amounts in place."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os as _os
    workers = workers or min(16, _os.cpu_count() or 1)
    if n < 65536 or workers == 1:
        c = generate_cells(K, n, config, seed)
        if out_amounts is not None:
            out_amounts[:] = c.amounts
            c.amounts = out_amounts
        return c
    bounds = [n * w // workers for w in range(workers + 1)]
    jobs = [(K, bounds[w + 1] - bounds[w], config, seed, bounds[w]) for w in range(workers)]
    P, T, V, N = (np.empty(n) for _ in range(4))
    amounts = out_amounts if out_amounts is not None else np.empty((K - 1, n))
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        for (lo, hi), (p, t, v, a, tot) in zip(zip(bounds[:-1], bounds[1:]), ex.map(_cells_window, jobs)):
            P[lo:hi], T[lo:hi], V[lo:hi], amounts[:, lo:hi], N[lo:hi] = p, t, v, a, tot
    return Cells(pressure_R=P, temperature=T, volume=V, amounts=amounts, total_amount=N)
