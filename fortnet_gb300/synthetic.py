"""Seeded synthetic datasets of the benchmark configurations.

The reference publishes no benchmark dataset, so every workload is generated here: random
dense-liquid (or jittered FCC) periodic structures, cubic cells, coordinates in Bohr, and
Morse pair-potential total energies as global targets (summed over every periodic image
pair within 6 Angstrom, in Hartree).

* C1 — 64 x 32-atom jittered FCC aluminium, 8 G2 at 4.0 A, network 8-10-10-1 (FP64)
* C2 — 2,000 structures of 64-256 atoms, species O:Si = 1:2, 24 G2 + 16 G5 base functions
       at 6.0 A (96 features after species expansion), network 96-32-32-1
* C3 — 20,000 structures of 8-2,048 atoms (log-uniform), H/C/O, same base functions
       (168 features), network 168-64-64-1, mini-batches of 256 structures
* C4 — 5,000 structures of 100-500 atoms, H/C/O, nR = 10, nA = 6 at 6.5 A (66 features),
       network 66-64-64-1, energies and forces
* C5 — request stream: Poisson arrivals at 2,000 req/s, 16-4,096 atoms (log-uniform), the
       C4 model; a pool of distinct structures that the stream cycles through
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np

from .fnetdata import Dataset
from .gfunctions import AA__BOHR, GFunction, process_acsf_functions

DENSITY = 0.066          # atoms / A^3
MIN_SEP = 1.6            # A
EV__HARTREE = 1.0 / 27.2113845
MORSE_CUT = 6.0          # A

# (D eV, a 1/A, r0 A) per species pair, species in order A, B, C
MORSE = {
    (0, 0): (0.30, 1.2, 2.86), (0, 1): (0.25, 1.1, 2.5), (0, 2): (0.20, 1.0, 2.2),
    (1, 1): (0.35, 1.3, 3.0), (1, 2): (0.40, 1.4, 2.7), (2, 2): (0.28, 1.15, 2.4),
}


def morse_params(si, sj):
    return MORSE[(min(si, sj), max(si, sj))]


@dataclass
class Config:
    name: str
    nstruct: int
    natoms: tuple          # (lo, hi)
    dist: str              # 'uniform' | 'loguniform' | 'fixed'
    atomic_numbers: tuple
    ratios: tuple
    rcut: float            # A
    n_g2: int
    g2_eta: tuple          # A^-2 range, log-spaced
    g5: dict | None        # {'zeta': (..), 'lambda': (..), 'eta': (lo, hi, n)}
    hidden: tuple
    seed: int
    fcc: bool = False


CONFIGS = {
    "C1": Config("C1", 64, (32, 32), "fixed", (13,), (1.0,), 4.0, 8, (0.01, 2.0), None,
                 (10, 10), 1001, fcc=True),
    "C2": Config("C2", 2000, (64, 256), "uniform", (8, 14), (1.0, 2.0), 6.0, 24, (0.01, 2.0),
                 {"zeta": (1.0, 4.0), "lambda": (1.0, -1.0), "eta": (0.005, 0.05, 4)},
                 (32, 32), 1002),
    "C3": Config("C3", 20000, (8, 2048), "loguniform", (1, 6, 8), (1.0, 1.0, 1.0), 6.0, 24,
                 (0.01, 2.0), {"zeta": (1.0, 4.0), "lambda": (1.0, -1.0), "eta": (0.005, 0.05, 4)},
                 (64, 64), 1003),
    "C4": Config("C4", 5000, (100, 500), "uniform", (1, 6, 8), (1.0, 1.0, 1.0), 6.5, 10,
                 (0.01, 2.0), {"zeta": (1.0, 2.0, 4.0), "lambda": (1.0, -1.0),
                               "eta": (0.005, 0.005, 1)},
                 (64, 64), 1004),
    # request pool of the serving stream: the C4 model and functions, 16-4,096 atoms
    "C5": Config("C5", 64, (16, 4096), "loguniform", (1, 6, 8), (1.0, 1.0, 1.0), 6.5, 10,
                 (0.01, 2.0), {"zeta": (1.0, 2.0, 4.0), "lambda": (1.0, -1.0),
                               "eta": (0.005, 0.005, 1)},
                 (64, 64), 1005),
}

C5_RATE = 2000.0  # requests / s (Poisson arrivals)


def arrivals(n, rate=C5_RATE, seed=1005):
    """Arrival times (s) of a Poisson stream of n requests at the given rate."""
    rng = np.random.default_rng(seed + 7)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def base_functions(cfg: Config):
    """Base G-functions (before species expansion), parameters converted to Bohr."""
    rc = cfg.rcut * AA__BOHR
    b2 = (1.0 / AA__BOHR) ** 2  # A^-2 -> Bohr^-2
    funcs = [GFunction("g2", rc, rs=0.0, eta=float(e) * b2)
             for e in np.geomspace(cfg.g2_eta[0], cfg.g2_eta[1], cfg.n_g2)]
    if cfg.g5:
        lo, hi, n = cfg.g5["eta"]
        for z in cfg.g5["zeta"]:
            for lam in cfg.g5["lambda"]:
                for e in np.geomspace(lo, hi, n):
                    funcs.append(GFunction("g5", rc, xi=float(z), lam=float(lam), eta=float(e) * b2))
    return funcs


def gfunctions(cfg: Config):
    return process_acsf_functions(base_functions(cfg), cfg.atomic_numbers)


def network_dims(cfg: Config):
    return [len(gfunctions(cfg))] + list(cfg.hidden) + [1]


def param_layout(dims):
    """Offsets of the reference's parameter order (network.F90:397-427): every layer's weight
    matrix column-major (the output layer's ww(d_L, 1) included), then every layer's biases."""
    woff, boff, ind = [], [], 0
    for l in range(len(dims)):
        woff.append(ind)
        ind += dims[l] * (dims[l + 1] if l < len(dims) - 1 else 1)
    for l in range(len(dims)):
        boff.append(ind)
        ind += dims[l]
    return woff, boff, ind


def normal_params(dims, nspecies, seed):
    """Well-conditioned synthetic networks in the reference order: weights N(0, 1/fan_in),
    biases N(0, 0.1^2), the unused entries (ww(d_L, 1), input-layer biases) zero.  Unlike the
    reference's normalXavier draw (all weights positive Gaussian pdf values), these keep the
    tanh units of z-scored inputs out of saturation."""
    rng = np.random.default_rng(seed)
    woff, boff, n = param_layout(dims)
    p = np.zeros((nspecies, n))
    for s in range(nspecies):
        for l in range(len(dims) - 1):
            k = dims[l] * dims[l + 1]
            p[s, woff[l]:woff[l] + k] = rng.normal(0, 1 / np.sqrt(dims[l]), size=k)
            p[s, boff[l + 1]:boff[l + 1] + dims[l + 1]] = rng.normal(0, 0.1, size=dims[l + 1])
    return p


def _natoms(cfg, rng, n):
    lo, hi = cfg.natoms
    if cfg.dist == "fixed":
        return np.full(n, lo, dtype=np.int64)
    if cfg.dist == "uniform":
        return rng.integers(lo, hi + 1, size=n)
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size=n))).astype(np.int64)


def _rsa_box(n, L, rng, min_sep=MIN_SEP):
    """Random sequential addition in a cubic box with minimum-image separation >= min_sep
    (candidates proposed in batches and screened with periodic k-d trees)."""
    from scipy.spatial import cKDTree

    pos = np.empty((0, 3))
    rounds = 0
    while len(pos) < n:
        rounds += 1
        if rounds > 10000:
            raise RuntimeError("random sequential addition did not converge")
        need = n - len(pos)
        cand = rng.uniform(0.0, L, size=(max(8, int(need * 1.3) + 4), 3))
        if len(pos):
            tree = cKDTree(pos, boxsize=L)
            d, _ = tree.query(cand, k=1)
            cand = cand[d >= min_sep]
        if len(cand) == 0:
            continue
        # resolve conflicts inside the batch: keep the earlier candidate of every close pair
        ct = cKDTree(cand, boxsize=L)
        drop = np.zeros(len(cand), dtype=bool)
        for a, b in sorted(ct.query_pairs(min_sep)):
            if not drop[a]:
                drop[b] = True
        cand = cand[~drop][:need]
        pos = np.concatenate([pos, cand])
    return pos


def _fcc(rng, jitter=0.05, a=4.05, reps=2):
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([[i, j, k] for i in range(reps) for j in range(reps) for k in range(reps)])
    frac = (cells[:, None, :] + base[None, :, :]).reshape(-1, 3) / reps
    L = a * reps
    return frac * L + rng.normal(0.0, jitter, size=frac.shape), L


def _morse_pairs(pos_A, species, L, cut):
    """Every (atom, periodic image of an atom) pair within cut (A): centre index, neighbour
    index, displacement centre - neighbour image (A), distance, Morse (D, a, r0)."""
    from scipy.spatial import cKDTree

    n = len(pos_A)
    k = int(math.ceil(cut / L))
    rng_k = np.arange(-k, k + 1)
    shifts = np.stack(np.meshgrid(rng_k, rng_k, rng_k, indexing="ij"), -1).reshape(-1, 3) * L
    ghosts = (pos_A[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    gidx = np.tile(np.arange(n), len(shifts))
    tree = cKDTree(ghosts)
    pairs = tree.query_ball_point(pos_A, r=cut)
    ii = np.repeat(np.arange(n), [len(p) for p in pairs])
    gg = np.concatenate([np.asarray(p, dtype=np.int64) for p in pairs]) if n else np.zeros(0, int)
    jj = gidx[gg]
    d = pos_A[ii] - ghosts[gg]
    r = np.sqrt(np.einsum("ij,ij->i", d, d))
    keep = r > 1e-12  # drop the atom itself
    ii, jj, d, r = ii[keep], jj[keep], d[keep], r[keep]
    si, sj = species[ii], species[jj]
    lo, hi = np.minimum(si, sj), np.maximum(si, sj)
    D = np.zeros(len(r))
    A = np.zeros(len(r))
    R0 = np.zeros(len(r))
    for (a, b), (dv, av, rv) in MORSE.items():
        m = (lo == a) & (hi == b)
        D[m], A[m], R0[m] = dv, av, rv
    return ii, jj, d, r, D, A, R0


def morse_forces(pos_A, species, L, cut=MORSE_CUT):
    """Forces -dE/dr of morse_energy on every atom, Hartree / Bohr [n, 3]."""
    ii, jj, d, r, D, A, R0 = _morse_pairs(pos_A, species, L, cut)
    x = np.exp(-A * (r - R0))
    dedr = 2.0 * A * D * x * (1.0 - x)  # d/dr of D (x^2 - 2x), eV / A
    F = np.zeros_like(pos_A)
    np.add.at(F, ii, -(dedr / r)[:, None] * d)
    return F * EV__HARTREE / AA__BOHR


def morse_energy(pos_A, species, L, cut=MORSE_CUT):
    """Total Morse energy (Hartree) over unique pairs of all periodic images, r <= cut (A)."""
    from scipy.spatial import cKDTree

    n = len(pos_A)
    k = int(math.ceil(cut / L))
    rng_k = np.arange(-k, k + 1)
    shifts = np.stack(np.meshgrid(rng_k, rng_k, rng_k, indexing="ij"), -1).reshape(-1, 3) * L
    ghosts = (pos_A[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    gidx = np.tile(np.arange(n), len(shifts))
    tree = cKDTree(ghosts)
    pairs = tree.query_ball_point(pos_A, r=cut)
    ii = np.repeat(np.arange(n), [len(p) for p in pairs])
    gg = np.concatenate([np.asarray(p, dtype=np.int64) for p in pairs]) if n else np.zeros(0, int)
    jj = gidx[gg]
    d = ghosts[gg] - pos_A[ii]
    r = np.sqrt(np.einsum("ij,ij->i", d, d))
    keep = r > 1e-12  # drop the atom itself
    ii, jj, r = ii[keep], jj[keep], r[keep]
    si, sj = species[ii], species[jj]
    lo, hi = np.minimum(si, sj), np.maximum(si, sj)
    D = np.zeros(len(r))
    A = np.zeros(len(r))
    R0 = np.zeros(len(r))
    for (a, b), (dv, av, rv) in MORSE.items():
        m = (lo == a) & (hi == b)
        D[m], A[m], R0[m] = dv, av, rv
    x = np.exp(-A * (r - R0))
    return 0.5 * float(np.sum(D * (x * x - 2.0 * x))) * EV__HARTREE


def _structure(cfg: Config, seed: int, s: int, n: int, targets: bool, forces: bool = False):
    """Structure s of a configuration: its own random stream (seeded by (seed, s)), so that
    structures can be generated in any order and in parallel."""
    rng = np.random.default_rng([seed, s])
    nsp = len(cfg.atomic_numbers)
    ratios = np.asarray(cfg.ratios, dtype=np.float64) / np.sum(cfg.ratios)
    if cfg.fcc:
        pos, L = _fcc(rng)
        n = len(pos)
    else:
        L = (n / DENSITY) ** (1.0 / 3.0)
        pos = _rsa_box(n, L, rng)
    counts = np.floor(ratios * n).astype(int)
    counts[-1] = n - counts[:-1].sum()
    sp = np.repeat(np.arange(nsp), counts)
    rng.shuffle(sp)
    e = morse_energy(pos, sp, L) if targets else 0.0
    f = morse_forces(pos, sp, L) if forces else None
    return pos * AA__BOHR, sp.astype(np.int32), L * AA__BOHR, e, f


def _structure_job(job):
    return _structure(*job)


def generate(cfg: Config | str, nstruct=None, seed=None, targets=True, workers=None,
             forces=False) -> Dataset:
    """Generate (the first nstruct structures of) a configuration's dataset.  Large requests are
    spread over a process pool (spawned, so it is safe after CUDA initialisation); the result
    does not depend on the number of workers.  forces=True adds the Morse forces (Hartree /
    Bohr) as meta["forces"] [Ntot, 3]."""
    if isinstance(cfg, str):
        cfg = CONFIGS[cfg]
    seed = cfg.seed if seed is None else seed
    rng = np.random.default_rng(seed)
    S = cfg.nstruct if nstruct is None else nstruct
    nat = _natoms(cfg, rng, cfg.nstruct)[:S]
    jobs = [(cfg, seed, s, int(nat[s]), targets, forces) for s in range(S)]
    if workers is None:
        workers = min(os.cpu_count() or 1, 32) if S >= 1000 else 1
    if workers > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(workers) as pool:
            res = pool.map(_structure_job, jobs, chunksize=max(1, S // (8 * workers)))
    else:
        res = [_structure_job(j) for j in jobs]
    coords = [r[0] for r in res]
    species = [r[1] for r in res]
    atnum = [np.asarray(cfg.atomic_numbers, dtype=np.int32)[r[1]] for r in res]
    lat = [np.array([r[2], 0, 0, 0, r[2], 0, 0, 0, r[2]], dtype=np.float64) for r in res]
    gt = [[r[3]] for r in res]
    off = np.zeros(S + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(c) for c in coords])
    ntot = int(off[-1])
    return Dataset(
        atom_offsets=off,
        coords=np.ascontiguousarray(np.concatenate(coords)),
        atnum=np.concatenate(atnum),
        species=np.concatenate(species),
        periodic=np.ones(S, dtype=np.int32),
        latvecs=np.asarray(lat),
        atomic_numbers=np.asarray(cfg.atomic_numbers, dtype=np.int32),
        weights=np.ones(S, dtype=np.int32),
        atomic_weights=np.ones(ntot),
        global_targets=np.asarray(gt, dtype=np.float64).reshape(S, 1),
        atomic_targets=np.zeros((ntot, 0)),
        meta={"config": cfg.name,
              **({"forces": np.concatenate([r[4] for r in res])} if forces else {})},
    )
