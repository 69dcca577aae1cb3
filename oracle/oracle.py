"""ORACLE — test infrastructure only.

ctypes front end of ``liboracle.so`` (the FP64 CPU restatement of Fortnet's hot path in
``fnet_oracle.c``).  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs
of ``bench.py`` import this module; the product never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

ACT = {"tanh": 0, "sigmoid": 1, "relu": 2, "lrelu": 3, "softplus": 4, "bent": 5, "atan": 6,
       "gaussian": 7, "heaviside": 8, "linear": 9}
LOSS = {"mse": 0, "rms": 1, "mae": 2, "mape": 3}


def build():
    """Compile the oracle with the committed Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


class _GFunc(C.Structure):
    _fields_ = [("type", C.c_int32), ("atomid", C.c_int32), ("z1", C.c_int32),
                ("z2", C.c_int32), ("rcut", C.c_double), ("kappa", C.c_double),
                ("rs", C.c_double), ("eta", C.c_double), ("lam", C.c_double),
                ("xi", C.c_double)]


class _Batch(C.Structure):
    _fields_ = [("nstruct", C.c_int32), ("atom_offsets", C.c_void_p), ("coords", C.c_void_p),
                ("atnum", C.c_void_p), ("periodic", C.c_void_p), ("latvecs", C.c_void_p),
                ("ext", C.c_void_p), ("next", C.c_int32)]


class _Net(C.Structure):
    _fields_ = [("nlayer", C.c_int32), ("dims", C.c_void_p), ("activation", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        L.orc_ranlux_new.restype = vp
        L.orc_ranlux_new.argtypes = [i32, i32]
        L.orc_ranlux_get.argtypes = [vp, vp, i64]
        L.orc_ranlux_free.argtypes = [vp]
        L.orc_init_bpnn_params.argtypes = [vp, vp, i32, vp]
        L.orc_knuth_shuffle.argtypes = [vp, vp, i32]
        L.orc_recvecs2p.argtypes = [vp, vp]
        L.orc_neighbours.argtypes = [vp, dbl, vp, vp, vp, vp, vp, i32]
        L.orc_acsf.argtypes = [vp, vp, i32, i32, vp, i32]
        L.orc_acsf_prime.argtypes = [vp, i32, vp, i32, vp]
        L.orc_zscore_stats.argtypes = [vp, i64, i32, vp, i32, vp, vp]
        L.orc_zscore_apply.argtypes = [vp, i64, i32, vp]
        L.orc_nparams.restype = i64
        L.orc_nparams.argtypes = [vp]
        L.orc_predict.argtypes = [vp, vp, i32, vp, i64, vp, vp]
        L.orc_jacobian.argtypes = [vp, vp, i32, vp, i64, vp, vp]
        L.orc_train_gradients.argtypes = [vp, vp, i32, i32, vp, vp, i32, vp, i32, i32, vp, vp,
                                          vp, vp, vp, i32, vp, vp]
        L.orc_update_prepare.restype = dbl
        L.orc_update_prepare.argtypes = [vp, vp, i32, vp, dbl, dbl, dbl]
        L.orc_forces.argtypes = [vp, vp, i32, vp, i32, vp, vp]
        L.orc_forces_ex.argtypes = [vp, vp, i32, vp, i32, vp, i32, vp]
        L.orc_forces_mt.argtypes = [vp, vp, i32, vp, i32, vp, i32, vp, i32]
        L.orc_sd_new.restype = vp
        L.orc_sd_new.argtypes = [i32, dbl, dbl, dbl, vp]
        L.orc_sd_next.argtypes = [vp, vp, vp]
        L.orc_lbfgs_new.restype = vp
        L.orc_lbfgs_new.argtypes = [i32, dbl, dbl, dbl, i32, i32, i32, vp]
        L.orc_lbfgs_next.argtypes = [vp, dbl, vp, vp]
        L.orc_cg_new.restype = vp
        L.orc_cg_new.argtypes = [i32, dbl, dbl, vp]
        L.orc_cg_next.argtypes = [vp, dbl, vp, vp]
        L.orc_fire_new.restype = vp
        L.orc_fire_new.argtypes = [i32, dbl, dbl, vp]
        L.orc_fire_next.argtypes = [vp, vp, vp]
        L.orc_opt_free.argtypes = [vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class Batch:
    """Keeps the numpy arrays alive while the C struct points into them."""

    def __init__(self, ds):
        self.off = np.ascontiguousarray(ds.atom_offsets, dtype=np.int64)
        self.coords = np.ascontiguousarray(ds.coords, dtype=np.float64)
        self.atnum = np.ascontiguousarray(ds.atnum, dtype=np.int32)
        self.periodic = np.ascontiguousarray(ds.periodic, dtype=np.int32)
        self.latvecs = np.ascontiguousarray(ds.latvecs, dtype=np.float64)
        self.ext = None if ds.ext is None else np.ascontiguousarray(ds.ext, dtype=np.float64)
        self.s = _Batch(len(self.off) - 1, _p(self.off), _p(self.coords), _p(self.atnum),
                        _p(self.periodic), _p(self.latvecs), _p(self.ext),
                        0 if self.ext is None else self.ext.shape[1])

    @property
    def ref(self):
        return C.byref(self.s)


def _gfuncs(funcs):
    arr = (_GFunc * max(len(funcs), 1))()
    codes = {"g1": 1, "g2": 2, "g3": 3, "g4": 4, "g5": 5}
    for i, f in enumerate(funcs):
        arr[i] = _GFunc(codes[f.type], f.atomid, f.z1, f.z2, f.rcut, f.kappa, f.rs, f.eta,
                        f.lam, f.xi)
    return arr


class Net:
    def __init__(self, dims, activation):
        self.dims = np.ascontiguousarray(dims, dtype=np.int32)
        act = ACT[activation] if isinstance(activation, str) else int(activation)
        self.s = _Net(len(self.dims), _p(self.dims), act)

    @property
    def ref(self):
        return C.byref(self.s)

    @property
    def nparams(self):
        return int(lib().orc_nparams(self.ref))


# ------------------------------------------------------------------ ACSF
def neighbours(ds, rcut, nthreads=1):
    """Full neighbour lists in the reference iterator's order.
    Returns (offsets[Ntot+1], j[P], shift[P,3], d2[P])."""
    b = Batch(ds)
    counts = np.zeros(ds.ntot, dtype=np.int64)
    rc = lib().orc_neighbours(b.ref, float(rcut), _p(counts), None, None, None, None, nthreads)
    if rc:
        raise RuntimeError(f"orc_neighbours failed ({rc})")
    off = np.zeros(ds.ntot + 1, dtype=np.int64)
    off[1:] = np.cumsum(counts)
    P = int(off[-1])
    j = np.zeros(max(P, 1), dtype=np.int32)
    sh = np.zeros((max(P, 1), 3), dtype=np.int32)
    d2 = np.zeros(max(P, 1), dtype=np.float64)
    rc = lib().orc_neighbours(b.ref, float(rcut), _p(counts), _p(off), _p(j), _p(sh), _p(d2),
                              nthreads)
    if rc:
        raise RuntimeError(f"orc_neighbours failed ({rc})")
    return off, j[:P], sh[:P], d2[:P]


def acsf(ds, funcs, mode=1, nthreads=1):
    """Raw (not standardised) ACSF values [Ntot, nG]."""
    b = Batch(ds)
    g = _gfuncs(funcs)
    out = np.zeros((ds.ntot, len(funcs)), dtype=np.float64)
    if mode == 1 and len({f.rcut for f in funcs}) > 1:
        mode = 0
    rc = lib().orc_acsf(b.ref, g, len(funcs), mode, _p(out), nthreads)
    if rc:
        raise RuntimeError(f"orc_acsf failed ({rc})")
    return out


def acsf_prime(ds, s, funcs):
    """Dense dG/dR of structure s, Fortran order (3, nG, N, N) returned as such."""
    b = Batch(ds)
    g = _gfuncs(funcs)
    N = int(ds.atom_offsets[s + 1] - ds.atom_offsets[s])
    out = np.zeros(3 * len(funcs) * N * N, dtype=np.float64)
    rc = lib().orc_acsf_prime(b.ref, s, g, len(funcs), _p(out))
    if rc:
        raise RuntimeError(f"orc_acsf_prime failed ({rc})")
    return out.reshape((3, len(funcs), N, N), order="F")


def zscore_stats(vals, ds):
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    ng = vals.shape[1]
    z = np.zeros(2 * ng)
    w = np.ascontiguousarray(ds.weights, dtype=np.int32)
    off = np.ascontiguousarray(ds.atom_offsets, dtype=np.int64)
    lib().orc_zscore_stats(_p(vals), vals.shape[0], ng, _p(off), ds.nstruct, _p(w), _p(z))
    return z.reshape(2, ng)


def zscore_apply(vals, zprec):
    vals = np.array(vals, dtype=np.float64, order="C")
    z = np.ascontiguousarray(zprec, dtype=np.float64).reshape(-1)
    lib().orc_zscore_apply(_p(vals), vals.shape[0], vals.shape[1], _p(z))
    return vals


# ------------------------------------------------------------------ network
def predict(dims, activation, params, feats, species):
    net = Net(dims, activation)
    feats = np.ascontiguousarray(feats, dtype=np.float64)
    params = np.ascontiguousarray(params, dtype=np.float64)
    sp = np.ascontiguousarray(species, dtype=np.int32)
    out = np.zeros((feats.shape[0], dims[-1]))
    lib().orc_predict(net.ref, _p(params), feats.shape[1], _p(feats), feats.shape[0], _p(sp),
                      _p(out))
    return out


def jacobian(dims, activation, params, feats, species):
    """Per-atom Jacobian, shape [Ntot, nOut, nF]."""
    net = Net(dims, activation)
    feats = np.ascontiguousarray(feats, dtype=np.float64)
    params = np.ascontiguousarray(params, dtype=np.float64)
    sp = np.ascontiguousarray(species, dtype=np.int32)
    nout, nf = dims[-1], feats.shape[1]
    out = np.zeros(feats.shape[0] * nout * nf)
    lib().orc_jacobian(net.ref, _p(params), nf, _p(feats), feats.shape[0], _p(sp), _p(out))
    return out.reshape(feats.shape[0], nf, nout).transpose(0, 2, 1).copy()


def forces(ds, funcs, zprec, jac, physical=False, nthreads=1):
    """Analytical forces [Ntot, nOut, 3] from per-atom Jacobians [Ntot, nOut, nG]; physical
    selects the exact derivative (every periodic image contributes) over the reference's."""
    b = Batch(ds)
    g = _gfuncs(funcs)
    nout = jac.shape[1]
    jf = np.ascontiguousarray(jac.transpose(0, 2, 1).reshape(jac.shape[0], -1))
    z = None if zprec is None else np.ascontiguousarray(zprec, dtype=np.float64).reshape(-1)
    out = np.zeros(ds.ntot * 3 * nout)
    rc = lib().orc_forces_mt(b.ref, g, len(funcs), _p(z), nout, _p(jf), int(physical), _p(out),
                             int(nthreads))
    if rc:
        raise RuntimeError(f"orc_forces failed ({rc})")
    return out.reshape(ds.ntot, nout, 3)


def train_gradients(dims, activation, params, feats, ds, order=None, loss="mse"):
    """Raw accumulated gradients [nSpecies, nParams] and per-atom predictions."""
    net = Net(dims, activation)
    params = np.ascontiguousarray(params, dtype=np.float64)
    nsp = params.shape[0]
    feats = np.ascontiguousarray(feats, dtype=np.float64)
    ngt = ds.global_targets.shape[1]
    nat = ds.atomic_targets.shape[1]
    gt = np.ascontiguousarray(ds.global_targets, dtype=np.float64)
    at = np.ascontiguousarray(ds.atomic_targets, dtype=np.float64)
    aw = np.ascontiguousarray(ds.atomic_weights, dtype=np.float64)
    w = np.ascontiguousarray(ds.weights, dtype=np.int32)
    sp = np.ascontiguousarray(ds.species, dtype=np.int32)
    off = np.ascontiguousarray(ds.atom_offsets, dtype=np.int64)
    if order is None:
        order = np.arange(1, ds.nstruct + 1, dtype=np.int32)
    order = np.ascontiguousarray(order, dtype=np.int32)
    dd = np.zeros_like(params)
    pred = np.zeros((ds.ntot, dims[-1]))
    rc = lib().orc_train_gradients(net.ref, _p(params), nsp, feats.shape[1], _p(feats), _p(sp),
                                   ds.nstruct, _p(off), ngt, nat, _p(gt), _p(at), _p(aw), _p(w),
                                   _p(order), LOSS[loss], _p(dd), _p(pred))
    if rc:
        raise RuntimeError(f"orc_train_gradients failed ({rc})")
    return dd, pred


def update_prepare(dims, activation, params, grad, strength=0.0, alpha=0.0, sum_weights=1.0):
    net = Net(dims, activation)
    params = np.ascontiguousarray(params, dtype=np.float64)
    g = np.array(grad, dtype=np.float64, order="C")
    nrm = lib().orc_update_prepare(net.ref, _p(params), params.shape[0], _p(g), strength, alpha,
                                   float(sum_weights))
    return g, nrm


def loss(kind, pred, ds, ngt, nat):
    """Dataset loss of loss.F90 (msLoss 512-579 and siblings), FP64, in loop order."""
    w = ds.weights
    aw = ds.atomic_weights
    off = ds.atom_offsets
    tot, nval = 0.0, 0.0

    def simple(p, t):
        p = np.asarray(p, dtype=np.float64)
        t = np.asarray(t, dtype=np.float64)
        if kind == "mse":
            return float(np.sum((t - p) ** 2) / p.size)
        if kind == "rms":
            return float(np.sqrt(np.sum((t - p) ** 2) / p.size))
        if kind == "mae":
            return float(np.sum(np.abs(t - p)) / p.size)
        if kind == "mape":
            return float(100.0 * np.sum(np.abs((t - p) / t)) / p.size)
        raise ValueError(kind)

    if ngt > 0:
        for s in range(ds.nstruct):
            gp = pred[off[s]:off[s + 1], :ngt].sum(axis=0)
            sw = float(np.sum(aw[off[s]:off[s + 1]]))
            tot += float(w[s]) * sw * simple(gp, ds.global_targets[s])
            nval += float(w[s]) * sw
    if nat > 0:
        for s in range(ds.nstruct):
            for a in range(off[s], off[s + 1]):
                tot += float(w[s]) * aw[a] * simple(pred[a, ngt:], ds.atomic_targets[a])
                nval += float(w[s]) * aw[a]
    return tot / nval


# ------------------------------------------------------------------ RNG / init / optimisers
class Ranlux:
    def __init__(self, seed, luxlev=3):
        self.h = lib().orc_ranlux_new(luxlev, seed)

    def get(self, n):
        out = np.zeros(n)
        lib().orc_ranlux_get(self.h, _p(out), n)
        return out

    def init_bpnn(self, dims, activation, nspecies):
        net = Net(dims, activation)
        out = np.zeros((nspecies, net.nparams))
        lib().orc_init_bpnn_params(self.h, net.ref, nspecies, _p(out))
        return out

    def shuffle(self, arr):
        a = np.ascontiguousarray(arr, dtype=np.int32).copy()
        lib().orc_knuth_shuffle(self.h, _p(a), len(a))
        return a

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_ranlux_free(self.h)
            self.h = None


class SteepestDescent:
    def __init__(self, x0, tol, maxdisp, lr):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        self.n = len(x0)
        self.h = lib().orc_sd_new(self.n, tol, maxdisp, lr, _p(x0))

    def next(self, fx, grad):
        g = np.ascontiguousarray(grad, dtype=np.float64)
        x = np.zeros(self.n)
        conv = lib().orc_sd_next(self.h, _p(g), _p(x))
        return x, bool(conv)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_opt_free(self.h)
            self.h = None


class _Opt:
    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_opt_free(self.h)
            self.h = None


class ConjGrad(_Opt):
    """conjgrad.F90 with its line minimiser (threshold, MaxDisplacement)."""

    def __init__(self, x0, tol, maxdisp):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        self.n = len(x0)
        self.h = lib().orc_cg_new(self.n, tol, maxdisp, _p(x0))

    def next(self, fx, grad):
        g = np.ascontiguousarray(grad, dtype=np.float64)
        x = np.zeros(self.n)
        conv = lib().orc_cg_next(self.h, float(fx), _p(g), _p(x))
        return x, bool(conv)


class Fire(_Opt):
    """fire.F90 (threshold, MaxDisplacement as the largest time step)."""

    def __init__(self, x0, tol, maxstep):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        self.n = len(x0)
        self.h = lib().orc_fire_new(self.n, tol, maxstep, _p(x0))

    def next(self, fx, grad):
        g = np.ascontiguousarray(grad, dtype=np.float64)
        x = np.zeros(self.n)
        conv = lib().orc_fire_next(self.h, _p(g), _p(x))
        return x, bool(conv)


class Lbfgs:
    def __init__(self, x0, tol, mindisp, maxdisp, mem=1000, linesearch=True, qndisp=False):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        self.n = len(x0)
        self.h = lib().orc_lbfgs_new(self.n, tol, mindisp, maxdisp, mem, int(linesearch),
                                     int(qndisp), _p(x0))

    def next(self, fx, grad):
        g = np.ascontiguousarray(grad, dtype=np.float64)
        x = np.zeros(self.n)
        conv = lib().orc_lbfgs_next(self.h, float(fx), _p(g), _p(x))
        return x, bool(conv)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_opt_free(self.h)
            self.h = None
