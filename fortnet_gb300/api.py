"""ctypes binding of libfnetg (include/fnetg.h) and a host-side mirror of the reference's
feature / network / loss interface for the hot path.

There is no CPU fallback: every call goes to the CUDA library, and a missing library or
GPU raises :class:`FnetgError`.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .gfunctions import GFUNC_DTYPE, pack

FP32, FP64 = 32, 64
ACT = {"tanh": 0, "sigmoid": 1, "relu": 2, "lrelu": 3, "softplus": 4, "bent": 5, "atan": 6,
       "gaussian": 7, "heaviside": 8, "linear": 9}
LOSS = {"mse": 0, "rms": 1, "mae": 2, "mape": 3}
OPT = {"sd": 0, "lbfgs": 1, "cg": 2, "fire": 3}
ERRORS = {-1: "invalid argument", -2: "shape mismatch", -3: "out of device memory",
          -4: "CUDA error", -5: "timeout", -6: "invalid geometry", -7: "unsupported"}

_lib = None


class FnetgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fnetg error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class _GFunc(C.Structure):
    _fields_ = [("type", C.c_int32), ("atomid", C.c_int32), ("z1", C.c_int32),
                ("z2", C.c_int32), ("rcut", C.c_double), ("kappa", C.c_double),
                ("rs", C.c_double), ("eta", C.c_double), ("lam", C.c_double),
                ("xi", C.c_double)]


assert C.sizeof(_GFunc) == GFUNC_DTYPE.itemsize


def library_path():
    return _build.LIB


_others = {}  # other builds of the library (the bounds-checked one), by path


def load(build_if_missing=True, path=None):
    """Load libfnetg.so (building it first if it is missing and nvcc is available); path
    selects another build of the library, for example the bounds-checked one
    (fortnet_gb300.build.build(checks=True))."""
    global _lib
    if path is not None and os.path.abspath(path) != os.path.abspath(_build.LIB):
        path = os.path.abspath(path)
        if path not in _others:
            if not os.path.exists(path):
                raise FnetgError(-7, f"{path} missing")
            _others[path] = _bind(C.CDLL(path))
        return _others[path]
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise FnetgError(-7, f"{path} missing; build it with fortnet_gb300.build.build()")
        _build.build()
    _lib = _bind(C.CDLL(path))
    return _lib


def _bind(L):
    """Argument and result types of every entry point."""
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "fnetg_create": (C.c_int, [C.POINTER(vp), i32, i32]),
        "fnetg_destroy": (C.c_int, [vp]),
        "fnetg_last_error": (C.c_char_p, [vp]),
        "fnetg_abi_version": (C.c_int, []),
        "fnetg_upload_structures": (C.c_int, [vp, i32, vp, vp, vp, vp, vp, vp, i32]),
        "fnetg_update_coords": (C.c_int, [vp, vp]),
        "fnetg_set_species": (C.c_int, [vp, vp]),
        "fnetg_set_gfunctions": (C.c_int, [vp, i32, vp]),
        "fnetg_neighbors": (C.c_int, [vp, dbl, C.POINTER(i64)]),
        "fnetg_get_neighbors": (C.c_int, [vp, vp, vp, vp, vp]),
        "fnetg_acsf": (C.c_int, [vp, vp]),
        "fnetg_acsf_zscore": (C.c_int, [vp, vp, vp, i32]),
        "fnetg_set_external_inputs": (C.c_int, [vp, i32, vp]),
        "fnetg_get_features": (C.c_int, [vp, vp, C.POINTER(i32)]),
        "fnetg_set_features": (C.c_int, [vp, i32, vp]),
        "fnetg_set_network": (C.c_int, [vp, i32, i32, vp, i32, vp]),
        "fnetg_get_params": (C.c_int, [vp, vp]),
        "fnetg_nparams": (i64, [i32, vp]),
        "fnetg_predict": (C.c_int, [vp, vp, vp]),
        "fnetg_jacobian": (C.c_int, [vp, vp]),
        "fnetg_forces": (C.c_int, [vp, vp]),
        "fnetg_forces_fd": (C.c_int, [vp, C.c_double, vp]),
        "fnetg_set_targets": (C.c_int, [vp, i32, i32, vp, vp, vp, vp]),
        "fnetg_train_gradients": (C.c_int, [vp, i32, vp, vp, vp, vp]),
        "fnetg_update_prepare": (C.c_int, [vp, vp, dbl, dbl, vp]),
        "fnetg_optimizer_init": (C.c_int, [vp, i32, dbl, dbl, dbl, dbl, i32, i32, i32]),
        "fnetg_train_iteration": (C.c_int, [vp, i32, dbl, dbl, vp, vp, vp, vp]),
        "fnetg_rng_create": (vp, [i32]),
        "fnetg_rng_destroy": (None, [vp]),
        "fnetg_rng_uniform": (C.c_int, [vp, vp, i64]),
        "fnetg_rng_init_params": (C.c_int, [vp, i32, i32, vp, vp]),
        "fnetg_rng_shuffle": (C.c_int, [vp, vp, i32]),
        "fnetg_get_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "fnetg_profile_enable": (C.c_int, [vp, i32]),
        "fnetg_profile_read": (C.c_int, [vp, C.c_char_p, C.POINTER(dbl), C.POINTER(i64)]),
        "fnetg_profile_reset": (C.c_int, [vp]),
        "fnetg_launch_count": (i64, [vp]),
        "fnetg_synchronize": (C.c_int, [vp]),
        "fnetg_check_status": (C.c_int, [vp, C.POINTER(i32)]),
        "fnetg_probe_peaks": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]),
        "fnetg_features_jvp": (C.c_int, [vp, vp, vp]),
        "fnetg_set_force_targets": (C.c_int, [vp, dbl, vp]),
        "fnetg_last_losses": (C.c_int, [vp, C.POINTER(dbl), C.POINTER(dbl)]),
        "fnetg_batch_setup": (C.c_int, [vp, i32]),
        "fnetg_batch_info": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i32),
                                       C.POINTER(i32)]),
        "fnetg_batch_gradients": (C.c_int, [vp, i32, i32, vp, vp]),
        "fnetg_batch_epoch": (C.c_int, [vp, i32, dbl, dbl, vp]),
        "fnetg_batch_predict": (C.c_int, [vp, vp, vp]),
        "fnetg_batch_sync_params": (C.c_int, [vp]),
        "fnetg_batch_train_bf16": (C.c_int, [vp, i32]),
        "fnetg_batch_forces": (C.c_int, [vp, vp, vp]),
        "fnetg_server_create": (C.c_int, [C.POINTER(vp), vp, i32, vp, i32, vp, vp, i32, vp, i32,
                                          vp]),
        "fnetg_server_destroy": (C.c_int, [vp]),
        "fnetg_server_last_error": (C.c_char_p, [vp]),
        "fnetg_server_clock_ns": (i64, []),
        "fnetg_server_submit": (C.c_int, [vp, i32, vp, vp, i32, vp, i64, C.POINTER(i64)]),
        "fnetg_server_wait": (C.c_int, [vp, i64, dbl, vp, vp, C.POINTER(dbl)]),
        "fnetg_server_stats_get": (C.c_int, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


def _check_out(a, shape):
    """A caller-owned output buffer must be writeable, C-contiguous float64 of the result's
    shape (the library writes through its raw pointer)."""
    if (a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]
            or tuple(a.shape) != tuple(shape)):
        raise ValueError("output buffer must be writeable, C-contiguous float64 of shape %s"
                         % (shape,))


class Context:
    """One library context: a CUDA stream, device-resident structures, features, network."""

    def __init__(self, precision=FP32, device=0, library=None):
        self.lib = load(path=library)
        h = C.c_void_p()
        rc = self.lib.fnetg_create(C.byref(h), int(precision), int(device))
        if rc != 0:
            raise FnetgError(rc, "fnetg_create failed (no usable CUDA device?)")
        self.h = h
        self.precision = precision
        self.nstruct = 0
        self.ntot = 0
        self.dims = None
        self.nspecies = 0
        self.ng = 0
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.fnetg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise FnetgError(rc, self.lib.fnetg_last_error(self.h).decode(errors="replace"))

    # -- structures -------------------------------------------------------------------
    def upload(self, ds):
        """Upload a fnetdata.Dataset (coordinates in Bohr)."""
        off = _c(ds.atom_offsets, np.int64)
        atnum = _c(ds.atnum, np.int32)
        coords = _c(ds.coords, np.float64)
        per = _c(ds.periodic, np.int32)
        lat = _c(ds.latvecs, np.float64)
        ext = _c(ds.ext, np.float64)
        next_ = 0 if ext is None else ext.shape[1]
        self._check(self.lib.fnetg_upload_structures(self.h, len(off) - 1, _p(off), _p(atnum),
                                                     _p(coords), _p(per), _p(lat), _p(ext),
                                                     next_))
        self.nstruct = len(off) - 1
        self.ntot = int(off[-1])
        self.offsets = off
        return self

    def update_coords(self, coords):
        coords = _c(coords, np.float64)
        self._check(self.lib.fnetg_update_coords(self.h, _p(coords)))

    def set_species(self, species):
        sp = _c(species, np.int32)
        self._check(self.lib.fnetg_set_species(self.h, _p(sp)))

    # -- ACSF --------------------------------------------------------------------------
    def set_gfunctions(self, funcs):
        arr = pack(funcs) if not isinstance(funcs, np.ndarray) else funcs
        arr = np.ascontiguousarray(arr, dtype=GFUNC_DTYPE)
        self._check(self.lib.fnetg_set_gfunctions(self.h, len(arr), _p(arr)))
        self.ng = len(arr)

    def neighbors(self, rcut=0.0):
        n = C.c_int64()
        self._check(self.lib.fnetg_neighbors(self.h, float(rcut), C.byref(n)))
        return n.value

    def get_neighbors(self):
        n = C.c_int64()
        off = np.zeros(self.ntot + 1, dtype=np.int64)
        self._check(self.lib.fnetg_get_neighbors(self.h, _p(off), None, None, None))
        P = int(off[-1])
        j = np.zeros(max(P, 1), dtype=np.int32)
        sh = np.zeros((max(P, 1), 3), dtype=np.int32)
        d2 = np.zeros(max(P, 1), dtype=np.float64)
        self._check(self.lib.fnetg_get_neighbors(self.h, _p(off), _p(j), _p(sh), _p(d2)))
        del n
        return off, j[:P], sh[:P], d2[:P]

    def acsf(self, download=True):
        out = np.zeros((self.ntot, self.ng)) if download else None
        self._check(self.lib.fnetg_acsf(self.h, _p(out)))
        return out

    def zscore(self, weights=None, zprec=None):
        """compute (zprec None) or apply given [2, nG] statistics; returns them."""
        w = _c(weights, np.int32)
        if zprec is None:
            z = np.zeros(2 * self.ng)
            self._check(self.lib.fnetg_acsf_zscore(self.h, _p(w), _p(z), 1))
        else:
            z = np.ascontiguousarray(zprec, dtype=np.float64).reshape(-1).copy()
            self._check(self.lib.fnetg_acsf_zscore(self.h, _p(w), _p(z), 0))
        return z.reshape(2, self.ng)

    def set_external_inputs(self, indices):
        idx = _c(np.asarray(indices if indices is not None else [], dtype=np.int32), np.int32)
        self._check(self.lib.fnetg_set_external_inputs(self.h, len(idx), _p(idx)))

    def features(self):
        nf = C.c_int32()
        self._check(self.lib.fnetg_get_features(self.h, None, C.byref(nf)))
        out = np.zeros((self.ntot, nf.value))
        self._check(self.lib.fnetg_get_features(self.h, _p(out), C.byref(nf)))
        return out

    def set_features(self, feats):
        f = _c(feats, np.float64)
        self._check(self.lib.fnetg_set_features(self.h, f.shape[1], _p(f)))

    # -- network -----------------------------------------------------------------------
    def set_network(self, dims, activation, params):
        dims_a = _c(dims, np.int32)
        params = _c(params, np.float64)
        act = ACT[activation] if isinstance(activation, str) else int(activation)
        nsp = params.shape[0] if params.ndim == 2 else 1
        self._check(self.lib.fnetg_set_network(self.h, nsp, len(dims_a), _p(dims_a), act,
                                               _p(params)))
        self.dims = [int(d) for d in dims_a]
        self.nspecies = nsp

    @property
    def nparams(self):
        d = _c(self.dims, np.int32)
        return int(self.lib.fnetg_nparams(len(d), _p(d)))

    def params(self):
        out = np.zeros((self.nspecies, self.nparams))
        self._check(self.lib.fnetg_get_params(self.h, _p(out)))
        return out

    def predict(self, atomic=True, out_atomic=None, out_global=None):
        """(atomic outputs [Ntot, nOut] or None, per-structure sums [S, nOut]).  out_atomic /
        out_global: caller-owned C-contiguous float64 buffers to fill (for example pinned host
        memory); atomic=False downloads the sums only (summed on the device in atom order)."""
        nout = self.dims[-1]
        at = None
        if atomic:
            at = out_atomic if out_atomic is not None else np.zeros((self.ntot, nout))
            _check_out(at, (self.ntot, nout))
        gl = out_global if out_global is not None else np.zeros((self.nstruct, nout))
        _check_out(gl, (self.nstruct, nout))
        self._check(self.lib.fnetg_predict(self.h, _p(at), _p(gl)))
        return at, gl

    def jacobian(self):
        nout = self.dims[-1]
        nf = self.dims[0]
        out = np.zeros((self.ntot, nout, nf))
        self._check(self.lib.fnetg_jacobian(self.h, _p(out)))
        return out

    def forces(self, out=None):
        """Analytical forces [Ntot, nOut, 3]; out: a caller-owned float64 buffer to fill."""
        nout = self.dims[-1]
        if out is None:
            out = np.zeros((self.ntot, nout, 3))
        _check_out(out, (self.ntot, nout, 3))
        self._check(self.lib.fnetg_forces(self.h, _p(out)))
        return out

    def forces_fd(self, delta):
        """Central finite-difference forces [Ntot, nOut, 3] with displacement delta (Bohr)."""
        nout = self.dims[-1]
        out = np.zeros((self.ntot, nout, 3))
        self._check(self.lib.fnetg_forces_fd(self.h, float(delta), _p(out)))
        return out

    def features_jvp(self, w):
        """Derivative of every atom's standardised inputs along per-atom vectors w [Ntot, 3]:
        [Ntot, nf] (the dense dG/dR of calculatePrime contracted with w)."""
        wv = _c(w, np.float64).reshape(self.ntot, 3)
        nf = C.c_int32()
        self._check(self.lib.fnetg_get_features(self.h, None, C.byref(nf)))
        out = np.zeros((self.ntot, nf.value))
        self._check(self.lib.fnetg_features_jvp(self.h, _p(wv), _p(out)))
        return out

    # -- training ----------------------------------------------------------------------
    def set_force_targets(self, weight, forces=None):
        """Force term weight / (3 Ntot) sum |F - F*|^2 in the training loss (0: off)."""
        f = None if forces is None else _c(forces, np.float64).reshape(self.ntot, 3)
        self._check(self.lib.fnetg_set_force_targets(self.h, float(weight), _p(f)))

    def last_losses(self):
        le, lf = C.c_double(), C.c_double()
        self._check(self.lib.fnetg_last_losses(self.h, C.byref(le), C.byref(lf)))
        return le.value, lf.value

    def set_targets(self, ds):
        gt = _c(ds.global_targets, np.float64)
        at = _c(ds.atomic_targets, np.float64)
        aw = _c(ds.atomic_weights, np.float64)
        w = _c(ds.weights, np.int32)
        self._check(self.lib.fnetg_set_targets(self.h, gt.shape[1], at.shape[1], _p(gt), _p(at),
                                               _p(aw), _p(w)))

    def train_gradients(self, loss="mse", order=None):
        grad = np.zeros((self.nspecies, self.nparams))
        lv = np.zeros(1)
        at = np.zeros((self.ntot, self.dims[-1]))
        o = _c(order, np.int32)
        self._check(self.lib.fnetg_train_gradients(self.h, LOSS[loss], _p(o), _p(grad), _p(lv),
                                                   _p(at)))
        return grad, float(lv[0]), at

    def update_prepare(self, grad, strength=0.0, alpha=0.0):
        g = np.array(grad, dtype=np.float64, order="C")
        nrm = np.zeros(1)
        self._check(self.lib.fnetg_update_prepare(self.h, _p(g), strength, alpha, _p(nrm)))
        return g, float(nrm[0])

    def optimizer_init(self, kind, threshold, min_disp, max_disp, learning_rate=0.01,
                       memory=1000, linemin=True, qn_max_disp=False):
        self._check(self.lib.fnetg_optimizer_init(self.h, OPT[kind], threshold, min_disp,
                                                  max_disp, learning_rate, memory, int(linemin),
                                                  int(qn_max_disp)))

    def train_iteration(self, loss="mse", strength=0.0, alpha=0.0, order=None):
        lv = C.c_double()
        gn = C.c_double()
        conv = C.c_int32()
        o = _c(order, np.int32)
        self._check(self.lib.fnetg_train_iteration(self.h, LOSS[loss], strength, alpha, _p(o),
                                                   C.byref(lv), C.byref(gn), C.byref(conv)))
        return lv.value, gn.value, bool(conv.value)

    # -- batched mixed-precision form (include/fnetg_batch.h) ---------------------------
    def batch_setup(self, batch_structures=256):
        """Mini-batches of consecutive structures, BF16 feature tiles and weight images for the
        tensor-core kernels (after features, z-score, network and targets are set)."""
        self._check(self.lib.fnetg_batch_setup(self.h, int(batch_structures)))
        self._batch_off = None

    def batch_info(self):
        nb, nt, cf, ct = C.c_int32(), C.c_int64(), C.c_int32(), C.c_int32()
        self._check(self.lib.fnetg_batch_info(self.h, C.byref(nb), C.byref(nt), C.byref(cf),
                                              C.byref(ct)))
        return {"batches": nb.value, "tiles": nt.value, "ctas_forward": cf.value,
                "ctas_train": ct.value}

    def batch_gradients(self, batch, loss="mse", natoms=None):
        """Raw gradient [nSpecies, nParams] of one mini-batch and its atoms' outputs (natoms:
        the mini-batch's atom count, to size the output; None skips the outputs)."""
        grad = np.zeros((self.nspecies, self.nparams))
        at = None if natoms is None else np.zeros(natoms)
        self._check(self.lib.fnetg_batch_gradients(self.h, int(batch), LOSS[loss], _p(grad),
                                                   _p(at)))
        return grad, at

    def batch_epoch(self, loss="mse", learning_rate=0.01, max_disp=1e4, want_loss=True):
        lv = np.zeros(1)
        self._check(self.lib.fnetg_batch_epoch(self.h, LOSS[loss], float(learning_rate),
                                               float(max_disp), _p(lv) if want_loss else None))
        return float(lv[0]) if want_loss else None

    def batch_predict(self, atomic=True, out_global=None):
        at = np.zeros(self.ntot) if atomic else None
        gl = out_global if out_global is not None else np.zeros((self.nstruct, 1))
        _check_out(gl, (self.nstruct, 1))
        self._check(self.lib.fnetg_batch_predict(self.h, _p(at), _p(gl)))
        return at, gl

    def batch_forces(self, out_global=None, out_forces=None):
        """Energies [S, 1] and forces [N, 1, 3] with the network passes on the tensor cores."""
        gl = out_global if out_global is not None else np.zeros((self.nstruct, 1))
        _check_out(gl, (self.nstruct, 1))
        fo = out_forces if out_forces is not None else np.zeros((self.ntot, 1, 3))
        _check_out(fo, (self.ntot, 1, 3))
        self._check(self.lib.fnetg_batch_forces(self.h, _p(gl), _p(fo)))
        return gl, fo

    def batch_train_bf16(self, on=True):
        """Full-batch training gradients from the tensor-core kernels (the precision form)."""
        self._check(self.lib.fnetg_batch_train_bf16(self.h, int(on)))

    def batch_sync_params(self):
        self._check(self.lib.fnetg_batch_sync_params(self.h))

    # -- plumbing ----------------------------------------------------------------------
    def check_status(self):
        """The first failed index check of the bounds-checked build since the last call
        (file code x 100000 + line), 0 if none; always 0 for the default build."""
        site = C.c_int32()
        self._check(self.lib.fnetg_check_status(self.h, C.byref(site)))
        return site.value

    def probe_peaks(self):
        """Measured FP32 FMA rate (TFLOP/s), ex2 rate (10^12 op/s) and FP64 FMA rate (TFLOP/s)
        of the device."""
        f, e, d = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.fnetg_probe_peaks(self.h, C.byref(f), C.byref(e), C.byref(d)))
        return f.value, e.value, d.value

    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.fnetg_get_stream(self.h, C.byref(s)))
        return s.value

    def profile(self, enable=True):
        self._check(self.lib.fnetg_profile_enable(self.h, int(enable)))

    def profile_read(self, name):
        ms = C.c_double()
        n = C.c_int64()
        self.lib.fnetg_profile_read(self.h, name.encode(), C.byref(ms), C.byref(n))
        return ms.value, n.value

    def profile_reset(self):
        self._check(self.lib.fnetg_profile_reset(self.h))

    def launch_count(self):
        return int(self.lib.fnetg_launch_count(self.h))

    def synchronize(self):
        self._check(self.lib.fnetg_synchronize(self.h))


class Rng:
    """RANLUX stream of the reference (luxury level 3)."""

    def __init__(self, seed):
        self.lib = load()
        self.h = self.lib.fnetg_rng_create(int(seed))

    def uniform(self, n):
        out = np.zeros(n)
        self.lib.fnetg_rng_uniform(self.h, _p(out), n)
        return out

    def init_params(self, dims, nspecies):
        d = _c(dims, np.int32)
        n = int(self.lib.fnetg_nparams(len(d), _p(d)))
        out = np.zeros((nspecies, n))
        rc = self.lib.fnetg_rng_init_params(self.h, nspecies, len(d), _p(d), _p(out))
        if rc:
            raise FnetgError(rc, "rng_init_params")
        return out

    def shuffle(self, arr):
        a = np.array(arr, dtype=np.int32)
        self.lib.fnetg_rng_shuffle(self.h, _p(a), len(a))
        return a

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.fnetg_rng_destroy(self.h)
            self.h = None


class _ServerConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("lanes", C.c_int32),
                ("tensor_cores", C.c_int32), ("max_batch_atoms", C.c_int64),
                ("hbm_budget_bytes", C.c_int64), ("reserve_bytes", C.c_int64)]


class _ServerStats(C.Structure):
    _fields_ = [("requests", C.c_int64), ("batches", C.c_int64), ("atoms", C.c_int64),
                ("max_batch_atoms", C.c_int64), ("max_batch_requests", C.c_int64),
                ("device_bytes", C.c_int64), ("batch_cap_atoms", C.c_int64),
                ("lanes", C.c_int32), ("max_in_flight", C.c_int32), ("busy_s", C.c_double),
                ("max_batch_s", C.c_double)]


class Server:
    """Energy/force prediction service (include/fnetg_serve.h): requests queued from any
    thread, served by continuous batching over ``lanes`` concurrent device batches."""

    def __init__(self, atomic_numbers, funcs, zprec, dims, activation, params, precision=FP32,
                 device=0, lanes=0, max_batch_atoms=0, hbm_budget_bytes=0, reserve_bytes=0,
                 tensor_cores=False):
        self.lib = load()
        cfg = _ServerConfig(int(precision), int(device), int(lanes), int(bool(tensor_cores)),
                            int(max_batch_atoms), int(hbm_budget_bytes), int(reserve_bytes))
        g = pack(funcs) if not isinstance(funcs, np.ndarray) else funcs
        self.ng = len(g)
        self.dims = [int(d) for d in dims]
        self.nout = self.dims[-1]
        zn = _c(np.asarray(atomic_numbers), np.int32)
        zp = _c(zprec, np.float64)
        dm = _c(self.dims, np.int32)
        pr = _c(params, np.float64)
        h = C.c_void_p()
        act = ACT[activation] if isinstance(activation, str) else int(activation)
        rc = self.lib.fnetg_server_create(C.byref(h), C.byref(cfg), len(zn), _p(zn), self.ng,
                                          g.ctypes.data_as(C.c_void_p), _p(zp), len(dm), _p(dm),
                                          act, _p(pr))
        if rc != 0:
            raise FnetgError(rc, "fnetg_server_create failed")
        self.h = h

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.fnetg_server_last_error(self.h)
            raise FnetgError(rc, msg.decode() if msg else "")

    def clock_ns(self):
        return int(self.lib.fnetg_server_clock_ns())

    def submit(self, atnum, coords, latvecs=None, arrival_ns=0):
        """Queue one structure (coordinates in Bohr, [n, 3]); returns its ticket."""
        an = _c(atnum, np.int32)
        xyz = _c(coords, np.float64)
        lat = None if latvecs is None else _c(latvecs, np.float64)
        t = C.c_int64()
        self._check(self.lib.fnetg_server_submit(self.h, len(an), _p(an), _p(xyz),
                                                 0 if lat is None else 1, _p(lat),
                                                 int(arrival_ns), C.byref(t)))
        return t.value, len(an)

    def wait(self, ticket, natoms, timeout=-1.0, forces=True):
        """(energy[nout], forces[natoms, nout, 3] or None, latency in ms)."""
        e = np.zeros(self.nout)
        f = np.zeros((natoms, self.nout, 3)) if forces else None
        lat = C.c_double()
        self._check(self.lib.fnetg_server_wait(self.h, int(ticket), float(timeout), _p(e),
                                               _p(f), C.byref(lat)))
        return e, f, lat.value

    def stats(self):
        st = _ServerStats()
        self._check(self.lib.fnetg_server_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.fnetg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
