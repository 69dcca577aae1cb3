"""Fortnet netstat files (trained network + ACSF configuration), read side.

Mirrors ``TAcsf_fromFile`` (prog/fortnet/lib_descriptors/acsf.F90:1908-2135) and
``TBpnn_fromFile`` (prog/fortnet/lib_nn/bpnn.F90:1141-1288).  Network parameters are
returned as the reference's serialised vector per sub-network (H10 order of
``TNetwork_serializedWeightsAndBiases``, network.F90:397-427): every layer's weight
matrix column-major (including the zero ``ww(d_L, 1)`` of the output layer), then every
layer's bias vector (including the zero bias of the input layer).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import hdf5lite
from .fnetdata import element_symbol
from .gfunctions import GFunction

ACTIVATIONS = {
    "tanh": 0, "sigmoid": 1, "relu": 2, "lrelu": 3, "softplus": 4, "bent": 5, "atan": 6,
    "gaussian": 7, "heaviside": 8, "linear": 9,
}


def n_params(dims) -> int:
    dims = list(dims)
    return sum(dims[l] * dims[l + 1] for l in range(len(dims) - 1)) + dims[-1] + sum(dims)


def param_layout(dims):
    """Offsets of every layer's weights and biases in the serialised vector."""
    dims = list(dims)
    L = len(dims)
    woff, boff, ind = [], [], 0
    for l in range(L):
        woff.append(ind)
        ind += dims[l] * (dims[l + 1] if l < L - 1 else 1)
    for l in range(L):
        boff.append(ind)
        ind += dims[l]
    return woff, boff, ind


@dataclass
class Netstat:
    gfunctions: list            # list[GFunction] (empty if no ACSF mapping)
    zprec: np.ndarray | None    # [2, nG]: means, standard deviations
    atomic_numbers: np.ndarray  # sub-network order
    dims: list
    activation: str
    nglobal: int
    natomic: int
    params: np.ndarray          # [nSpecies, nParams]
    ext_indices: np.ndarray | None = None  # 1-based dataset external-feature columns


    @property
    def nspecies(self) -> int:
        return len(self.atomic_numbers)


def _scalar(v, cast=float):
    return cast(np.asarray(v).ravel()[0])


def read_netstat(path) -> Netstat:
    root = hdf5lite.read(path)
    ns = root["netstat"]
    gfuncs, zprec = [], None
    if "mapping" in ns:
        mp = ns["mapping"]
        nf = _scalar(mp.attrs["nfunctions"], int)
        for i in range(1, nf + 1):
            a = mp[f"function{i}"].attrs
            zz = np.asarray(a.get("atomicnumbers", [0, 0])).ravel()
            gfuncs.append(GFunction(
                type=str(a["type"]).strip().lower(),
                rcut=_scalar(a["cutoff"]),
                kappa=_scalar(a.get("kappa", 0.0)),
                rs=_scalar(a.get("rs", 0.0)),
                eta=_scalar(a.get("eta", 0.0)),
                lam=_scalar(a.get("lambda", 0.0)),
                xi=_scalar(a.get("xi", 0.0)),
                atomid=_scalar(a.get("atomid", 0), int),
                z1=int(zz[0]), z2=int(zz[1]),
            ))
        if "preconditioning" in mp:
            pc = mp["preconditioning"]
            zprec = np.stack([np.asarray(pc["means"].value, dtype=np.float64).ravel(),
                              np.asarray(pc["variances"].value, dtype=np.float64).ravel()])
    ext_indices = None
    if "external" in ns:
        ext_indices = np.asarray(ns["external/indices"].value, dtype=np.int32).ravel()
    bp = ns["bpnn"]
    atomic_numbers = np.asarray(bp["atomicnumbers"].value, dtype=np.int32).ravel()
    nglobal = _scalar(bp.attrs["nglobaltargets"], int)
    natomic = _scalar(bp.attrs["natomictargets"], int)
    dims, act, params = None, None, []
    for z in atomic_numbers:
        sub = bp[f"{element_symbol(int(z)).lower()}-subnetwork"]
        d = [int(x) for x in np.asarray(sub["topology"].value).ravel()]
        a = str(sub.attrs["activation"]).strip().lower()
        if dims is None:
            dims, act = d, a
        elif d != dims or a != act:
            raise ValueError("sub-networks with different topologies are not supported")
        woff, boff, npar = param_layout(dims)
        p = np.zeros(npar)
        for l in range(len(dims) - 1):
            lay = sub[f"layer{l + 1}"]
            w = np.asarray(lay["weights"].value, dtype=np.float64)  # (d_{l+1}, d_l) = ww^T
            p[woff[l]:woff[l] + dims[l] * dims[l + 1]] = w.reshape(-1)
            b = np.asarray(lay["bias"].value, dtype=np.float64).ravel()
            p[boff[l + 1]:boff[l + 1] + dims[l + 1]] = b
        params.append(p)
    return Netstat(gfunctions=gfuncs, zprec=zprec, atomic_numbers=atomic_numbers, dims=dims,
                   activation=act, nglobal=nglobal, natomic=natomic,
                   params=np.asarray(params), ext_indices=ext_indices)
