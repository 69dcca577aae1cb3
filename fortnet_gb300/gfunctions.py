"""ACSF G-function descriptions (TGFunction, prog/fortnet/lib_descriptors/acsf.F90:40-75).

The packed form (``pack``) is the ``fnetg_gfunc`` record array the C-ABI takes.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, replace
from itertools import combinations_with_replacement

import numpy as np

BOHR__AA = 0.529177249              # lib_dftbp/constants.F90:18
AA__BOHR = 1.0 / BOHR__AA           # lib_dftbp/constants.F90:21

TYPE_CODES = {"g1": 1, "g2": 2, "g3": 3, "g4": 4, "g5": 5}

# numpy view of the C struct fnetg_gfunc (include/fnetg.h)
GFUNC_DTYPE = np.dtype([
    ("type", "<i4"), ("atomid", "<i4"), ("z1", "<i4"), ("z2", "<i4"),
    ("rcut", "<f8"), ("kappa", "<f8"), ("rs", "<f8"), ("eta", "<f8"),
    ("lambda", "<f8"), ("xi", "<f8"),
])


@dataclass(frozen=True)
class GFunction:
    type: str           # 'g1' .. 'g5'
    rcut: float         # Bohr
    kappa: float = 0.0
    rs: float = 0.0
    eta: float = 0.0
    lam: float = 0.0
    xi: float = 0.0
    atomid: int = 0
    z1: int = 0
    z2: int = 0

    @property
    def angular(self) -> bool:
        return self.type in ("g4", "g5")

    @property
    def radial(self) -> bool:
        return not self.angular


def from_auto_scheme(rcut: float, n_radial: int, n_angular: int, atomid: int = 0):
    """TGFunctions_fromAutoScheme (acsf.F90:276-363); rcut in Bohr."""
    rs_step = rcut / (n_radial - 1)
    g2eta = 5.0 * math.log(10.0) / (2.0 * rs_step) ** 2
    g2rs = [0.0] + [ii * rs_step for ii in range(1, n_radial)]
    g5eta = 2.0 * math.log(10.0) / rcut ** 2
    lam, xis = [], []
    ind = 1
    for ii in range(0, math.ceil(n_angular / 2.0 - 1.0) + 1):
        xi = 1.0 if n_angular <= 2 else 1.0 + ii * 30.0 / (n_angular - 2.0)
        stop = False
        for jj in (1, -1):
            lam.append(float(jj))
            xis.append(xi)
            if ind >= n_angular:
                stop = True
                break
            ind += 1
        if stop:
            break
    funcs = [GFunction("g2", rcut, rs=g2rs[i], eta=g2eta, atomid=atomid) for i in range(n_radial)]
    funcs += [GFunction("g5", rcut, xi=xis[i], eta=g5eta, lam=lam[i], atomid=atomid)
              for i in range(n_angular)]
    return funcs


def process_acsf_functions(funcs, atomic_numbers, reduce: bool = False):
    """Species expansion of processAcsfFunctions (lib_fortnet/initprogram.F90:1453-1527):
    radial functions once per species, angular ones once per combination with replacement
    (lib_utils/intmanip.F90:84-142), interleaved in input order."""
    atomic_numbers = [int(z) for z in atomic_numbers]
    if reduce or len(atomic_numbers) <= 1:
        return list(funcs)
    combs = list(combinations_with_replacement(atomic_numbers, 2))
    out = []
    for f in funcs:
        if f.radial:
            out += [replace(f, z1=z, z2=0) for z in atomic_numbers]
        else:
            out += [replace(f, z1=a, z2=b) for a, b in combs]
    return out


def pack(funcs) -> np.ndarray:
    arr = np.zeros(len(funcs), dtype=GFUNC_DTYPE)
    for i, f in enumerate(funcs):
        arr[i] = (TYPE_CODES[f.type], f.atomid, f.z1, f.z2, f.rcut, f.kappa, f.rs, f.eta,
                  f.lam, f.xi)
    return arr


def unpack(arr) -> list:
    inv = {v: k for k, v in TYPE_CODES.items()}
    return [GFunction(inv[int(r["type"])], float(r["rcut"]), float(r["kappa"]), float(r["rs"]),
                      float(r["eta"]), float(r["lambda"]), float(r["xi"]), int(r["atomid"]),
                      int(r["z1"]), int(r["z2"])) for r in arr]
