"""Fortnet datasets (``fnetdata`` HDF5 files) as flat, device-ready arrays.

Mirrors ``readHdfDataset`` (prog/fortnet/lib_io/fnetdata.F90:994-1216): the ragged
per-datapoint ``TGeometry`` / target containers become one CSR batch (``atom_offsets``)
of every array, which is the layout the GPU library consumes directly.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import hdf5lite

ELEMENTS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge "
    "As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm "
    "Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U "
    "Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og"
).split()


def element_symbol(z: int) -> str:
    return ELEMENTS[z - 1]


@dataclass
class Dataset:
    """A batch of structures in CSR form (coordinates in Bohr, cartesian)."""

    atom_offsets: np.ndarray            # int64 [S+1]
    coords: np.ndarray                  # float64 [Ntot, 3]
    atnum: np.ndarray                   # int32 [Ntot] atomic numbers
    species: np.ndarray                 # int32 [Ntot] 0-based global species (sub-network) index
    periodic: np.ndarray                # int32 [S]
    latvecs: np.ndarray                 # float64 [S, 9]; latvecs[s, i + 3k] = latVecs(i, k)
    atomic_numbers: np.ndarray          # int32 [nSpecies] (dataset order = sub-network order)
    weights: np.ndarray                 # int32 [S] datapoint weights
    atomic_weights: np.ndarray          # float64 [Ntot]
    global_targets: np.ndarray          # float64 [S, nGlobalTargets]
    atomic_targets: np.ndarray          # float64 [Ntot, nAtomicTargets]
    ext: np.ndarray | None = None       # float64 [Ntot, nExt]
    meta: dict = field(default_factory=dict)

    @property
    def nstruct(self) -> int:
        return int(self.atom_offsets.shape[0] - 1)

    @property
    def ntot(self) -> int:
        return int(self.atom_offsets[-1])

    @property
    def natoms(self) -> np.ndarray:
        return np.diff(self.atom_offsets)

    def subset(self, idx) -> "Dataset":
        """Structures ``idx`` (in that order) as a new batch."""
        idx = np.asarray(idx, dtype=np.int64)
        n = self.natoms[idx]
        off = np.zeros(len(idx) + 1, dtype=np.int64)
        off[1:] = np.cumsum(n)
        rows = np.concatenate([np.arange(self.atom_offsets[i], self.atom_offsets[i + 1])
                               for i in idx]) if len(idx) else np.zeros(0, dtype=np.int64)
        return Dataset(
            atom_offsets=off,
            coords=self.coords[rows].copy(),
            atnum=self.atnum[rows].copy(),
            species=self.species[rows].copy(),
            periodic=self.periodic[idx].copy(),
            latvecs=self.latvecs[idx].copy(),
            atomic_numbers=self.atomic_numbers.copy(),
            weights=self.weights[idx].copy(),
            atomic_weights=self.atomic_weights[rows].copy(),
            global_targets=self.global_targets[idx].copy(),
            atomic_targets=self.atomic_targets[rows].copy(),
            ext=None if self.ext is None else self.ext[rows].copy(),
            meta=dict(self.meta),
        )


def frac_to_cart(latvecs9: np.ndarray, frac: np.ndarray) -> np.ndarray:
    """``matmul(latVecs, coords)`` of fnetdata.F90:1136-1138, summed in index order."""
    L = latvecs9.reshape(3, 3).T  # L[i, k] = latVecs(i, k)
    out = np.empty_like(frac)
    for i in range(3):
        acc = L[i, 0] * frac[:, 0]
        acc = acc + L[i, 1] * frac[:, 1]
        acc = acc + L[i, 2] * frac[:, 2]
        out[:, i] = acc
    return out


def read_hdf_dataset(path) -> Dataset:
    """Read a Fortnet dataset file (``fnetdata/dataset``)."""
    root = hdf5lite.read(path)
    ds = root["fnetdata/dataset"]
    tr = ds["training"]
    npts = int(ds.attrs["ndatapoints"])
    next_ = int(ds.attrs["nextfeatures"])
    if int(ds.attrs["withstructures"]) != 1:
        raise ValueError("datasets without structures carry no geometry for ACSF")
    ngt = int(tr.attrs["nglobaltargets"])
    nat = int(tr.attrs["natomictargets"])
    atomic_numbers = np.asarray(ds["atomicnumbers"].value, dtype=np.int32).ravel()
    coords, atnum, gsp, per, lat, w, aw, gt, at, ext = ([] for _ in range(10))
    offsets = [0]
    for i in range(1, npts + 1):
        dp = ds[f"datapoint{i}"]
        geo = dp["geometry"]
        w.append(int(dp.attrs["weight"]))
        c = np.array(geo["coordinates"].value, dtype=np.float64).reshape(-1, 3)
        periodic = int(geo.attrs["periodic"]) == 1
        frac = int(geo.attrs["fractional"]) == 1
        L9 = np.zeros(9)
        if periodic:
            L9 = np.array(geo["basis"].value, dtype=np.float64).reshape(9)
            if frac:
                c = frac_to_cart(L9, c)
        n = c.shape[0]
        coords.append(c)
        atnum.append(np.asarray(geo["localattoatnum"].value, dtype=np.int32).ravel())
        gsp.append(np.asarray(geo["localattoglobalsp"].value, dtype=np.int32).ravel() - 1)
        per.append(1 if periodic else 0)
        lat.append(L9)
        if "atomicweights" in dp:
            aw.append(np.asarray(dp["atomicweights"].value, dtype=np.float64).ravel())
        else:
            aw.append(np.ones(n))
        gt.append(np.asarray(dp["globaltargets"].value, dtype=np.float64).ravel()
                  if ngt > 0 else np.zeros(0))
        at.append(np.asarray(dp["atomictargets"].value, dtype=np.float64).reshape(n, nat)
                  if nat > 0 else np.zeros((n, 0)))
        if next_ > 0:
            ext.append(np.asarray(dp["extfeatures"].value, dtype=np.float64).reshape(n, next_))
        offsets.append(offsets[-1] + n)
    return Dataset(
        atom_offsets=np.asarray(offsets, dtype=np.int64),
        coords=np.ascontiguousarray(np.concatenate(coords)),
        atnum=np.concatenate(atnum).astype(np.int32),
        species=np.concatenate(gsp).astype(np.int32),
        periodic=np.asarray(per, dtype=np.int32),
        latvecs=np.asarray(lat, dtype=np.float64).reshape(npts, 9),
        atomic_numbers=atomic_numbers,
        weights=np.asarray(w, dtype=np.int32),
        atomic_weights=np.concatenate(aw),
        global_targets=np.asarray(gt, dtype=np.float64).reshape(npts, ngt),
        atomic_targets=np.concatenate(at).reshape(offsets[-1], nat),
        ext=np.ascontiguousarray(np.concatenate(ext)) if next_ > 0 else None,
    )
