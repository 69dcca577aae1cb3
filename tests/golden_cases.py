"""Loader for the golden cases extracted from the reference's regression tests, and the
reference's program flow for one case (feature assembly, training iterations) written
against a pluggable backend (the oracle on the CPU, the CUDA library on the GPU)."""

from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np

from fortnet_gb300.fnetdata import Dataset
from fortnet_gb300.gfunctions import unpack

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# comparison tolerance of the reference's own test driver (testwithworkdir.py:24-25)
ATOL = 1e-10
RTOL = 1e-09


def case_names():
    with open(os.path.join(GOLDEN, "INDEX.json")) as fh:
        return json.load(fh)["cases"]


def load_dataset(name) -> Dataset:
    z = np.load(os.path.join(GOLDEN, "datasets", name + ".npz"))
    return Dataset(
        atom_offsets=z["atom_offsets"], coords=z["coords"], atnum=z["atnum"],
        species=z["species"], periodic=z["periodic"], latvecs=z["latvecs"],
        atomic_numbers=z["atomic_numbers"], weights=z["weights"],
        atomic_weights=z["atomic_weights"], global_targets=z["global_targets"],
        atomic_targets=z["atomic_targets"], ext=z["ext"] if "ext" in z else None)


@dataclass
class Case:
    name: str
    settings: dict
    arrays: dict
    ds: Dataset

    def net(self, prefix):
        a = self.arrays
        return dict(
            gfuncs=unpack(a[f"{prefix}gfuncs"]) if a[f"{prefix}gfuncs"].size else [],
            zprec=a.get(f"{prefix}zprec"),
            dims=[int(x) for x in a[f"{prefix}dims"]],
            params=a[f"{prefix}params"],
            atomic_numbers=a[f"{prefix}atomic_numbers"],
            nglobal=int(a[f"{prefix}nglobal"]),
            natomic=int(a[f"{prefix}natomic"]),
            activation=self.settings[f"{prefix}activation"],
            ext_indices=a.get(f"{prefix}ext_indices"),
        )


def load_case(name) -> Case:
    z = np.load(os.path.join(GOLDEN, "cases", name.replace("/", "__") + ".npz"))
    arrays = {k: z[k] for k in z.files}
    settings = json.loads(bytes(arrays.pop("settings")).decode())
    if "hsd" in arrays:
        settings["hsd"] = bytes(arrays.pop("hsd")).decode()
    return Case(name, settings, arrays, load_dataset(settings["dataset"]))


def species_index(ds, atomic_numbers):
    """Map every atom to its sub-network (localAtToGlobalSp for the network's species)."""
    lut = {int(z): i for i, z in enumerate(atomic_numbers)}
    return np.array([lut[int(z)] for z in ds.atnum], dtype=np.int32)


def assemble_features(acsf_vals, ds, ext_indices):
    """TFeatures_collect (lib_types/features.F90:200-265): [ACSF ; external features]."""
    parts = []
    if acsf_vals is not None and acsf_vals.shape[1] > 0:
        parts.append(acsf_vals)
    if ext_indices is not None and len(ext_indices) > 0:
        parts.append(ds.ext[:, np.asarray(ext_indices) - 1])
    return np.ascontiguousarray(np.concatenate(parts, axis=1))


def run_training(case, backend):
    """The train-mode flow of fortnet.F90 (handleInitialisation, calculateMappings, nTrain)
    with SD or L-BFGS; returns (zprec or None, final params)."""
    st = case.settings
    ds = case.ds
    out = case.net("out_")
    gfuncs = out["gfuncs"]
    if st["read_netstat"]:
        inp = case.net("in_")
        params = inp["params"].copy()
        zprec = inp["zprec"]
        ext_idx = inp["ext_indices"]
        dims, act = inp["dims"], inp["activation"]
    else:
        zprec = None
        ext_idx = case.arrays.get("hsd_ext_indices")
        dims, act = out["dims"], out["activation"]
        params = None
    vals = backend.acsf(ds, gfuncs) if gfuncs else None
    if vals is not None and st.get("standardize") and zprec is None:
        zprec = backend.zscore_stats(vals, ds)
    if vals is not None and zprec is not None:
        vals = backend.zscore_apply(vals, zprec)
    feats = assemble_features(vals, ds, ext_idx)
    rng = backend.ranlux(st["seed"])
    nsp = len(ds.atomic_numbers)
    if params is None:
        params = rng.init_bpnn(dims, act, nsp)
    sp = species_index(ds, ds.atomic_numbers)
    dsv = Dataset(**{**ds.__dict__, "species": sp})
    order = np.arange(1, ds.nstruct + 1, dtype=np.int32)
    if st["shuffle"]:
        order = rng.shuffle(order)
    if st["optimizer"] == "sd":
        opts = [backend.sd(params[s], st["threshold"], st["max_disp"], st["learning_rate"])
                for s in range(nsp)]
    elif st["optimizer"] == "cg":
        opts = [backend.cg(params[s], st["threshold"], st["max_disp"]) for s in range(nsp)]
    elif st["optimizer"] == "fire":
        opts = [backend.fire(params[s], st["threshold"], st["max_disp"]) for s in range(nsp)]
    else:
        opts = [backend.lbfgs(params[s], st["threshold"], st["min_disp"], st["max_disp"],
                              st["memory"], st["linemin"], st["qn_max_disp"])
                for s in range(nsp)]
    dd, _ = backend.train_gradients(dims, act, params, feats, dsv, order, st["loss"])
    for _ in range(st["niter"]):
        grad, _ = backend.update_prepare(dims, act, params, dd, st["regu_strength"],
                                         st["regu_alpha"], float(np.sum(ds.weights)))
        newp = np.zeros_like(params)
        for s in range(nsp):
            newp[s], _ = opts[s].next(0.0, grad[s])
        params = newp
        if st["shuffle"]:
            order = rng.shuffle(order)
        dd, _ = backend.train_gradients(dims, act, params, feats, dsv, order, st["loss"])
    return zprec, params


def fd_forces(backend, ds, inp, sp, delta):
    """forceAnalysis_finiteDiff (forces.F90:182-306): central differences of each structure's
    summed outputs under displacements -delta / +delta of one coordinate.  [Ntot, 3*nOut]"""
    nout = inp["dims"][-1]
    out = np.zeros((ds.ntot, 3 * nout))
    for s in range(ds.nstruct):
        a0, a1 = int(ds.atom_offsets[s]), int(ds.atom_offsets[s + 1])
        n = a1 - a0
        copies = []
        for a in range(a0, a1):
            for c in range(3):
                for sign in (-1.0, 1.0):
                    x = ds.coords[a0:a1].copy()
                    x[a - a0, c] += sign * delta
                    copies.append(x)
        m = len(copies)
        sub = Dataset(
            atom_offsets=np.arange(m + 1, dtype=np.int64) * n, coords=np.concatenate(copies),
            atnum=np.tile(ds.atnum[a0:a1], m), species=np.tile(sp[a0:a1], m),
            periodic=np.repeat(ds.periodic[s:s + 1], m), latvecs=np.repeat(ds.latvecs[s:s + 1], m, 0),
            atomic_numbers=ds.atomic_numbers, weights=np.ones(m, np.int32),
            atomic_weights=np.ones(m * n), global_targets=np.zeros((m, 0)),
            atomic_targets=np.zeros((m * n, 0)),
            ext=None if ds.ext is None else np.tile(ds.ext[a0:a1], (m, 1)))
        vals = backend.acsf(sub, inp["gfuncs"])
        if inp["zprec"] is not None:
            vals = backend.zscore_apply(vals, inp["zprec"])
        feats = assemble_features(vals, sub, inp["ext_indices"])
        pred = backend.predict(inp["dims"], inp["activation"], inp["params"], feats,
                               np.tile(sp[a0:a1], m))
        glob = np.add.reduceat(pred, sub.atom_offsets[:-1], axis=0)
        k = 0
        for a in range(a0, a1):
            for c in range(3):
                out[a, c::3] = (glob[k] - glob[k + 1]) / (2.0 * delta)
                k += 2
    return out


def run_prediction(case, backend):
    """predict/validate-mode flow: features from the input netstat, iPredict per atom and
    (if requested) analytical forces.  Returns (raw predictions [Ntot,nOut], forces|None)."""
    ds = case.ds
    inp = case.net("in_")
    vals = backend.acsf(ds, inp["gfuncs"]) if inp["gfuncs"] else None
    if vals is not None and inp["zprec"] is not None:
        vals = backend.zscore_apply(vals, inp["zprec"])
    feats = assemble_features(vals, ds, inp["ext_indices"])
    sp = species_index(ds, inp["atomic_numbers"])
    pred = backend.predict(inp["dims"], inp["activation"], inp["params"], feats, sp)
    forces = None
    if case.settings.get("forces") == "finitedifferences":
        forces = fd_forces(backend, ds, inp, sp, case.settings["fd_delta"])
    if case.settings.get("forces") == "analytical":
        jac = backend.jacobian(inp["dims"], inp["activation"], inp["params"], feats, sp)
        ng = len(inp["gfuncs"])
        forces = backend.forces(ds, inp["gfuncs"], inp["zprec"], jac[:, :, :ng])
    return pred, forces
