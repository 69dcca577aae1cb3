"""The reference program's flows for one golden case, run through the CUDA library's C-ABI
(prediction / validation with analytical forces, and training with SD or L-BFGS)."""

from __future__ import annotations

import numpy as np

import golden_cases as G
from fortnet_gb300 import api


def prediction(case, precision=api.FP64):
    ds = case.ds
    inp = case.net("in_")
    with api.Context(precision) as ctx:
        ctx.upload(ds)
        ctx.set_species(G.species_index(ds, inp["atomic_numbers"]))
        gf = inp["gfuncs"]
        ext = inp["ext_indices"]
        if gf:
            ctx.set_gfunctions(gf)
            ctx.set_external_inputs(ext if ext is not None else [])
            ctx.acsf(download=False)
            if inp["zprec"] is not None:
                ctx.zscore(zprec=inp["zprec"])
        else:
            ctx.set_features(ds.ext[:, np.asarray(ext) - 1])
        ctx.set_network(inp["dims"], inp["activation"], inp["params"])
        pred, _ = ctx.predict()
        forces = None
        if case.settings.get("forces") == "analytical":
            forces = ctx.forces()
        elif case.settings.get("forces") == "finitedifferences":
            forces = ctx.forces_fd(case.settings["fd_delta"])
        return pred, forces


def training(case, precision=api.FP64):
    st = case.settings
    ds = case.ds
    out = case.net("out_")
    gf = out["gfuncs"]
    if st["read_netstat"]:
        inp = case.net("in_")
        params, zprec, ext = inp["params"], inp["zprec"], inp["ext_indices"]
        dims, act = inp["dims"], inp["activation"]
    else:
        params, zprec = None, None
        ext = case.arrays.get("hsd_ext_indices")
        dims, act = out["dims"], out["activation"]
    rng = api.Rng(st["seed"])
    with api.Context(precision) as ctx:
        ctx.upload(ds)
        ctx.set_species(ds.species)
        if gf:
            ctx.set_gfunctions(gf)
            ctx.set_external_inputs(ext if ext is not None else [])
            ctx.acsf(download=False)
            if st.get("standardize") and zprec is None:
                zprec = ctx.zscore(weights=ds.weights)
            elif zprec is not None:
                ctx.zscore(zprec=zprec)
        else:
            ctx.set_features(ds.ext[:, np.asarray(ext) - 1])
        nsp = len(ds.atomic_numbers)
        if params is None:
            params = rng.init_params(dims, nsp)
        ctx.set_network(dims, act, params)
        ctx.set_targets(ds)
        ctx.optimizer_init(st["optimizer"], st["threshold"], st["min_disp"], st["max_disp"],
                           st["learning_rate"], st["memory"], st["linemin"], st["qn_max_disp"])
        for _ in range(st["niter"]):
            ctx.train_iteration(st["loss"], st["regu_strength"], st["regu_alpha"])
        return (zprec if st.get("standardize") or st["read_netstat"] else None), ctx.params()
