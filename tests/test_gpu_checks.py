"""The bounds-checked build of the library (-DFNETG_CHECKS; fortnet_gb300.build.build(checks=True)):
every index guard of the neighbour search, ACSF, force, MLP, tensor-core and JVP kernels
compiled in.  A failed guard records its site (file code x 100000 + line) and skips the
access it guards; fnetg_check_status reads the record.  The cases are the small ones that
reach the edges of those index paths: cells smaller than the cutoff (self and repeated
images), clusters of 1-40 atoms, and C3 structures large enough for the cell-list neighbour
search.  Each runs featurisation, prediction, forces, the training gradient and the feature
JVP (FP64 and FP32), and the tensor-core forms (FP32), through both builds: no guard may fail,
and the checked build's results equal the default build's (the guards change no arithmetic;
FP32 forces are accumulated with float atomics, so they agree to 1e-6 of their largest
component; the tensor-core gradient sums FP32 per-CTA partials whose number each build tunes
for itself, 1e-5; everything else to 1e-12).
"""

import dataclasses

import numpy as np
import pytest

from fortnet_gb300 import api, build, synthetic
from test_gpu_parity import cluster_dataset, mixed_functions, small_cell_dataset

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib():
    return build.build(checks=True)


def c3_sample():
    cfg = dataclasses.replace(synthetic.CONFIGS["C3"], nstruct=6, natoms=(120, 400), seed=77)
    return cfg, synthetic.generate(cfg, forces=True)


def cases():
    ds_small = small_cell_dataset(seed=21, n=5, L_bohr=6.0)
    f_small = [f for f in mixed_functions(7.0) if f.type != "g4"]
    ds_cl = cluster_dataset()
    f_cl = [f for f in mixed_functions(6.0, zs=(1, 6)) if f.type != "g4"]
    cfg, ds_c3 = c3_sample()
    return {"small_cells": (ds_small, f_small), "clusters": (ds_cl, f_cl),
            "c3_cell_lists": (ds_c3, synthetic.gfunctions(cfg))}


def run_flow(library, precision, ds, funcs, tc):
    nf = len(funcs)
    dims = [nf, 8, 6, 1]
    nsp = 1
    params = synthetic.normal_params(dims, nsp, 3)
    w = np.random.default_rng(5).normal(size=(ds.ntot, 3))
    out = {}
    sites = []
    with api.Context(precision, library=library) as ctx:
        ctx.upload(ds)
        ctx.set_species(np.zeros(ds.ntot, dtype=np.int32))
        ctx.set_gfunctions(funcs)
        out["pairs"] = ctx.neighbors()
        ctx.acsf(download=False)
        ctx.zscore(weights=ds.weights)
        out["features"] = ctx.features()
        ctx.set_network(dims, "tanh", params)
        ctx.set_targets(ds)
        out["atomic"], _ = ctx.predict()
        out["forces"] = ctx.forces()
        out["gradient"], _, _ = ctx.train_gradients("mse")
        out["jvp"] = ctx.features_jvp(w)
        sites.append(ctx.check_status())
        if tc:
            ctx.batch_setup(2)
            out["tc_atomic"], _ = ctx.batch_predict()
            out["tc_gradient"], _ = ctx.batch_gradients(0, natoms=int(ds.atom_offsets[2]))
            sites.append(ctx.check_status())
    return out, sites


@pytest.mark.parametrize("precision", [api.FP64, api.FP32])
@pytest.mark.parametrize("name", ["small_cells", "clusters", "c3_cell_lists"])
def test_checked_build_passes_every_guard_and_matches(checked_lib, name, precision):
    ds, funcs = cases()[name]
    tc = precision == api.FP32
    ref, s_ref = run_flow(None, precision, ds, funcs, tc)
    got, s_got = run_flow(checked_lib, precision, ds, funcs, tc)
    assert s_ref == [0] * len(s_ref)
    assert s_got == [0] * len(s_got), f"failed index check at site {max(s_got)}"
    for k, v in ref.items():
        g = got[k]
        if k == "pairs":
            assert g == v
            continue
        scale = max(float(np.max(np.abs(v))), 1e-300)
        tol = 1e-12
        if k == "forces" and precision == api.FP32:
            tol = 1e-6  # float vector atomics: accumulation order
        if k == "tc_gradient":
            tol = 1e-5  # FP32 per-CTA partials: the tuned CTA count may differ between builds
        assert float(np.max(np.abs(np.asarray(g) - np.asarray(v)))) <= tol * scale, k
    print(f"{name} ({'FP64' if precision == api.FP64 else 'FP32'}): checked build green, "
          f"{ds.ntot} atoms, {len(funcs)} functions")
