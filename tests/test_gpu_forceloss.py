"""Force-loss training (include/fnetg.h: fnetg_features_jvp, fnetg_set_force_targets) against
the oracle.

* The matrix-free dG/dR product u = (dx/dR) w (jvp.cu) against central differences of the
  oracle's standardised features along w: FP64 within 1e-6 relative to each feature's largest
  derivative, FP32 within 1e-4; on cells smaller than the cutoff (self images, repeated
  images), with G1, G2, G3 and G5 (integer and non-integer xi), species resolved and not.
* The gradient of the force term L_F = c / (3N) sum |F - F*|^2 (forceloss.cu) against central
  differences of the oracle's L_F in the parameters (oracle forces from its dense dG/dR with
  the physical derivative), FP64, within 1e-6 of the gradient's largest component.
* The FP32 gradient of L_E + L_F against the FP64 one (norm-wise 1e-3, printed), and training
  iterations that lower both loss terms.
"""

import dataclasses

import numpy as np
import pytest

import oracle as O
from fortnet_gb300 import api, synthetic
from fortnet_gb300.fnetdata import Dataset
from test_gpu_batch import random_params
from test_gpu_parity import mixed_functions, small_cell_dataset

pytestmark = pytest.mark.gpu


def shifted(ds, coords):
    return Dataset(**{**ds.__dict__, "coords": coords})


def oracle_x(ds, funcs, zprec):
    return O.zscore_apply(O.acsf(ds, funcs), zprec)


def gpu_ctx(precision, ds, funcs, zprec, species=None):
    ctx = api.Context(precision)
    ctx.upload(ds)
    ctx.set_species(ds.species if species is None else species)
    ctx.set_gfunctions(funcs)
    ctx.acsf(download=False)
    ctx.zscore(zprec=zprec)
    return ctx


def small_c4(nstruct=3, natoms=(20, 30), seed=11):
    """C4's species and functions on small cells (L ~ 7 A < 2 rc: repeated images)."""
    cfg = dataclasses.replace(synthetic.CONFIGS["C4"], nstruct=nstruct, natoms=natoms, seed=seed)
    return cfg, synthetic.generate(cfg, forces=True)


@pytest.mark.parametrize("kind", ["small_cells", "c4_small"])
def test_features_jvp_matches_oracle_finite_differences(kind):
    if kind == "small_cells":
        ds = small_cell_dataset(seed=21, n=5, L_bohr=6.0)
        funcs = [f for f in mixed_functions(7.0) if f.type != "g4"]
    else:
        cfg, ds = small_c4()
        funcs = synthetic.gfunctions(cfg)
    zprec = O.zscore_stats(O.acsf(ds, funcs), ds)
    w = np.random.default_rng(3).normal(size=(ds.ntot, 3))
    h = 1e-6
    u_fd = (oracle_x(shifted(ds, ds.coords + h * w), funcs, zprec)
            - oracle_x(shifted(ds, ds.coords - h * w), funcs, zprec)) / (2 * h)
    scale = np.maximum(np.abs(u_fd).max(axis=0), 1e-12)
    errs = {}
    for prec in (api.FP64, api.FP32):
        with gpu_ctx(prec, ds, funcs, zprec) as ctx:
            u = ctx.features_jvp(w)
        errs[prec] = float(np.max(np.abs(u - u_fd) / scale))
    print(f"{kind}: dG/dR . w vs oracle differences: FP64 {errs[api.FP64]:.2e}, "
          f"FP32 {errs[api.FP32]:.2e} of each feature's scale")
    assert errs[api.FP64] <= 1e-6
    assert errs[api.FP32] <= 1e-4


def oracle_force_loss(ds, funcs, zprec, dims, params, Ft, c):
    feats = oracle_x(ds, funcs, zprec)
    jac = O.jacobian(dims, "tanh", params, feats, ds.species)
    F = O.forces(ds, funcs, zprec, jac, physical=True)[:, 0, :]
    return c / (3 * ds.ntot) * float(np.sum((F - Ft) ** 2))


def test_force_loss_gradient_matches_oracle_finite_differences():
    cfg, ds = small_c4()
    funcs = synthetic.gfunctions(cfg)
    dims = [len(funcs), 8, 6, 1]
    params = random_params(dims, 3, seed=9)
    zprec = O.zscore_stats(O.acsf(ds, funcs), ds)
    Ft = ds.meta["forces"]
    c = 0.1
    with gpu_ctx(api.FP64, ds, funcs, zprec) as ctx:
        ctx.set_network(dims, "tanh", params)
        ctx.set_targets(ds)
        g_e, le, _ = ctx.train_gradients("mse")
        ctx.set_force_targets(c, Ft)
        g_all, l_all, _ = ctx.train_gradients("mse")
        le2, lf = ctx.last_losses()
    sumw = float(ds.weights.sum())
    g_f = (g_all - g_e) / sumw
    lf_ref = oracle_force_loss(ds, funcs, zprec, dims, params, Ft, c)
    assert abs(lf - lf_ref) <= 1e-10 * lf_ref
    assert abs(le2 - le) <= 1e-12 * abs(le) and abs(l_all - (le + lf)) <= 1e-12 * l_all
    rng = np.random.default_rng(4)
    picks = [(s, int(q)) for s in range(3)
             for q in rng.choice(params.shape[1], size=6, replace=False)]
    worst = 0.0
    gmax = np.abs(g_f).max()
    for s, q in picks:
        hq = 1e-5
        pp, pm = params.copy(), params.copy()
        pp[s, q] += hq
        pm[s, q] -= hq
        fd = (oracle_force_loss(ds, funcs, zprec, dims, pp, Ft, c)
              - oracle_force_loss(ds, funcs, zprec, dims, pm, Ft, c)) / (2 * hq)
        worst = max(worst, abs(fd - g_f[s, q]) / gmax)
    print(f"force-loss gradient vs oracle differences: {worst:.2e} of the largest component")
    assert worst <= 1e-6


def test_force_loss_fp32_gradient_and_training():
    cfg = synthetic.CONFIGS["C4"]
    ds = synthetic.generate(cfg, nstruct=8, forces=True)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = random_params(dims, 3, seed=2)
    zprec = O.zscore_stats(O.acsf(ds, funcs), ds)
    Ft = ds.meta["forces"]
    grads = {}
    for prec in (api.FP64, api.FP32):
        with gpu_ctx(prec, ds, funcs, zprec) as ctx:
            ctx.set_network(dims, "tanh", params)
            ctx.set_targets(ds)
            ctx.set_force_targets(0.1, Ft)
            grads[prec], _, _ = ctx.train_gradients("mse")
    err = max(float(np.linalg.norm(grads[api.FP32][s] - grads[api.FP64][s])
                    / np.linalg.norm(grads[api.FP64][s])) for s in range(3))
    print(f"C4 FP32 gradient of E + 0.1 F-MSE vs FP64: norm-wise {err:.2e}")
    assert err <= 1e-3
    with gpu_ctx(api.FP32, ds, funcs, zprec) as ctx:
        ctx.set_network(dims, "tanh", params)
        ctx.set_targets(ds)
        ctx.set_force_targets(0.1, Ft)
        ctx.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=100, linemin=True)
        hist = []
        for _ in range(12):
            ctx.train_iteration("mse")
            hist.append(ctx.last_losses())
    print("C4 force-loss L-BFGS (L_E, L_F): " + ", ".join(f"({a:.3e}, {b:.3e})" for a, b in hist))
    assert hist[-1][1] < hist[0][1]
    assert sum(hist[-1]) < sum(hist[0])
