"""The batched mixed-precision form (include/fnetg_batch.h): tensor-core BF16 layer GEMMs with
FP32 accumulation, FP64 gradient sums and steepest-descent steps per mini-batch.

* forward: against an emulation of the same BF16 roundings in FP64 (features, weights and
  first-layer activations rounded to BF16 where the kernel rounds them) within 1e-2 of the
  output scale (the kernel's tanh is the hardware approximation, ~5e-4 relative), which pins the
  tensor-core data layout; and against the FP64 oracle, error printed;
* mini-batch gradients: against the FP64 oracle's gradient over the mini-batch's structures,
  norm-wise within 3e-2 per sub-network (BF16 operands, 8-bit significands);
* one epoch of per-mini-batch steepest descent: against the oracle's sequence of mini-batch
  gradients and SD steps, parameters' displacement within 5e-2 of its norm;
* prediction of every structure in one launch, and epochs that lower the loss.
Configurations: C2 (96-32-32-1, two species), C3 (168-64-64-1, 176 padded inputs: two
128-input tiles of the first-layer gradient) and C4 (66-64-64-1), small samples.
"""

import numpy as np
import pytest

import oracle as O
from fortnet_gb300 import api, synthetic

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def layout(dims):
    return synthetic.param_layout(dims)


def random_params(dims, nsp, seed):
    return synthetic.normal_params(dims, nsp, seed)


def unpack(p, dims):
    woff, boff, _ = layout(dims)
    nf, h1, h2 = dims[0], dims[1], dims[2]
    W0 = p[woff[0]:woff[0] + nf * h1].reshape(h1, nf).T
    W1 = p[woff[1]:woff[1] + h1 * h2].reshape(h2, h1).T
    w2 = p[woff[2]:woff[2] + h2]
    return W0, p[boff[1]:boff[1] + h1], W1, p[boff[2]:boff[2] + h2], w2, p[boff[3]]


def emulate_forward(feats, species, params, dims):
    """The tensor-core forward's roundings in FP64: BF16 features, weights, biases and first
    activations; FP32-exact output layer."""
    y = np.zeros(len(feats))
    for s in range(params.shape[0]):
        m = species == s
        W0, b1, W1, b2, w2, b3 = unpack(params[s], dims)
        z1 = bf16(feats[m]) @ bf16(W0) + bf16(b1)
        a1 = bf16(np.tanh(z1))
        z2 = a1 @ bf16(W1) + bf16(b2)
        y[m] = np.tanh(z2) @ w2.astype(np.float32).astype(np.float64) + float(np.float32(b3))
    return y


def subset(ds, s0, s1):
    from fortnet_gb300.fnetdata import Dataset

    a0, a1 = ds.atom_offsets[s0], ds.atom_offsets[s1]
    return Dataset(atom_offsets=ds.atom_offsets[s0:s1 + 1] - a0, coords=ds.coords[a0:a1],
                   atnum=ds.atnum[a0:a1], species=ds.species[a0:a1],
                   periodic=ds.periodic[s0:s1], latvecs=ds.latvecs[s0:s1],
                   atomic_numbers=ds.atomic_numbers, weights=ds.weights[s0:s1],
                   atomic_weights=ds.atomic_weights[a0:a1],
                   global_targets=ds.global_targets[s0:s1], atomic_targets=ds.atomic_targets[a0:a1])


def setup(cfg_name, nstruct, batch, seed=5):
    cfg = synthetic.CONFIGS[cfg_name]
    ds = synthetic.generate(cfg, nstruct=nstruct)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = random_params(dims, len(cfg.atomic_numbers), seed)
    ctx = api.Context(api.FP32)
    ctx.upload(ds)
    ctx.set_species(ds.species)
    ctx.set_gfunctions(funcs)
    ctx.acsf(download=False)
    ctx.zscore(weights=ds.weights)
    feats = ctx.features()
    ctx.set_network(dims, "tanh", params)
    ctx.set_targets(ds)
    ctx.batch_setup(batch)
    return ctx, ds, dims, params, feats


CASES = [("C2", 12, 5), ("C3", 40, 16), ("C4", 12, 5)]


@pytest.mark.parametrize("cfg_name,nstruct,batch", CASES)
def test_batch_forward_matches_bf16_emulation_and_oracle(cfg_name, nstruct, batch):
    ctx, ds, dims, params, feats = setup(cfg_name, nstruct, batch)
    with ctx:
        at, gl = ctx.batch_predict()
    emu = emulate_forward(feats, ds.species, params, dims)
    ref = O.predict(dims, "tanh", params, feats, ds.species)[:, 0]
    scale = np.abs(ref).mean()
    err_emu = float(np.max(np.abs(at - emu)) / scale)
    err64 = float(np.max(np.abs(at - ref)) / scale)
    e_ref = np.add.reduceat(ref, ds.atom_offsets[:-1])
    e_err = float(np.max(np.abs(gl[:, 0] - e_ref) / np.abs(e_ref)))
    print(f"{cfg_name} BF16 forward: vs emulation {err_emu:.2e}, vs FP64 {err64:.2e} of the "
          f"mean |output|, structure energies vs FP64 {e_err:.2e}")
    np.testing.assert_allclose(gl[:, 0], np.add.reduceat(at, ds.atom_offsets[:-1]), rtol=1e-12)
    assert err_emu <= 1e-2
    assert err64 <= 5e-2


@pytest.mark.parametrize("cfg_name,nstruct,batch", CASES)
def test_batch_gradients_match_oracle(cfg_name, nstruct, batch):
    ctx, ds, dims, params, feats = setup(cfg_name, nstruct, batch)
    errs = []
    with ctx:
        nb = ctx.batch_info()["batches"]
        for k in range(nb):
            s0, s1 = k * batch, min(ds.nstruct, (k + 1) * batch)
            sub = subset(ds, s0, s1)
            a0, a1 = ds.atom_offsets[s0], ds.atom_offsets[s1]
            g, at = ctx.batch_gradients(k, natoms=int(a1 - a0))
            ref, pred = O.train_gradients(dims, "tanh", params, feats[a0:a1], sub)
            for s in range(ref.shape[0]):
                errs.append(float(np.linalg.norm(g[s] - ref[s]) / np.linalg.norm(ref[s])))
            assert np.max(np.abs(at - pred[:, 0])) <= 5e-2 * np.abs(pred).mean()
    print(f"{cfg_name} BF16 mini-batch gradients vs FP64: worst norm-wise {max(errs):.2e}")
    assert max(errs) <= 3e-2


def test_batch_epoch_matches_oracle_sd_sequence():
    cfg_name, nstruct, batch = "C4", 12, 5
    ctx, ds, dims, params0, feats = setup(cfg_name, nstruct, batch)
    lr = 1e-3
    p = params0.copy()
    for s0 in range(0, ds.nstruct, batch):
        s1 = min(ds.nstruct, s0 + batch)
        sub = subset(ds, s0, s1)
        a0, a1 = ds.atom_offsets[s0], ds.atom_offsets[s1]
        dd, _ = O.train_gradients(dims, "tanh", p, feats[a0:a1], sub)
        g, _ = O.update_prepare(dims, "tanh", p, dd, 0.0, 0.0, float(sub.weights.sum()))
        p = np.stack([O.SteepestDescent(p[s], 1e-30, 1e4, lr).next(0.0, g[s])[0]
                      for s in range(p.shape[0])])
    with ctx:
        ctx.batch_epoch("mse", lr, 1e4)
        got = ctx.params()
    err = float(np.linalg.norm(got - p) / np.linalg.norm(p - params0))
    print(f"C4 one BF16 epoch of mini-batch SD vs FP64: displacement error {err:.2e}")
    assert err <= 5e-2


def test_batch_epochs_lower_the_loss_and_sync_to_the_plain_form():
    ctx, ds, dims, params0, feats = setup("C2", 16, 4)
    with ctx:
        losses = [ctx.batch_epoch("mse", 2e-3, 1e4) for _ in range(6)]
        info = ctx.batch_info()
        ctx.batch_sync_params()
        _, e_plain = ctx.predict(atomic=False)
        _, e_tc = ctx.batch_predict(atomic=False)
        p = ctx.params()
    print(f"C2 epoch losses {['%.3e' % l for l in losses]}, tuned CTAs {info}")
    assert losses[-1] < losses[0]
    assert info["ctas_forward"] > 0 and info["ctas_train"] > 0
    # the plain FP32 form on the trained FP64 parameters agrees with the BF16 form
    ref = O.predict(dims, "tanh", p, feats, ds.species)[:, 0]
    e_ref = np.add.reduceat(ref, ds.atom_offsets[:-1])
    assert np.max(np.abs(e_plain[:, 0] - e_ref) / np.abs(e_ref)) <= 1e-5
    assert np.max(np.abs(e_tc[:, 0] - e_ref) / np.abs(e_ref)) <= 5e-2


@pytest.mark.parametrize("force_weight", [0.0, 0.1])
def test_tensor_core_training_gradients_match_fp64(force_weight):
    """The precision form's full-batch gradient (fnetg_batch_train_bf16): BF16 tensor-core
    forward, input Jacobian and reverse passes, FP32 forces and dG/dR contraction, FP64 sums;
    against the FP64 plain kernels' gradient of the same loss (energies, or energies + 0.1 x
    force MSE), norm-wise within 5e-2 per sub-network; then L-BFGS iterations on it lower the
    loss."""
    cfg = synthetic.CONFIGS["C4"]
    ds = synthetic.generate(cfg, nstruct=10, forces=True)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = random_params(dims, 3, seed=4)
    zprec = O.zscore_stats(O.acsf(ds, funcs), ds)

    def ctx_for(prec):
        c = api.Context(prec)
        c.upload(ds)
        c.set_species(ds.species)
        c.set_gfunctions(funcs)
        c.acsf(download=False)
        c.zscore(zprec=zprec)
        c.set_network(dims, "tanh", params)
        c.set_targets(ds)
        if force_weight > 0:
            c.set_force_targets(force_weight, ds.meta["forces"])
        return c

    with ctx_for(api.FP64) as c:
        g64, l64, _ = c.train_gradients("mse")
    with ctx_for(api.FP32) as c:
        c.batch_setup(4)
        c.batch_train_bf16(True)
        g16, l16, _ = c.train_gradients("mse")
        c.optimizer_init("lbfgs", 1e-20, 1e-6, 1e4, memory=100, linemin=True)
        hist = [c.train_iteration("mse")[0] for _ in range(8)]
    err = max(float(np.linalg.norm(g16[s] - g64[s]) / np.linalg.norm(g64[s])) for s in range(3))
    print(f"C4 BF16 gradient (force weight {force_weight}) vs FP64: norm-wise {err:.2e}, loss "
          f"{abs(l16 - l64) / l64:.2e}; L-BFGS losses {['%.3e' % h for h in hist]}")
    assert err <= 5e-2
    assert abs(l16 - l64) <= 2e-2 * l64
    assert hist[-1] < hist[0]


@pytest.mark.parametrize("force_weight", [0.0, 0.1])
def test_full_batch_gradient_over_many_small_mini_batches(force_weight):
    """A full-batch tensor-core launch over a plan of many small mini-batches: with two
    structures per mini-batch (a handful of tiles each) and about 600 tiles over one CTA per SM,
    most CTAs meet a species again after other species, in the next mini-batch, and must add to
    the gradient partial they stored for it before.  Energy loss: equal to the sum of the
    per-mini-batch gradients (the same BF16 tile arithmetic, FP32 sums grouped differently:
    norm-wise 1e-4); with the force term: within 5e-2 of the FP64 plain kernels, as on few
    tiles."""
    cfg = synthetic.CONFIGS["C4"]
    ds = synthetic.generate(cfg, nstruct=200, forces=force_weight > 0)
    funcs = synthetic.gfunctions(cfg)
    dims = synthetic.network_dims(cfg)
    params = random_params(dims, 3, seed=5)

    def ctx_for(prec, zprec=None):
        c = api.Context(prec)
        c.upload(ds)
        c.set_species(ds.species)
        c.set_gfunctions(funcs)
        c.acsf(download=False)
        z = c.zscore(zprec=zprec)
        c.set_network(dims, "tanh", params)
        c.set_targets(ds)
        if force_weight > 0:
            c.set_force_targets(force_weight, ds.meta["forces"])
        return c, z

    c, zprec = ctx_for(api.FP64)
    with c:
        g64, _, _ = c.train_gradients("mse")
    c, _ = ctx_for(api.FP32, zprec)
    with c:
        c.batch_setup(2)
        info = c.batch_info()
        nbatch, ntiles = info["batches"], info["tiles"]
        assert ntiles >= 4 * 152 and nbatch == 100
        c.batch_train_bf16(True)
        g16, _, _ = c.train_gradients("mse")
        if force_weight == 0:
            gsum = np.zeros_like(g16)
            for k in range(nbatch):
                gsum += c.batch_gradients(k)[0]
    err64 = max(float(np.linalg.norm(g16[s] - g64[s]) / np.linalg.norm(g64[s]))
                for s in range(3))
    msg = f"full-batch BF16 gradient over {ntiles} tiles vs FP64: {err64:.2e}"
    if force_weight == 0:
        errsum = max(float(np.linalg.norm(g16[s] - gsum[s]) / np.linalg.norm(gsum[s]))
                     for s in range(3))
        msg += f"; vs the sum of {nbatch} mini-batch gradients: {errsum:.2e}"
        assert errsum <= 1e-4
    print(msg)
    assert err64 <= 5e-2
