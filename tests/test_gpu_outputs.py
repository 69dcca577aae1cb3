"""Output paths of the public API: per-structure sums computed on the device equal the host's
atom-order sums bit for bit, and caller-owned (pinned) output buffers receive exactly what
freshly allocated ones do."""

import dataclasses

import numpy as np
import pytest
import torch

from fortnet_gb300 import api, synthetic

pytestmark = pytest.mark.gpu

C4 = synthetic.CONFIGS["C4"]


@pytest.mark.parametrize("precision", [api.FP32, api.FP64])
def test_device_sums_and_caller_buffers(precision):
    ds = synthetic.generate(C4, nstruct=12, targets=False)
    funcs = synthetic.gfunctions(C4)
    dims = synthetic.network_dims(C4)
    params = api.Rng(11).init_params(dims, len(C4.atomic_numbers))
    with api.Context(precision) as ctx:
        ctx.upload(ds)
        ctx.set_species(ds.species)
        ctx.set_gfunctions(funcs)
        ctx.neighbors()
        ctx.acsf(download=False)
        ctx.zscore(weights=ds.weights)
        ctx.set_network(dims, "tanh", 0.1 * params)
        at, gl = ctx.predict()
        # host sums of the atomic outputs in atom order, as the reference sums them
        ref = np.array([[sum_in_order(at[a:b, o]) for o in range(at.shape[1])]
                        for a, b in zip(ds.atom_offsets[:-1], ds.atom_offsets[1:])])
        np.testing.assert_array_equal(gl, ref)
        # sums only, on the device, into a pinned buffer: the same bits
        g_pin = torch.empty(gl.shape, dtype=torch.float64, pin_memory=True).numpy()
        none, g2 = ctx.predict(atomic=False, out_global=g_pin)
        assert none is None and g2 is g_pin
        np.testing.assert_array_equal(g_pin, gl)
        # atomic outputs into a caller buffer
        a_pin = torch.empty(at.shape, dtype=torch.float64, pin_memory=True).numpy()
        a2, g3 = ctx.predict(out_atomic=a_pin)
        assert a2 is a_pin
        np.testing.assert_array_equal(a_pin, at)
        np.testing.assert_array_equal(g3, gl)
        # forces into a caller buffer; FP32 contexts accumulate in another order per call
        f = ctx.forces()
        f_pin = torch.empty(f.shape, dtype=torch.float64, pin_memory=True).numpy()
        assert ctx.forces(out=f_pin) is f_pin
        fscale = float(np.max(np.abs(f)))
        tol = 1e-12 if precision == api.FP64 else 1e-6
        np.testing.assert_allclose(f_pin, f, rtol=0.0, atol=tol * fscale)
        # wrong buffers are refused before any copy
        with pytest.raises(ValueError):
            ctx.forces(out=np.zeros((ds.ntot, 3)))
        with pytest.raises(ValueError):
            ctx.predict(atomic=False, out_global=np.zeros(gl.shape, dtype=np.float32))


def sum_in_order(v):
    acc = 0.0
    for x in v:
        acc += float(x)
    return acc


def test_update_coords_refuses_non_finite_and_keeps_the_context():
    """fnetg_update_coords checks the new coordinates on the device before they replace the
    context's: a NaN is refused with FNETG_E_GEOMETRY and the previous geometry (and its pair
    list) stays; finite moved coordinates are taken."""
    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=6, targets=False)
    with api.Context(api.FP32) as ctx:
        ctx.upload(ds)
        ctx.set_species(ds.species)
        ctx.set_gfunctions(synthetic.gfunctions(cfg))
        p0 = ctx.neighbors()
        off0, j0, _, _ = ctx.get_neighbors()
        bad = ds.coords.copy()
        bad[len(bad) // 2, 1] = np.nan
        with pytest.raises(api.FnetgError) as err:
            ctx.update_coords(bad)
        assert err.value.code == -6
        assert ctx.neighbors() == p0
        off1, j1, _, _ = ctx.get_neighbors()
        assert np.array_equal(off0, off1) and np.array_equal(j0, j1)
        moved = ds.coords * 1.05
        ctx.update_coords(moved)
        ctx.neighbors()
        off2, j2, _, _ = ctx.get_neighbors()
    fresh = dataclasses.replace(ds, coords=moved)
    with api.Context(api.FP32) as ctx:
        ctx.upload(fresh)
        ctx.set_species(ds.species)
        ctx.set_gfunctions(synthetic.gfunctions(cfg))
        ctx.neighbors()
        off3, j3, _, _ = ctx.get_neighbors()
    assert np.array_equal(off2, off3) and np.array_equal(j2, j3)
