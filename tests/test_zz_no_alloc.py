"""fnetg_acsf_zscore_stats_noalloc against the allocating entry point fnetg_acsf_zscore.

The no-alloc call reads its weights from and writes its statistics to device memory (torch
tensors here, used only as device buffers).  Two calls in a row must give the same statistics
as each other and as fnetg_acsf_zscore(..., compute = 1) on the same features.
"""

import ctypes as C

import numpy as np
import pytest

from fortnet_gb300 import api, synthetic

pytestmark = pytest.mark.gpu


def _lib_fn(ctx):
    fn = ctx.lib.fnetg_acsf_zscore_stats_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


def _features_ctx(precision, ds, funcs):
    ctx = api.Context(precision)
    ctx.upload(ds)
    ctx.set_species(ds.species)
    ctx.set_gfunctions(funcs)
    ctx.acsf(download=False)
    return ctx


@pytest.mark.parametrize("precision", [api.FP64, api.FP32])
@pytest.mark.parametrize("weighted", [False, True])
def test_noalloc_stats_match_allocating_entry_point(precision, weighted):
    torch = pytest.importorskip("torch")
    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=24, targets=False)
    funcs = synthetic.gfunctions(cfg)
    ng = len(funcs)
    w = np.random.default_rng(7).integers(1, 4, size=ds.nstruct).astype(np.int32)
    with _features_ctx(precision, ds, funcs) as ctx:
        fn = _lib_fn(ctx)
        d_w = torch.tensor(w, dtype=torch.int32, device="cuda") if weighted else None
        outs = []
        for _ in range(2):
            d_z = torch.full((2 * ng,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc = fn(ctx.h, d_w.data_ptr() if weighted else None, d_z.data_ptr())
            assert rc == 0, ctx.lib.fnetg_last_error(ctx.h)
            ctx.synchronize()
            outs.append(d_z.cpu().numpy().reshape(2, ng))
        ref = ctx.zscore(weights=w if weighted else None)
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.all(np.isfinite(outs[0]))
    np.testing.assert_allclose(outs[0], ref, rtol=1e-13, atol=0.0)


def test_noalloc_stats_rejects_missing_features():
    torch = pytest.importorskip("torch")
    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=2, targets=False)
    with api.Context(api.FP32) as ctx:
        ctx.upload(ds)
        ctx.set_species(ds.species)
        ctx.set_gfunctions(synthetic.gfunctions(cfg))
        d_z = torch.zeros(2 * 96, dtype=torch.float64, device="cuda")
        assert _lib_fn(ctx)(ctx.h, None, d_z.data_ptr()) == -1  # FNETG_E_INVALID


def _wide_ctx(ng, nstruct=3):
    """A context whose network inputs are ng uploaded columns (G2 functions set only to fix
    the column count; the features themselves come from fnetg_set_features)."""
    from fortnet_gb300.gfunctions import GFunction

    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=nstruct, targets=False)
    funcs = [GFunction("g2", 8.0, eta=0.01 + 1e-4 * k) for k in range(ng)]
    ctx = api.Context(api.FP64)
    ctx.upload(ds)
    ctx.set_species(ds.species)
    ctx.set_gfunctions(funcs)
    feats = np.random.default_rng(ng).normal(3.0, 0.5, size=(ds.ntot, ng))
    ctx.set_features(feats)
    return ctx, ds


def test_noalloc_stats_at_the_column_limit():
    """nG = 4095, the largest the fixed scratch array takes: at most 32 chunks of 4096 partial
    columns, so with ~9,600 atoms every chunk holds more than the minimum 256 atoms.  It matches
    the allocating path; nG = 4096 is refused with FNETG_E_UNSUPPORTED."""
    torch = pytest.importorskip("torch")
    ctx, ds = _wide_ctx(4095, nstruct=60)
    assert ds.ntot > 32 * 256
    with ctx:
        d_z = torch.full((2 * 4095,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = _lib_fn(ctx)(ctx.h, None, d_z.data_ptr())
        assert rc == 0, ctx.lib.fnetg_last_error(ctx.h)
        ctx.synchronize()
        got = d_z.cpu().numpy().reshape(2, 4095)
        ref = ctx.zscore()
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=0.0)
    ctx, _ = _wide_ctx(4096, nstruct=1)
    with ctx:
        d_z = torch.zeros(2 * 4096, dtype=torch.float64, device="cuda")
        assert _lib_fn(ctx)(ctx.h, None, d_z.data_ptr()) == -7  # FNETG_E_UNSUPPORTED


def test_noalloc_stats_refuse_standardised_features():
    """After fnetg_acsf_zscore the device features are standardised; the statistics of the
    raw features can no longer be formed and the call is refused (FNETG_E_INVALID)."""
    torch = pytest.importorskip("torch")
    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=4, targets=False)
    funcs = synthetic.gfunctions(cfg)
    with _features_ctx(api.FP32, ds, funcs) as ctx:
        ctx.zscore()
        d_z = torch.zeros(2 * len(funcs), dtype=torch.float64, device="cuda")
        assert _lib_fn(ctx)(ctx.h, None, d_z.data_ptr()) == -1


def test_noalloc_stats_zero_weight_total_is_not_finite():
    """The weights are read on the device and not checked: an all-zero weight vector gives the
    documented non-finite statistics (0/0) instead of an error code."""
    torch = pytest.importorskip("torch")
    cfg = synthetic.CONFIGS["C2"]
    ds = synthetic.generate(cfg, nstruct=4, targets=False)
    funcs = synthetic.gfunctions(cfg)
    with _features_ctx(api.FP64, ds, funcs) as ctx:
        d_w = torch.zeros(ds.nstruct, dtype=torch.int32, device="cuda")
        d_z = torch.zeros(2 * len(funcs), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert _lib_fn(ctx)(ctx.h, d_w.data_ptr(), d_z.data_ptr()) == 0
        ctx.synchronize()
        assert not np.any(np.isfinite(d_z.cpu().numpy()))
