"""The C-ABI library builds, loads and exports every entry point of include/*.h; its
host-side initialisation RNG reproduces the reference's RANLUX draws (no GPU needed)."""

import os
import re

import numpy as np

import oracle as O
from fortnet_gb300 import api

INCLUDE = os.path.join(os.path.dirname(__file__), "..", "include")
HEADERS = sorted(os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h"))


def declared_symbols():
    syms = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        syms |= set(re.findall(r"\b(fnetg_[a-z0-9_]+)\s*\(", text))
    return sorted(syms)


def test_library_exports_every_declared_symbol():
    lib = api.load()
    syms = declared_symbols()
    assert len(syms) > 30 and "fnetg_server_submit" in syms
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version():
    assert api.load().fnetg_abi_version() == 1


def test_nparams_matches_reference_count():
    # nBiases + nWeights of TNetwork_countParams (network.F90:126-142)
    for dims in ([8, 10, 10, 1], [96, 32, 32, 1], [168, 64, 64, 1], [3, 2]):
        d = np.asarray(dims, dtype=np.int32)
        n = api.load().fnetg_nparams(len(d), d.ctypes.data)
        ref = sum(dims) + sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1)) + dims[-1]
        assert n == ref


def test_ranlux_stream_matches_oracle():
    for seed in (1, 123456, 2**31 - 1):
        a = api.Rng(seed).uniform(5000)
        b = O.Ranlux(seed).get(5000)
        assert np.array_equal(a, b)


def test_initial_parameters_match_oracle():
    for dims, nsp in (([18, 3, 3, 1], 2), ([96, 32, 32, 1], 2), ([8, 10, 10, 1], 1)):
        a = api.Rng(123456).init_params(dims, nsp)
        b = O.Ranlux(123456).init_bpnn(dims, "tanh", nsp)
        assert np.array_equal(a, b)


def test_shuffle_matches_oracle():
    r1, r2 = api.Rng(99), O.Ranlux(99)
    x = np.arange(1, 101, dtype=np.int32)
    for _ in range(3):
        a = r1.shuffle(x)
        b = r2.shuffle(x)
        assert np.array_equal(a, b)
        x = a


def test_no_gpu_context_creation_fails_cleanly():
    import ctypes as C

    lib = api.load()
    h = C.c_void_p()
    rc = lib.fnetg_create(C.byref(h), 16, 0)  # invalid precision
    assert rc == -1 and not h.value


def test_caller_output_buffers_are_checked_on_the_host():
    """predict/forces accept caller-owned buffers only as writeable, C-contiguous float64 of
    the result's shape (checked before the library is called)."""
    good = np.zeros((5, 1, 3))
    api._check_out(good, (5, 1, 3))
    readonly = np.zeros((5, 1, 3))
    readonly.flags.writeable = False
    frombuf = np.frombuffer(bytes(5 * 3 * 8), dtype=np.float64).reshape(5, 1, 3)
    for bad in (np.zeros((5, 3)), np.zeros((5, 1, 3), dtype=np.float32),
                np.zeros((5, 1, 6))[:, :, ::2], readonly, frombuf):
        try:
            api._check_out(bad, (5, 1, 3))
        except ValueError:
            continue
        raise AssertionError("accepted %r" % (bad.shape,))
