"""HDF5 writers of the C++ host layer (netstat: lib_io/netstat.F90, acsf.F90:1759-1906,
bpnn.F90:1062-1140; fnetout: lib_io/fnetout.F90:33-158).  Every netstat and fnetout file of
the reference's regression suite is read, written back through the writers, and read again:
the trees must be identical.  Plus a written model read back through both readers."""

import glob
import os
import subprocess

import numpy as np
import pytest

from fortnet_gb300 import api, build as B, hdf5lite, netstat
from fortnet_gb300.gfunctions import GFUNC_DTYPE, GFunction, pack
from h5tree import assert_same_tree

from conftest import REFERENCE as REF
NETSTATS = sorted(glob.glob(os.path.join(REF, "test", "prog", "fortnet", "**", "*fortnet.hdf5"),
                            recursive=True))
FNETOUTS = sorted(glob.glob(os.path.join(REF, "test", "prog", "fortnet", "**", "_fnetout.hdf5"),
                            recursive=True))
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    B.build_host()
    exe = str(tmp_path_factory.mktemp("h5w") / "h5_writers")
    cmd = (["g++", "-o", exe] + B.host_flags() + [os.path.join(HERE, "cpp", "h5_writers.cpp")]
           + B.host_link_flags())
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def write_model(path, atomic_numbers, funcs, zprec, dims, activation, nglobal, natomic, params,
                ext_indices=None):
    """The model file read by tests/cpp/h5_writers.cpp (zprec None: no z-score statistics)."""
    g = pack(funcs) if len(funcs) else np.zeros(0, dtype=GFUNC_DTYPE)
    with open(path, "wb") as fh:
        fh.write(np.int32(len(atomic_numbers)).tobytes())
        fh.write(np.asarray(atomic_numbers, dtype="<i4").tobytes())
        fh.write(np.int32(len(g)).tobytes())
        fh.write(g.tobytes())
        fh.write(np.int32(0 if zprec is None else 1).tobytes())
        if zprec is not None:
            fh.write(np.asarray(zprec, dtype="<f8").reshape(-1).tobytes())
        fh.write(np.int32(len(dims)).tobytes())
        fh.write(np.asarray(dims, dtype="<i4").tobytes())
        fh.write(np.int32(api.ACT[activation]).tobytes())
        fh.write(np.int32(nglobal).tobytes())
        fh.write(np.int32(natomic).tobytes())
        fh.write(np.asarray(params, dtype="<f8").reshape(-1).tobytes())
        ext = np.zeros(0, dtype="<i4") if ext_indices is None else np.asarray(ext_indices, "<i4")
        fh.write(np.int32(len(ext)).tobytes())
        fh.write(ext.tobytes())


@pytest.mark.skipif(not NETSTATS, reason="reference netstat files not available")
@pytest.mark.parametrize("path", NETSTATS[::7], ids=lambda p: os.path.relpath(p, REF))
def test_netstat_round_trip_is_identical(path, tmp_path):
    out = str(tmp_path / "netstat.hdf5")
    res = subprocess.run([B.HOST_RUN, "--copy-netstat", path, out], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert_same_tree(hdf5lite.read(path), hdf5lite.read(out))


@pytest.mark.skipif(not NETSTATS, reason="reference netstat files not available")
def test_every_reference_netstat_round_trips(tmp_path):
    out = str(tmp_path / "netstat.hdf5")
    for path in NETSTATS:
        res = subprocess.run([B.HOST_RUN, "--copy-netstat", path, out], capture_output=True,
                             text=True)
        assert res.returncode == 0, (path, res.stderr)
        assert_same_tree(hdf5lite.read(path), hdf5lite.read(out), os.path.relpath(path, REF))


def drop_absent_targets(tree):
    """The regression fixtures were written by an earlier writeFnetout that stored both target
    datasets in validate mode, as placeholders when a kind of target is absent (an empty
    0 x 0 'atomictargets', a one-element 'globaltargets'); the current fnetout.F90:106-121
    writes each only when that kind of target exists, and so does the writer here."""
    out = tree["fnetout/output"]
    for key, count in (("atomictargets", "natomictargets"), ("globaltargets", "nglobaltargets")):
        if int(out.attrs[count][0]) == 0:
            for dp in out.children.values():
                dp.children.pop(key, None)
    return tree


@pytest.mark.skipif(not FNETOUTS, reason="reference fnetout files not available")
def test_every_reference_fnetout_round_trips(tool, tmp_path):
    out = str(tmp_path / "fnetout.hdf5")
    for path in FNETOUTS:
        res = subprocess.run([tool, "fnetout", path, out], capture_output=True, text=True)
        assert res.returncode == 0, (path, res.stderr)
        assert_same_tree(drop_absent_targets(hdf5lite.read(path)), hdf5lite.read(out),
                         os.path.relpath(path, REF))


def test_written_model_reads_back(tool, tmp_path):
    """A model with every G-function type, z-score statistics, three species and a deep
    network (more than 8 members per group: several symbol-table nodes) through the writer
    and both readers."""
    rng = np.random.default_rng(3)
    z = [1, 6, 8]
    funcs = []
    for k in range(40):
        t = ["g1", "g2", "g3", "g4", "g5"][k % 5]
        funcs.append(GFunction(t, 7.5 + 0.1 * k, kappa=0.3 if t == "g3" else 0.0,
                               rs=0.5 if t == "g2" else 0.0,
                               eta=0.01 * (k + 1) if t in ("g2", "g4", "g5") else 0.0,
                               lam=(-1.0 if k % 2 else 1.0) if t in ("g4", "g5") else 0.0,
                               xi=float(1 + k % 4) if t in ("g4", "g5") else 0.0, atomid=k % 2,
                               z1=z[k % 3], z2=z[(k + 1) % 3] if t in ("g4", "g5") else 0))
    dims = [40, 12, 9, 7, 5, 3, 2]
    nparams = sum(dims) + sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1)) + dims[-1]
    params = rng.normal(size=(3, nparams))
    # entries the file does not hold (and the networks never use): the output layer's ww and
    # the input layer's bb of the serialised order (network.F90:397-427)
    nw = sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    params[:, nw:nw + dims[-1] + dims[0]] = 0.0
    zprec = np.concatenate([rng.normal(size=40), rng.uniform(0.1, 2.0, size=40)])
    model = str(tmp_path / "model.bin")
    out = str(tmp_path / "netstat.hdf5")
    write_model(model, z, funcs, zprec, dims, "lrelu", 2, 0, params)
    res = subprocess.run([tool, "netstat", model, out], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    ns = netstat.read_netstat(out)
    assert list(ns.atomic_numbers) == z and list(ns.dims) == dims
    np.testing.assert_array_equal(ns.params, params)
    np.testing.assert_array_equal(np.asarray(ns.zprec).reshape(-1), zprec)
    for a, b in zip(ns.gfunctions, funcs):
        assert (a.type, a.rcut, a.atomid, a.z1, a.z2) == (b.type, b.rcut, b.atomid, b.z1, b.z2)
        assert (a.kappa, a.rs, a.eta, a.lam, a.xi) == (b.kappa, b.rs, b.eta, b.lam, b.xi)
    # the C++ reader sees the same model: copy it once more and compare the trees
    out2 = str(tmp_path / "netstat2.hdf5")
    res = subprocess.run([B.HOST_RUN, "--copy-netstat", out, out2], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert_same_tree(hdf5lite.read(out), hdf5lite.read(out2))
