"""The C++ host layer (fortnet_gb300/host): its HDF5 readers against the Python readers on the
reference's datasets and netstats (CPU, where the reference sources are available), and its
TAcsf / TBpnn / force-analysis / training classes on the GPU against the oracle."""

import glob
import json
import os
import subprocess

import numpy as np
import pytest

from fortnet_gb300 import build as B
from fortnet_gb300 import fnetdata, netstat
from fortnet_gb300.gfunctions import TYPE_CODES

from conftest import REFERENCE as REF
DATASETS = sorted(glob.glob(os.path.join(REF, "test", "prog", "fortnet", "datasets", "*.hdf5")))
NETSTATS = sorted(glob.glob(os.path.join(REF, "test", "prog", "fortnet", "prediction", "**",
                                         "fortnet.hdf5"), recursive=True))
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host():
    B.build_host()
    return B.HOST_RUN


def _dump(run, *files):
    res = subprocess.run([run, "--dump", *files], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    return json.loads(res.stdout)


@pytest.mark.skipif(not DATASETS, reason="reference datasets not available")
@pytest.mark.parametrize("path", DATASETS, ids=os.path.basename)
def test_cpp_dataset_reader_matches_python(host, path):
    got = _dump(host, path)
    ref = fnetdata.read_hdf_dataset(path)
    assert got["ndatapoints"] == ref.nstruct and got["ntotal"] == ref.ntot
    np.testing.assert_array_equal(got["atom_offsets"], ref.atom_offsets)
    np.testing.assert_array_equal(np.reshape(got["coords"], (-1, 3)), ref.coords)
    np.testing.assert_array_equal(got["atnum"], ref.atnum)
    np.testing.assert_array_equal(got["species"], ref.species)
    np.testing.assert_array_equal(got["periodic"], ref.periodic)
    np.testing.assert_array_equal(np.reshape(got["latvecs"], (-1, 9)), ref.latvecs)
    np.testing.assert_array_equal(got["weights"], ref.weights)
    np.testing.assert_array_equal(got["atomic_weights"], ref.atomic_weights)
    np.testing.assert_array_equal(np.ravel(got["global_targets"]), ref.global_targets.ravel())
    np.testing.assert_array_equal(np.ravel(got["atomic_targets"]), ref.atomic_targets.ravel())
    if ref.ext is not None:
        np.testing.assert_array_equal(np.ravel(got["ext"]), ref.ext.ravel())


@pytest.mark.skipif(not (DATASETS and NETSTATS), reason="reference netstats not available")
@pytest.mark.parametrize("path", NETSTATS[:12], ids=lambda p: os.path.relpath(p, REF))
def test_cpp_netstat_reader_matches_python(host, path):
    got = _dump(host, DATASETS[0], path)
    ref = netstat.read_netstat(path)
    gf = np.reshape(got["gfunctions"], (-1, 10)) if got["gfunctions"] else np.zeros((0, 10))
    assert len(gf) == len(ref.gfunctions)
    for row, g in zip(gf, ref.gfunctions):
        assert row[0] == TYPE_CODES[g.type]
        np.testing.assert_array_equal(row[1:7], [g.rcut, g.kappa, g.rs, g.eta, g.lam, g.xi])
        np.testing.assert_array_equal(row[7:], [g.atomid, g.z1, g.z2])
    if ref.zprec is not None:
        np.testing.assert_array_equal(got["zprec"], ref.zprec.ravel())
    np.testing.assert_array_equal(got["dims"], ref.dims)
    np.testing.assert_array_equal(got["net_atomic_numbers"], ref.atomic_numbers)
    np.testing.assert_array_equal(np.reshape(got["params"], ref.params.shape), ref.params)


@pytest.mark.gpu
def test_cpp_host_classes_match_oracle(host, tmp_path):
    """TAcsf / TBpnn / forceAnalysis / nTrain through the C++ host layer vs the oracle."""
    oracle_dir = os.path.join(HERE, "..", "oracle")
    subprocess.run(["make", "-C", oracle_dir], check=True, capture_output=True)
    exe = str(tmp_path / "host_parity")
    cmd = (["g++", "-o", exe] + B.host_flags()
           + ["-I", oracle_dir, os.path.join(HERE, "cpp", "host_parity.cpp"),
              "-L", os.path.join(oracle_dir, "_build"), "-loracle",
              "-Wl,-rpath," + os.path.abspath(os.path.join(oracle_dir, "_build"))]
           + B.host_link_flags())
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(run.stdout)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "ALL PASSED" in run.stdout
