"""The socket-driven prediction loop (fnetg_ipi: prg_fnet/fortnet.F90:126-169 over the GPU
prediction service) against an i-PI server: energies and forces of every geometry the server
sends equal the oracle's, and the virial is the reference's placeholder (cell volume times
ones).  The model reaches the program as a netstat file written by the host layer."""

import os
import subprocess

import numpy as np
import pytest

import oracle as O
from fortnet_gb300 import api, build as B, synthetic
from ipi_server import IpiServer
from test_h5_writers import write_model

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
C5 = synthetic.CONFIGS["C5"]


@pytest.fixture(scope="module")
def writer(tmp_path_factory):
    B.build_host()
    exe = str(tmp_path_factory.mktemp("ipi_gpu") / "h5_writers")
    cmd = (["g++", "-o", exe] + B.host_flags() + [os.path.join(HERE, "cpp", "h5_writers.cpp")]
           + B.host_link_flags())
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_socket_driver_matches_oracle(writer, tmp_path, precision):
    cfg = synthetic.Config("ipi", 3, (24, 24), "fixed", C5.atomic_numbers, C5.ratios, C5.rcut,
                           C5.n_g2, C5.g2_eta, C5.g5, C5.hidden, 91)
    ds = synthetic.generate(cfg, targets=False)
    # one atom list for every step (the driver's AtomicNumbers): structure 0's
    n = int(ds.natoms[0])
    atnum = ds.atnum[:n]
    for s in range(ds.nstruct):
        a = ds.atom_offsets[s]
        ds.atnum[a:a + n] = atnum
        ds.species[a:a + n] = ds.species[:n]
    funcs = synthetic.gfunctions(C5)
    dims = [len(funcs), 16, 1]
    params = 0.1 * api.Rng(7).init_params(dims, 3)
    vals = O.acsf(ds, funcs)
    zprec = O.zscore_stats(vals, ds)
    feats = O.zscore_apply(vals, zprec)
    atomic = O.predict(dims, "tanh", params, feats, ds.species)
    jac = O.jacobian(dims, "tanh", params, feats, ds.species)
    f_orc = O.forces(ds, funcs, zprec, jac, physical=True)[:, 0, :]
    model, ns = str(tmp_path / "model.bin"), str(tmp_path / "netstat.hdf5")
    write_model(model, C5.atomic_numbers, funcs, zprec, dims, "tanh", 1, 0, params)
    res = subprocess.run([writer, "netstat", model, ns], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    srv = IpiServer()
    cmd = [B.HOST_IPI, ns, "--atomic-numbers", ",".join(str(int(z)) for z in atnum), "--periodic",
           "--host", "127.0.0.1", "--port", str(srv.port), "--max-steps", "-1"]
    if precision == "fp32":
        cmd.append("--fp32")
    proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    got = []
    try:
        srv.accept()
        for s in range(ds.nstruct):
            a = ds.atom_offsets[s]
            h = ds.latvecs[s].reshape(3, 3).T  # columns are the lattice vectors
            got.append(srv.evaluate(ds.coords[a:a + n], h))
        srv.exit()
        stdout, stderr = proc.communicate(timeout=120)
    finally:
        if proc.poll() is None:
            proc.kill()
        srv.close()
    assert proc.returncode == 0, stderr
    assert int(stdout.strip()) == ds.nstruct
    e_tol, f_tol = (1e-10, 1e-9) if precision == "fp64" else (1e-5, 1e-4)
    for s, (e, f, vir, extra) in enumerate(got):
        a = ds.atom_offsets[s]
        e_ref = float(np.sum(atomic[a:a + n, 0]))
        scale = abs(e_ref) if precision == "fp64" else float(np.sum(np.abs(atomic[a:a + n, 0])))
        assert abs(e - e_ref) <= e_tol * scale
        fmax = float(np.max(np.abs(f_orc[a:a + n])))
        assert np.max(np.abs(f - f_orc[a:a + n])) <= f_tol * fmax
        vol = abs(np.linalg.det(ds.latvecs[s].reshape(3, 3)))
        np.testing.assert_allclose(vir, np.full((3, 3), vol), rtol=1e-14)
        assert extra == ""
