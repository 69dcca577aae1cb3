"""The i-PI socket client of the C++ host layer (lib_io/ipisocket.F90 semantics): message
sequence, byte layout of cell / positions / forces / virial, EXIT handling, TCP and UNIX
sockets.  The client runs a host-side toy model, so no GPU is needed."""

import os
import subprocess

import numpy as np
import pytest

from fortnet_gb300 import build as B
from ipi_server import IpiServer

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    B.build_host()
    exe = str(tmp_path_factory.mktemp("ipi") / "ipi_protocol")
    cmd = (["g++", "-o", exe] + B.host_flags() + [os.path.join(HERE, "cpp", "ipi_protocol.cpp")]
           + B.host_link_flags())
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def run_session(client, server, args, geometries):
    proc = subprocess.Popen([client] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                            text=True)
    out = []
    try:
        server.accept()
        for pos, h in geometries:
            out.append(server.evaluate(pos, h))
        server.exit()
        stdout, stderr = proc.communicate(timeout=60)
    finally:
        if proc.poll() is None:
            proc.kill()
        server.close()
    assert proc.returncode == 0, stderr
    assert int(stdout.strip()) == len(geometries)
    return out


def geometries(n, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        h = np.diag(rng.uniform(8, 12, 3)) + rng.uniform(-0.5, 0.5, (3, 3))
        out.append((rng.uniform(-5, 5, (n, 3)), h))
    return out


@pytest.mark.parametrize("transport", ["tcp", "unix"])
def test_protocol_round_trip(client, tmp_path, transport):
    n = 7
    geos = geometries(n, 3, 5)
    if transport == "tcp":
        srv = IpiServer()
        args = ["--host", "127.0.0.1", "--port", str(srv.port), str(n)]
    else:
        path = str(tmp_path / "ipi_sock")
        srv = IpiServer(unix_path=path)
        args = ["--unix", path, str(n)]
    res = run_session(client, srv, args, geos)
    for (pos, h), (e, f, vir, extra) in zip(geos, res):
        assert e == pytest.approx(float(np.sum(pos * pos)), rel=1e-15)
        np.testing.assert_array_equal(f, -2.0 * pos)
        # the client echoes latVecs(i, k) = transpose(reshape(buffer, [3, 3]))(i, k) row by
        # row: with h sent row-major, latVecs(i, k) = h[i, k] (vector k is column k of h)
        np.testing.assert_array_equal(vir, h)
        assert extra == ""


def test_atom_count_mismatch_is_an_error(client):
    srv = IpiServer()
    proc = subprocess.Popen([client, "--host", "127.0.0.1", "--port", str(srv.port), "5"],
                            stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    try:
        srv.accept()
        pos, h = geometries(6, 1, 1)[0]
        with pytest.raises((ConnectionError, OSError, AssertionError)):
            srv.evaluate(pos, h)
        _, stderr = proc.communicate(timeout=60)
    finally:
        if proc.poll() is None:
            proc.kill()
        srv.close()
    assert proc.returncode == 1
    assert "Mismatch in number of atoms" in stderr
