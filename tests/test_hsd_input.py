"""The HSD input front end of the fnetg program (fortnet_gb300/host/hsd.cpp, fnet_input.cpp):
the fortnet_in.hsd of every case of the reference's regression suite (kept in the golden
fixtures) is parsed by `fnetg --parse-only` in a run directory holding the case's dataset
(written by the host layer's dataset writer); the settings must equal those the fixtures were
extracted with, and for training runs that start from scratch the species-expanded
G-functions (explicit functions, then the Auto scheme of acsf.F90:276-363, expanded per
initprogram.F90:1453-1527) must equal the functions in the reference's expected netstat.
No GPU."""

import json
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
from fnetg_cases import build_writer, materialise
from fortnet_gb300 import api, build as B

CASES = G.case_names()
LOSS = {"mse": 0, "rms": 1, "mae": 2, "mape": 3}
OPT = {"sd": 0, "lbfgs": 1, "cg": 2, "fire": 3}


@pytest.fixture(scope="module")
def fnetg():
    B.build_host()
    return B.HOST_FNETG


def parse(fnetg, path):
    res = subprocess.run([fnetg, path, "--parse-only"], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    return json.loads(res.stdout)


def test_every_reference_input_matches_the_golden_settings(fnetg, tmp_path):
    writer = build_writer(str(tmp_path))
    checked = funcs_checked = 0
    for name in CASES:
        case = G.load_case(name)
        st = case.settings
        hsd = materialise(case, str(tmp_path / name.replace("/", "__")), writer)
        got = parse(fnetg, hsd)
        assert got["mode"] == st["mode"], name
        assert bool(got["read_netstat"]) == st["read_netstat"], name
        assert got["seed"] == st["seed"], name
        if st["mode"] == "train":
            assert OPT[st["optimizer"]] == got["optimizer"], name
            for key in ("threshold", "min_disp", "max_disp", "learning_rate", "regu_strength",
                        "regu_alpha"):
                assert got[key] == pytest.approx(st[key], rel=1e-15, abs=0), (name, key)
            assert got["niter"] == st["niter"], name
            assert got["loss"] == LOSS[st["loss"]], name
            assert bool(got["shuffle"]) == st["shuffle"], name
            assert bool(got["linemin"]) == st["linemin"], name
            assert got["memory"] == st["memory"], name
            assert bool(got["qn_max_disp"]) == st["qn_max_disp"], name
            assert bool(got["standardize"]) == st["standardize"], name
        if "forces" in st:
            assert got["forces"] == st["forces"], name
            if st["forces"] == "finitedifferences":
                assert got["fd_delta"] == st["fd_delta"], name
        checked += 1
        # G-functions of a fresh training run against the reference's expected netstat
        out = case.net("out_") if "out_dims" in case.arrays else None
        if st["mode"] == "train" and not st["read_netstat"] and out is not None and out["gfuncs"]:
            g = np.asarray(got["gfunctions"], dtype=np.float64).reshape(-1, 10)
            ref = out["gfuncs"]
            assert len(g) == len(ref), name
            for row, f in zip(g, ref):
                assert (int(row[0]), int(row[1]), int(row[2]), int(row[3])) == (
                    {"g1": 1, "g2": 2, "g3": 3, "g4": 4, "g5": 5}[f.type], f.atomid, f.z1, f.z2), name
                np.testing.assert_allclose(row[4:], [f.rcut, f.kappa, f.rs, f.eta, f.lam, f.xi],
                                           rtol=1e-15, atol=0, err_msg=name)
            # the network topology follows from the functions, the hidden layers and targets
            assert out["dims"][1:-1] == got["hidden"], name
            assert api.ACT[out["activation"]] == got["activation"], name
            funcs_checked += 1
    assert checked == len(CASES) and funcs_checked > 50


def test_parse_errors_are_reported(fnetg, tmp_path):
    bad = tmp_path / "fortnet_in.hsd"
    bad.write_text("Options {\n  Mode = 'train'\n\nData {\n")
    res = subprocess.run([fnetg, str(bad), "--parse-only"], capture_output=True, text=True)
    assert res.returncode == 1 and "HSD" in res.stderr
    bad.write_text("Options { Mode = 'fly' }\nData { Dataset = 'x.hdf5' }\n")
    res = subprocess.run([fnetg, str(bad), "--parse-only"], capture_output=True, text=True)
    assert res.returncode == 1 and "Invalid program running mode" in res.stderr
