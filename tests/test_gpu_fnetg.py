"""The whole fnet program on the GPU library (fnetg: fortnet_in.hsd -> HDF5 outputs) on every
case of the reference's regression suite: each case's own input runs in a directory holding
its dataset (and input netstat), and the files fnetg writes must match the reference's
expected results at the reference's tolerance (rtol 1e-9, atol 1e-10,
test/prog/fortnet/testwithworkdir.py:24-25): the trained netstat's parameters and z-score
statistics in train mode, raw predictions and forces in fnetout.hdf5 otherwise."""

import concurrent.futures as cf
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
from fnetg_cases import build_writer, materialise
from fortnet_gb300 import build as B, hdf5lite, netstat

pytestmark = pytest.mark.gpu
RTOL, ATOL = 1e-9, 1e-10


def run_case(name, root, writer):
    case = G.load_case(name)
    st = case.settings
    wd = os.path.join(root, name.replace("/", "__"))
    hsd = materialise(case, wd, writer)
    res = subprocess.run([B.HOST_FNETG, hsd], capture_output=True, text=True, timeout=600)
    if res.returncode != 0:
        return f"{name}: fnetg failed: {res.stderr.strip()[-300:]}"
    try:
        if st["mode"] == "train":
            if "out_params" not in case.arrays:
                return None
            ns = netstat.read_netstat(os.path.join(wd, "fortnet.hdf5"))
            np.testing.assert_allclose(ns.params, case.arrays["out_params"], rtol=RTOL, atol=ATOL)
            if "out_zprec" in case.arrays:
                np.testing.assert_allclose(np.asarray(ns.zprec), case.arrays["out_zprec"],
                                           rtol=RTOL, atol=ATOL)
        else:
            out = hdf5lite.read(os.path.join(wd, "fnetout.hdf5"))["fnetout/output"]
            raw, frc = [], []
            for s in range(case.ds.nstruct):
                dp = out[f"datapoint{s + 1}"]
                raw.append(np.asarray(dp["rawpredictions"].value))
                if "forces" in dp:
                    frc.append(np.asarray(dp["forces"].value))
            if "out_rawpredictions" in case.arrays:
                np.testing.assert_allclose(np.concatenate(raw), case.arrays["out_rawpredictions"],
                                           rtol=RTOL, atol=ATOL)
            if "out_forces" in case.arrays:
                np.testing.assert_allclose(np.concatenate(frc), case.arrays["out_forces"],
                                           rtol=RTOL, atol=ATOL)
    except AssertionError as exc:
        return f"{name}: {str(exc).strip().splitlines()[0]} {str(exc).strip().splitlines()[-1]}"
    return None


def test_every_regression_case_through_the_program(tmp_path):
    writer = build_writer(str(tmp_path))
    names = G.case_names()
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(lambda n: run_case(n, str(tmp_path), writer), names))
    failures = [r for r in results if r]
    assert not failures, f"{len(failures)} of {len(names)} cases differ:\n" + "\n".join(failures[:20])
