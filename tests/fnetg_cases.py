"""Materialise a golden case as the directory the fnet program runs in: fortnet_in.hsd (the
case's own input, with its dataset paths pointing at the local copies), the dataset written
through the host layer's dataset writer and, when the run reads one, the input netstat written
through the netstat writer.  Test infrastructure for the fnetg program."""

from __future__ import annotations

import os
import re
import subprocess

import numpy as np

from fortnet_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def build_writer(outdir):
    B.build_host()
    exe = os.path.join(outdir, "h5_writers")
    if not os.path.exists(exe):
        cmd = (["g++", "-o", exe] + B.host_flags()
               + [os.path.join(HERE, "cpp", "h5_writers.cpp")] + B.host_link_flags())
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(res.stderr)
    return exe


def write_dataset_bin(path, ds):
    S, N = ds.nstruct, ds.ntot
    gt = np.asarray(ds.global_targets, dtype="<f8").reshape(S, -1)
    at = np.asarray(ds.atomic_targets, dtype="<f8").reshape(N, -1)
    ext = np.zeros((N, 0)) if ds.ext is None else np.asarray(ds.ext, dtype="<f8").reshape(N, -1)
    with open(path, "wb") as fh:
        fh.write(np.int32(S).tobytes())
        fh.write(np.asarray(ds.atom_offsets, dtype="<i8").tobytes())
        fh.write(np.asarray(ds.coords, dtype="<f8").tobytes())
        fh.write(np.asarray(ds.atnum, dtype="<i4").tobytes())
        fh.write(np.asarray(ds.species, dtype="<i4").tobytes())
        fh.write(np.asarray(ds.periodic, dtype="<i4").tobytes())
        fh.write(np.asarray(ds.latvecs, dtype="<f8").reshape(S, 9).tobytes())
        fh.write(np.int32(len(ds.atomic_numbers)).tobytes())
        fh.write(np.asarray(ds.atomic_numbers, dtype="<i4").tobytes())
        fh.write(np.asarray(ds.weights, dtype="<i4").tobytes())
        fh.write(np.asarray(ds.atomic_weights, dtype="<f8").tobytes())
        fh.write(np.int32(gt.shape[1]).tobytes())
        fh.write(np.int32(at.shape[1]).tobytes())
        fh.write(gt.tobytes())
        fh.write(at.tobytes())
        fh.write(np.int32(ext.shape[1]).tobytes())
        fh.write(ext.tobytes())


def _set_value(text, key, value):
    """Replace `Key = ...` (to the end of the line) in an HSD text; drop it when value is None."""
    pat = re.compile(rf"(?im)^(\s*){key}\s*=.*$")
    if value is None:
        return pat.sub("", text)
    return pat.sub(lambda m: f"{m.group(1)}{key} = '{value}'", text)


def materialise(case, workdir, writer):
    """Write the case's run directory; returns the path of its fortnet_in.hsd."""
    from test_h5_writers import write_model

    os.makedirs(workdir, exist_ok=True)
    st = case.settings
    bin_path = os.path.join(workdir, "dataset.bin")
    write_dataset_bin(bin_path, case.ds)
    res = subprocess.run([writer, "dataset", bin_path, os.path.join(workdir, "dataset.hdf5")],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(res.stderr)
    text = st["hsd"]
    text = _set_value(text, "Dataset", "dataset.hdf5")
    text = _set_value(text, "Validset", None)  # validation monitoring changes no output file
    text = _set_value(text, "NetstatFile", "fortnet.hdf5")
    if st["read_netstat"] or st["mode"] != "train":
        inp = case.net("in_")
        model = os.path.join(workdir, "model.bin")
        write_model(model, inp["atomic_numbers"], inp["gfuncs"], inp["zprec"], inp["dims"],
                    inp["activation"], inp["nglobal"], inp["natomic"], inp["params"],
                    inp["ext_indices"])
        res = subprocess.run([writer, "netstat", model, os.path.join(workdir, "fortnet.hdf5")],
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(res.stderr)
    path = os.path.join(workdir, "fortnet_in.hsd")
    with open(path, "w") as fh:
        fh.write(text)
    return path
