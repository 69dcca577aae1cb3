"""Extract golden vectors from the reference's own regression fixtures.

Reads the Fortnet test tree (datasets, ``fortnet_in.hsd`` inputs, input netstats and the
golden ``_fortnet.hdf5`` / ``_fnetout.hdf5`` outputs written by the reference program)
with the project's HDF5 reader and writes compact ``.npz`` files next to this script:

* ``datasets/<name>.npz``  one per reference dataset (CSR arrays of fnetdata.Dataset)
* ``cases/<case>.npz``     one per supported test case: settings, input netstat (if any)
                           and the reference's outputs (predictions, forces, trained
                           weights, z-score statistics)

Usage: python tests/golden/make_golden.py /path/to/fortnet/source
The GPU machine never runs this; the committed ``.npz`` files are what the tests read.
"""

from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from fortnet_gb300 import fnetdata, hdf5lite, netstat  # noqa: E402
from fortnet_gb300.gfunctions import pack  # noqa: E402


# ------------------------------------------------------------------ minimal HSD reader
def _tokens(text):
    text = re.sub(r"#.*", "", text)
    pat = re.compile(r"\s*(\{|\}|=|'[^']*'|\"[^\"]*\"|[^\s{}=]+)")
    pos, out = 0, []
    while True:
        m = pat.match(text, pos)
        if not m:
            break
        tok = m.group(1)
        # keep track of line breaks between value tokens
        nl = "\n" in text[pos:m.start(1)]
        out.append((tok, nl))
        pos = m.end()
    return out


def parse_hsd(text):
    """Nested dict: {key: value | (TypeName, dict) | [..]} ; repeated keys become lists."""
    toks = _tokens(text)
    i = 0

    def block():
        nonlocal i
        d = {}
        while i < len(toks):
            tok, _ = toks[i]
            if tok == "}":
                i += 1
                return d
            key = tok
            i += 1
            if i < len(toks) and toks[i][0] == "{":
                i += 1
                val = (None, block())
            elif i < len(toks) and toks[i][0] == "=":
                i += 1
                if i + 1 < len(toks) and toks[i + 1][0] == "{":
                    tname = toks[i][0]
                    i += 2
                    val = (tname, block())
                else:
                    vals = [toks[i][0]]
                    i += 1
                    while i < len(toks) and not toks[i][1] and toks[i][0] not in "{}=":
                        vals.append(toks[i][0])
                        i += 1
                    val = " ".join(v.strip("'\"") for v in vals)
            else:
                val = None
            if key in d:
                if not isinstance(d[key], list) or not d.get("__list__" + key):
                    d[key] = [d[key]]
                    d["__list__" + key] = True
                d[key].append(val)
            else:
                d[key] = val
        return d

    return block()


def _get(d, path, default=None):
    cur = d
    for p in path.split("/"):
        if isinstance(cur, tuple):
            cur = cur[1]
        if not isinstance(cur, dict):
            return default
        hit = [k for k in cur if k.lower() == p.lower()]
        if not hit:
            return default
        cur = cur[hit[0]]
    return cur


def _yes(v, default=False):
    if v is None:
        return default
    return str(v).strip().lower() in ("yes", "true", ".true.")


def range_to_int(spec, ntot):
    """convRangeToInt semantics: 'a b', 'a:b' (negative b counts from the end)."""
    out = []
    for tok in str(spec).split():
        if ":" in tok:
            a, b = (int(x) for x in tok.split(":"))
            a = ntot + a + 1 if a < 0 else a
            b = ntot + b + 1 if b < 0 else b
            out += list(range(a, b + 1))
        else:
            v = int(tok)
            out.append(ntot + v + 1 if v < 0 else v)
    return out


# ------------------------------------------------------------------ extraction
def save_dataset(ds, name, outdir):
    path = os.path.join(outdir, "datasets", name + ".npz")
    if os.path.exists(path):
        return
    arrays = dict(atom_offsets=ds.atom_offsets, coords=ds.coords, atnum=ds.atnum,
                  species=ds.species, periodic=ds.periodic, latvecs=ds.latvecs,
                  atomic_numbers=ds.atomic_numbers, weights=ds.weights,
                  atomic_weights=ds.atomic_weights, global_targets=ds.global_targets,
                  atomic_targets=ds.atomic_targets)
    if ds.ext is not None:
        arrays["ext"] = ds.ext
    np.savez_compressed(path, **arrays)


def netstat_arrays(ns, prefix):
    out = {
        f"{prefix}gfuncs": pack(ns.gfunctions) if ns.gfunctions else np.zeros(0),
        f"{prefix}atomic_numbers": ns.atomic_numbers,
        f"{prefix}dims": np.asarray(ns.dims, dtype=np.int32),
        f"{prefix}params": ns.params,
        f"{prefix}nglobal": np.int32(ns.nglobal),
        f"{prefix}natomic": np.int32(ns.natomic),
    }
    if ns.zprec is not None:
        out[f"{prefix}zprec"] = ns.zprec
    if ns.ext_indices is not None:
        out[f"{prefix}ext_indices"] = ns.ext_indices
    return out, ns.activation


def extract_case(ref_root, case, outdir):
    cdir = os.path.join(ref_root, "test", "prog", "fortnet", case)
    with open(os.path.join(cdir, "fortnet_in.hsd")) as fh:
        hsd_text = fh.read()
    hsd = parse_hsd(hsd_text)
    mode = str(_get(hsd, "Options/Mode", "train")).strip("'\"").lower()
    read_netstat = _yes(_get(hsd, "Options/ReadNetStats"))
    seed = int(_get(hsd, "Options/RandomSeed", "0"))
    feats = _get(hsd, "Features")
    training = _get(hsd, "Training")
    settings = {"mode": mode, "read_netstat": read_netstat, "seed": seed}
    ext = _get(hsd, "Features/External")
    ext_spec = None
    if isinstance(ext, tuple):
        ext_spec = _get(ext[1], "Indices")
    if mode == "train":
        tname = training[0].lower() if training else "sd"
        tname = {"conjgrads": "cg", "conjgrad": "cg"}.get(tname, tname)
        if tname not in ("sd", "lbfgs", "cg", "fire"):
            return None, f"optimizer {tname}"
        tb = training[1]
        settings.update({
            "optimizer": tname,
            "learning_rate": float(_get(tb, "LearningRate", "0.01")),
            "threshold": float(_get(tb, "Threshold", "2.2250738585072014e-308")),
            "min_disp": float(_get(tb, "MinDisplacement", "1e-06")),
            "max_disp": float(_get(tb, "MaxDisplacement", "1e+04")),
            "niter": int(_get(tb, "NIterations", "1")),
            "loss": str(_get(tb, "Loss", "mse")).strip("'\"").lower(),
            "shuffle": _yes(_get(tb, "Shuffle")),
            "linemin": _yes(_get(tb, "Linemin"), True),
            "memory": int(_get(tb, "Memory", "1000")),
            "qn_max_disp": _yes(_get(tb, "MaxForQNDisplacement")),
        })
        reg = _get(tb, "Regularization")
        strength, alpha = 0.0, 0.0
        if reg is not None:
            rtype = reg[0].lower()
            strength = float(_get(reg[1], "Strength", "0"))
            alpha = {"lasso": 1.0, "ridge": 0.0}.get(rtype, None)
            if alpha is None:
                alpha = float(_get(reg[1], "Alpha", "0"))
            if strength <= 0.0:
                strength, alpha = 0.0, 0.0
        settings["regu_strength"] = strength
        settings["regu_alpha"] = alpha
        tstd = _get(hsd, "Features/Mapping/Standardization")
        settings["standardize"] = _yes(tstd, False) if feats is not None else False
    analysis = _get(hsd, "Analysis/Forces")
    if analysis is not None:
        fm = analysis[0].lower() if isinstance(analysis, tuple) else str(analysis).lower()
        if fm not in ("analytical", "finitedifferences"):
            return None, f"forces {fm}"
        settings["forces"] = fm
        if fm == "finitedifferences":
            settings["fd_delta"] = float(_get(analysis[1], "Delta", "1e-02"))
    dspath = str(_get(hsd, "Data/Dataset")).strip("'\"")
    dsfile = os.path.normpath(os.path.join(cdir, dspath))
    dsname = os.path.splitext(os.path.basename(dsfile))[0]
    ds = fnetdata.read_hdf_dataset(dsfile)
    save_dataset(ds, dsname, outdir)
    settings["dataset"] = dsname
    arrays = {}
    if ext_spec is not None and mode == "train" and not read_netstat:
        next_tot = 0 if ds.ext is None else ds.ext.shape[1]
        arrays["hsd_ext_indices"] = np.asarray(range_to_int(ext_spec, next_tot), dtype=np.int32)
    if read_netstat:
        ns_in = netstat.read_netstat(os.path.join(cdir, "fortnet.hdf5"))
        a, act = netstat_arrays(ns_in, "in_")
        arrays.update(a)
        settings["in_activation"] = act
    gold = os.path.join(cdir, "_fortnet.hdf5")
    if mode == "train" and os.path.exists(gold):
        ns_out = netstat.read_netstat(gold)
        a, act = netstat_arrays(ns_out, "out_")
        arrays.update(a)
        settings["out_activation"] = act
    fout = os.path.join(cdir, "_fnetout.hdf5")
    if os.path.exists(fout):
        out = hdf5lite.read(fout)["fnetout/output"]
        raw, frc = [], []
        for s in range(ds.nstruct):
            dp = out[f"datapoint{s + 1}"]
            raw.append(np.asarray(dp["rawpredictions"].value, dtype=np.float64))
            if "forces" in dp:
                frc.append(np.asarray(dp["forces"].value, dtype=np.float64))
        arrays["out_rawpredictions"] = np.concatenate(raw)
        if frc:
            arrays["out_forces"] = np.concatenate(frc)
    arrays["settings"] = np.frombuffer(json.dumps(settings).encode(), dtype=np.uint8)
    # the input file itself, for running the whole program on the case
    arrays["hsd"] = np.frombuffer(hsd_text.encode(), dtype=np.uint8)
    fname = case.replace("/", "__") + ".npz"
    np.savez_compressed(os.path.join(outdir, "cases", fname), **arrays)
    return fname, None


def main(ref_root):
    outdir = HERE
    os.makedirs(os.path.join(outdir, "datasets"), exist_ok=True)
    os.makedirs(os.path.join(outdir, "cases"), exist_ok=True)
    with open(os.path.join(ref_root, "test", "prog", "fortnet", "tests")) as fh:
        cases = [ln.split("#")[0].strip() for ln in fh if ln.strip() and not ln.startswith("#")]
    cases = [c for c in cases if c and not c.startswith("sockets")]
    done, skipped = [], {}
    for case in cases:
        try:
            fname, why = extract_case(ref_root, case, outdir)
        except Exception as exc:  # noqa: BLE001 - report and continue
            fname, why = None, f"error: {exc}"
        if fname:
            done.append(case)
        else:
            skipped[case] = why
    with open(os.path.join(outdir, "INDEX.json"), "w") as fh:
        json.dump({"cases": done, "skipped": skipped}, fh, indent=1)
    print(f"{len(done)} cases extracted, {len(skipped)} skipped")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <fortnet source checkout>")
    main(sys.argv[1])
