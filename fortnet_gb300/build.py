"""Builds libfnetg.so (the CUDA library behind include/fnetg.h) in-tree with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then linked into
``fortnet_gb300/_build/libfnetg.so``.  No CMake, no PyTorch: nvcc and the CUDA runtime.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfnetg.so")
# the bounds-checked build (every index guard compiled in; slower, for tests)
CHECKS_DIR = os.path.join(OUT_DIR, "checks")
CHECKS_LIB = os.path.join(CHECKS_DIR, "libfnetg.so")
SOURCES = ["context.cu", "neighbors.cu", "acsf.cu", "mlp.cu", "forces.cu", "train.cu", "rng.cu",
           "noalloc.cu", "fd.cu", "serve.cu", "batch.cu", "jvp.cu",
           "forceloss.cu", "probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def common_flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", os.path.join(HERE, "..", "include")]


def _compile(src, extra, out_dir=OUT_DIR):
    obj = os.path.join(out_dir, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc_path(), "-c", os.path.join(CSRC, src), "-o", obj] + common_flags() + extra
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "fnetg.h"), os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra=None, checks=False):
    """Compile and link the library; returns its path.  checks=True builds the bounds-checked
    library (-DFNETG_CHECKS) into _build/checks/ instead."""
    lib, out_dir = (CHECKS_LIB, CHECKS_DIR) if checks else (LIB, OUT_DIR)
    if not force and not _stale(lib):
        return lib
    os.makedirs(out_dir, exist_ok=True)
    extra = list(extra or []) + (["-DFNETG_CHECKS"] if checks else [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra, out_dir), SOURCES))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [nvcc_path(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


HOST_DIR = os.path.join(HERE, "host")
HOST_LIB = os.path.join(OUT_DIR, "libfnetg_host.so")
HOST_RUN = os.path.join(OUT_DIR, "fnetg_run")
HOST_SOURCES = ["hdf5lite.cpp", "h5write.cpp", "fnet_host.cpp", "ipi.cpp", "hsd.cpp", "fnet_input.cpp"]
HOST_IPI = os.path.join(OUT_DIR, "fnetg_ipi")
HOST_FNETG = os.path.join(OUT_DIR, "fnetg")
# programs linked against the host layer: output path -> source
HOST_PROGRAMS = {HOST_RUN: "fnetg_run.cpp", HOST_IPI: "fnetg_ipi.cpp", HOST_FNETG: "fnetg_main.cpp"}


def cuda_lib_dir():
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path()))), "lib64")


def host_flags():
    """g++ flags for the C++ host layer and programs linked against it."""
    return ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", HOST_DIR,
            "-I", os.path.join(HERE, "..", "include")]


def host_link_flags():
    return ["-L", OUT_DIR, "-lfnetg_host", "-lfnetg", "-L", cuda_lib_dir(), "-lcudart",
            "-Wl,-rpath," + OUT_DIR, "-Wl,-rpath," + cuda_lib_dir()]


def build_host(force=False):
    """The C++ host layer (libfnetg_host.so) and the fnetg, fnetg_run and fnetg_ipi programs,
    on top of libfnetg."""
    build()
    srcs = [os.path.join(HOST_DIR, f) for f in HOST_SOURCES + list(HOST_PROGRAMS.values())]
    hdrs = [os.path.join(HOST_DIR, f) for f in os.listdir(HOST_DIR) if f.endswith(".hpp")]
    newest = max(os.path.getmtime(f) for f in srcs + hdrs + [LIB])
    outs = [HOST_LIB] + list(HOST_PROGRAMS)
    if not force and all(os.path.exists(o) and os.path.getmtime(o) >= newest for o in outs):
        return HOST_LIB
    cmd = (["g++", "-shared", "-o", HOST_LIB + ".tmp"] + host_flags()
           + [os.path.join(HOST_DIR, f) for f in HOST_SOURCES]
           + ["-L", OUT_DIR, "-lfnetg", "-Wl,-rpath," + OUT_DIR])
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"host library build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(HOST_LIB + ".tmp", HOST_LIB)

    def link(item):
        out, src = item
        cmd = (["g++", "-o", out + ".tmp"] + host_flags() + [os.path.join(HOST_DIR, src)]
               + host_link_flags())
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"{os.path.basename(out)} build failed:\n{res.stdout}\n{res.stderr}")
        os.replace(out + ".tmp", out)

    with cf.ThreadPoolExecutor(max_workers=len(HOST_PROGRAMS)) as ex:
        list(ex.map(link, HOST_PROGRAMS.items()))
    return HOST_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
    print(build_host(force="--force" in sys.argv))
