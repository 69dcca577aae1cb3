import os
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(__file__)):
    if p not in sys.path:
        sys.path.insert(0, p)

# A Fortnet source checkout, read by the CPU tests that compare the host readers and writers
# with the reference's own HDF5 files: $FORTNET_REFERENCE, else a checkout named "reference"
# beside this repository.  Those tests skip where neither exists (the GPU test machines).
REFERENCE = os.environ.get("FORTNET_REFERENCE") or os.path.normpath(
    os.path.join(ROOT, "..", "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
