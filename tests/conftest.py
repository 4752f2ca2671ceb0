"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs everything that needs no GPU (the oracle against the
golden fixtures, HEALPix identities, the host-side logic, the C-ABI library's
exports); ``-m gpu`` runs the parity tests proper on a GB300.
"""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "dm-annihilation-cxx_gb300", "pywrapper"), os.path.join(REPO, "oracle"),
          os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
