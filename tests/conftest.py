import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "c-2graph_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the library, the drop-in programs and the oracle (idempotent)."""
    import __graft_entry__

    __graft_entry__.build()
    import c2g

    return c2g.lib()


def golden_cases():
    """The graph fixtures (tests/golden/make_golden.py); convert_text.npz is the text
    converter's own fixture (tests/test_convert.py)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f != "convert_text.npz")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def write_dataset(d, g):
    """Write a golden case's arrays as a reference dataset directory."""
    for sub in ("origin", "sssp", "ppr"):
        os.makedirs(os.path.join(d, sub), exist_ok=True)
    for key, a in g.items():
        sub, _, name = key.partition("_")
        if sub in ("origin", "sssp", "ppr") and name:
            a.tofile(os.path.join(d, sub, name + ".bin"))
    g["hvmap"].tofile(os.path.join(d, "sssp", "hvmap.bin"))
    return d


@pytest.fixture(scope="session")
def gpu_available(built):
    import c2g

    assert c2g.device_count() >= 1, "GPU tests need a CUDA device"
    return True
