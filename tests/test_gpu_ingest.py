"""R-MAT generation on the GPU writes the same origin/ files as the host generator,
byte for byte (endpoint draws, dedup, weights and the normalised flist)."""
import filecmp
import os

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,ef,seed,wmax", [(12, 8, 3, 100), (16, 16, 1, 100), (18, 16, 2, 1000)])
def test_rmat_gpu_matches_host(gpu_available, built, tmp_path, scale, ef, seed, wmax):
    import c2g

    host, dev = str(tmp_path / "host"), str(tmp_path / "dev")
    c2g.rmat_write(host, scale, ef, seed, 1, wmax)
    c2g.rmat_write(dev, scale, ef, seed, 1, wmax, gpu=True)
    for f in ("vlist", "elist", "wlist", "flist"):
        a, b = os.path.join(host, "origin", f + ".bin"), os.path.join(dev, "origin", f + ".bin")
        assert filecmp.cmp(a, b, shallow=False), (scale, f)
