"""Adsorption label propagation (16 labels, per-vertex p_inj/p_cont/p_abnd from
Dirichlet(1,1,1), 30 iterations) on the GPU against the FP64 oracle recurrence.
Tolerance per label column: L1 <= 1e-6 * max(1, L1 norm of the FP64 column)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,ef", [(12, 8), (15, 16)])
def test_adsorption_vs_fp64(gpu_available, tmp_path, scale, ef):
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, scale, ef, 5, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(scale)
    pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
    seeds = rng.choice(V, 16, replace=False).astype(np.int32)
    with c2g.Graph.load(d, "origin") as g:
        Y, st = g.adsorption(seeds, pp[:, 0], pp[:, 1], pp[:, 2], iterations=30)
    ref = oracle.adsorption_labels(o["vlist"], o["elist"], o["flist"], seeds, pp[:, 0], pp[:, 1], 30)
    for l in range(16):
        err = float(np.abs(Y[:, l].astype(np.float64) - ref[:, l]).sum())
        assert err <= 1e-6 * max(1.0, float(np.abs(ref[:, l]).sum())), (l, err)
    assert st.iterations == 30
