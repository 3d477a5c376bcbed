"""Phase tracing of the persistent launches: the phases of the last launch on a handle
add up to its device time (block 0 timestamps at every grid barrier)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_last_phases_add_up(gpu_available, tmp_path):
    import c2g

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 16, 16, 3, 1, 1000)
    vl = c2g.read_array(d + "/origin/vlist.bin")
    deg = np.diff(vl)
    srcs = np.flatnonzero(deg > 0)[:40].astype(np.int32)
    with c2g.Graph.load(d, "origin") as g:
        runs = [lambda: g.sssp(int(srcs[0]))[1],
                lambda: g.ppr(int(srcs[0]), g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15))[2],
                lambda: g.sssp_batch(srcs)[1],
                lambda: g.ppr_batch(srcs, g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15))[2]]
        for run in runs:
            st = run()
            ph = g.last_phases()
            assert all(x >= 0.0 for x in ph) and ph[3] == 0.0
            assert ph[2] > 0.0
            # the launch's CUDA-event time brackets block 0's barrier-to-barrier time
            assert sum(ph) <= st.device_ms * 1.05 + 0.05, (ph, st.device_ms)
            assert sum(ph) >= st.device_ms * 0.5 - 0.05, (ph, st.device_ms)
