"""PPR adjoint on the GPU (transposed push on the reverse CSR + gradient pass) against
an FP64 dense solve and central finite differences, through a torch.autograd.Function
over the C ABI.

Configuration of the adjoint check: R-MAT scale 12, edge factor 8, alpha = 0.15,
rmax = 1e-8 (forward and backward push), 64 random targets, 200 random edges for finite
differences with h = 1e-4.  Tolerance: ||g_gpu - g_fp64|| / ||g_fp64|| <= 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALPHA = 0.15
EPS = 1e-8


@pytest.fixture(scope="module")
def g12(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("adj12"))
    c2g.rmat_write(d, 12, 8, 4, 1, 1000)
    return d


def dense_setup(vl, el, fl, s, targets):
    import scipy.linalg as sla

    V = len(vl) - 1
    P = np.zeros((V, V))
    src = np.repeat(np.arange(V), np.diff(vl))
    np.add.at(P, (src, el), fl.astype(np.float64))
    M = np.eye(V) - (1 - ALPHA) * P.T
    lu = sla.lu_factor(M)
    x = sla.lu_solve(lu, np.eye(V)[s])
    oneT = np.zeros(V)
    np.add.at(oneT, targets, 1.0)
    lam = np.linalg.solve(np.eye(V) - (1 - ALPHA) * P, oneT)
    grad = (1 - ALPHA) * (ALPHA * x[src]) * lam[el]
    return lu, x, oneT, src, grad


def test_adjoint_vs_dense_and_fd(gpu_available, g12):
    import scipy.linalg as sla

    import c2g
    import oracle

    o = oracle.load_dataset(g12, "origin")
    vl, el, fl = o["vlist"], o["elist"], o["flist"]
    V, E = len(vl) - 1, len(el)
    rng = np.random.default_rng(12)
    s = int(np.argmax(np.diff(vl)))
    targets = rng.choice(V, 64, replace=False).astype(np.int32)
    with c2g.Graph.load(g12, "origin") as g:
        prm = g.ppr_params(alpha=ALPHA, rmax=EPS, seeded=0, pr0=ALPHA, r0=1.0, max_iter=10000)
        grad, pi, lam, loss, st = g.ppr_adjoint(s, targets, prm, rmax_backward=EPS)
    assert st.status_flags == 0
    lu, x, oneT, src, gd = dense_setup(vl, el, fl, s, targets)
    # forward and loss
    assert np.abs(pi - ALPHA * x).sum() <= 1e-4
    assert abs(loss - ALPHA * x[targets].sum()) <= 1e-5
    # gradient vs the FP64 dense-solve gradient
    rel = np.linalg.norm(grad.astype(np.float64) - gd) / np.linalg.norm(gd)
    assert rel <= 1e-4, rel
    # central finite differences of the exact (dense) loss on 200 random edges; each
    # perturbation is a rank-one update of M, solved with Sherman-Morrison.
    h = 1e-4
    edges = rng.choice(E, 200, replace=False)
    fd = np.empty(len(edges))
    for k, e in enumerate(edges):
        u, v = src[e], el[e]
        Mv = sla.lu_solve(lu, np.eye(V)[v])
        vals = []
        for dlt in (h, -h):
            c = (1 - ALPHA) * dlt
            xp = x + c * Mv * x[u] / (1.0 - c * Mv[u])
            vals.append(ALPHA * (oneT @ xp))
        fd[k] = (vals[0] - vals[1]) / (2 * h)
    assert np.linalg.norm(fd - gd[edges]) / np.linalg.norm(gd[edges]) <= 1e-6
    assert np.linalg.norm(grad[edges] - fd) / np.linalg.norm(fd) <= 1e-4


def test_adjoint_autograd_function(gpu_available, g12):
    """torch.autograd.Function over the C ABI: forward = c2g_ppr with the given edge
    weights, backward = c2g_ppr_adjoint."""
    import torch

    import c2g
    import oracle

    o = oracle.load_dataset(g12, "origin")
    vl = o["vlist"]
    V = len(vl) - 1
    s = int(np.argmax(np.diff(vl)))
    targets = np.random.default_rng(3).choice(V, 64, replace=False).astype(np.int32)
    g = c2g.Graph.load(g12, "origin")
    prm = g.ppr_params(alpha=ALPHA, rmax=EPS, seeded=0, pr0=ALPHA, r0=1.0, max_iter=10000)

    class PPRScore(torch.autograd.Function):
        @staticmethod
        def forward(ctx, w):
            g.set_weights(w.detach().cpu().numpy())
            pr, _, _ = g.ppr(s, prm)
            return torch.tensor(float(pr[targets].astype(np.float64).sum()), dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            grad, _, _, _, _ = g.ppr_adjoint(s, targets, prm, rmax_backward=EPS)
            return gout * torch.from_numpy(grad).to(torch.float64)

    w0 = torch.from_numpy(o["flist"].astype(np.float64)).requires_grad_(True)
    loss = PPRScore.apply(w0)
    (gw,) = torch.autograd.grad(loss, w0)
    grad_direct, _, _, L, _ = g.ppr_adjoint(s, targets, prm, rmax_backward=EPS)
    # two adjoint runs agree up to FP32 atomic summation order
    rel = np.linalg.norm(gw.numpy() - grad_direct) / np.linalg.norm(grad_direct)
    assert rel <= 1e-5, rel
    assert abs(loss.item() - L) <= 1e-6
    # a small step along the gradient raises the loss by about |g|^2 * step
    step = 1e-3 / float(np.linalg.norm(grad_direct))
    w1 = (w0.detach() + step * gw).requires_grad_(False)
    l1 = PPRScore.apply(w1).item()
    pred = loss.item() + step * float((gw * gw).sum())
    assert abs(l1 - pred) <= 0.05 * abs(pred - loss.item())
    g.close()
