"""Adjoint kernel against FP64 central differences and the oracle's analytic
FP64 gradient of the restated dicer + shader (visibility fixed).

Workload: the displaced 16x16 Bezier heightfield at 512x512 (256 patches),
loss = sum over pixels and RGBA of (c - c*)^2 against a target rendered from
control points + N(0, 0.05) and amplitude 1.2.  Tolerance: 1e-3 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-3


def _setup(cuda):
    torch = cuda
    from micropolis_gb300 import adjoint, scenes
    sc = scenes.heightfield16_512x512()
    dr = adjoint.DiffRenderer(sc)
    dev = torch.device("cuda")
    cp0 = torch.tensor(sc.draws[0].mesh.cp, device=dev)
    rng = np.random.default_rng(sc.seed + 100)
    cpt = cp0 + torch.tensor(rng.normal(0, 0.05, size=cp0.shape).astype(np.float32), device=dev)
    target = dr.render(cpt, 1.2).clone()
    return sc, dr, cp0, target


def test_adjoint_matches_fp64(built, cuda):
    torch = cuda
    from micropolis_gb300 import adjoint
    from oracle import oracle
    sc, dr, cp0, target = _setup(cuda)
    cp = cp0.clone().requires_grad_(True)
    amp = torch.tensor(1.0, device="cuda", requires_grad=True)
    img = adjoint.render(cp, amp, dr)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    g_gpu = cp.grad.double().cpu().numpy()
    ga_gpu = float(amp.grad)
    # fixed visibility of this forward pass
    win = dr.r.visibility(0)
    _, pid, rng_ = dr.r.subpatches()
    tgt = target.cpu().numpy()
    cpd = cp0.double().cpu().numpy()
    L, g_ref, ga_ref = oracle.loss_fp64(sc, pid, rng_, win, tgt, cpd, 1.0)
    assert abs(L - float(loss.detach())) <= 1e-4 * abs(L)
    err = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    assert err < GRAD_RTOL, err
    assert abs(ga_gpu - ga_ref) <= GRAD_RTOL * abs(ga_ref)
    # FP64 central differences (eps = 1e-4) on 64 random coordinates
    flat = cpd.reshape(-1)
    sel = np.random.default_rng(7).choice(np.flatnonzero(np.abs(g_ref.reshape(-1)) > 1e-3 * np.abs(g_ref).max()),
                                          size=64, replace=False)
    eps = 1e-4
    fd = np.zeros(len(sel))
    for i, k in enumerate(sel):
        p_ = flat.copy(); p_[k] += eps
        m_ = flat.copy(); m_[k] -= eps
        fd[i] = (oracle.loss_fp64(sc, pid, rng_, win, tgt, p_.reshape(cpd.shape), 1.0, grad=False) -
                 oracle.loss_fp64(sc, pid, rng_, win, tgt, m_.reshape(cpd.shape), 1.0, grad=False)) / (2 * eps)
    g = g_gpu.reshape(-1)[sel]
    # relative error of the sampled gradient vector; single coordinates whose
    # value is a cancellation of large silhouette terms carry FP32 noise
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)
    assert np.all(np.abs(g - fd) <= 1e-2 * np.maximum(np.abs(fd), 1e-2 * np.abs(fd).max()))
    fa = (oracle.loss_fp64(sc, pid, rng_, win, tgt, cpd, 1.0 + eps, grad=False) -
          oracle.loss_fp64(sc, pid, rng_, win, tgt, cpd, 1.0 - eps, grad=False)) / (2 * eps)
    assert abs(ga_gpu - fa) <= GRAD_RTOL * abs(fa)


def test_adjoint_bwd_cost(built, cuda):
    from micropolis_gb300 import adjoint
    res = adjoint.bench_bwd_fwd(steps=5)
    assert res["bwd_over_fwd"] <= 2.5, res


def test_adjoint_gregory_matches_fp64(built, cuda):
    """The same check on the heightfield turned into Gregory patches (the
    20-point layout of tools/bez2mscene_greg.py), through the face blends."""
    torch = cuda
    from micropolis_gb300 import adjoint, scenes
    from oracle import oracle
    sc = scenes.heightfield16_512x512()
    d = sc.draws[0]
    d.mesh = scenes.Mesh(scenes.GREGORY, np.ascontiguousarray(d.mesh.cp[:, scenes.BEZIER_TO_GREGORY, :]))
    dr = adjoint.DiffRenderer(sc)
    dev = torch.device("cuda")
    cp0 = torch.tensor(d.mesh.cp, device=dev)
    rng = np.random.default_rng(sc.seed + 200)
    cpt = cp0 + torch.tensor(rng.normal(0, 0.05, size=cp0.shape).astype(np.float32), device=dev)
    target = dr.render(cpt, 1.2).clone()
    cp = cp0.clone().requires_grad_(True)
    amp = torch.tensor(1.0, device="cuda", requires_grad=True)
    img = adjoint.render(cp, amp, dr)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    win = dr.r.visibility(0)
    _, pid, rng_ = dr.r.subpatches()
    cpd = cp0.double().cpu().numpy()
    L, g_ref, ga_ref = oracle.loss_fp64(sc, pid, rng_, win, target.cpu().numpy(), cpd, 1.0)
    assert abs(L - float(loss.detach())) <= 1e-4 * abs(L)
    g_gpu = cp.grad.double().cpu().numpy()
    assert np.linalg.norm(g_gpu - g_ref) <= GRAD_RTOL * np.linalg.norm(g_ref)
    assert abs(float(amp.grad) - ga_ref) <= GRAD_RTOL * abs(ga_ref)
