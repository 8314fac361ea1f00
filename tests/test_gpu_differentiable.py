"""Occupation-weighted counts and their hand-written adjoint, against FP64
references: the C oracle's weighted counts and brute-force FP64 gradient, and
central finite differences (step 1e-4 in theta) of the FP64 forward."""
import numpy as np
import pytest
from scipy.special import erf

from oracle import oracle

pytestmark = pytest.mark.gpu

THETA = np.array([12.0, 0.3, 12.0, 13.3, 1.0])


def zheng07_np(theta, mass):
    logMmin, sig, logM0, logM1, alpha = theta
    ncen = 0.5 * (1.0 + erf((np.log10(mass) - logMmin) / sig))
    m0, m1 = 10.0 ** logM0, 10.0 ** logM1
    nsat = np.where(mass > m0, ((np.maximum(mass - m0, 0.0)) / m1) ** alpha, 0.0)
    return ncen + nsat


def halos(n, L, seed):
    from halotools_gb300 import mocks
    return mocks.halo_table(n, L, seed=seed)


def test_zheng07_weights_and_vjp(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    pos, mass, conc = halos(20000, 100.0, 1)
    th = torch.tensor(THETA, dtype=torch.float64, device="cuda", requires_grad=True)
    m = torch.from_numpy(mass).cuda()
    w = D.zheng07_weights(th, m)
    # 0.5 (1 + erf x) cancels for x << 0: compare to an absolute 1e-15 as well
    np.testing.assert_allclose(w.detach().cpu().numpy(), zheng07_np(THETA, mass), rtol=1e-12,
                               atol=1e-15)
    g = torch.from_numpy(np.random.default_rng(2).normal(size=len(mass))).cuda()
    (w * g).sum().backward()
    # finite differences of the FP64 numpy formula
    h = 1e-6
    fd = np.array([(np.dot(zheng07_np(THETA + h * e, mass), g.cpu().numpy()) -
                    np.dot(zheng07_np(THETA - h * e, mass), g.cpu().numpy())) / (2 * h)
                   for e in np.eye(5)])
    np.testing.assert_allclose(th.grad.cpu().numpy(), fd, rtol=1e-6, atol=1e-6)


def test_weighted_counts_forward_matches_fp64(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    L = 150.0
    pos, mass, _ = halos(40000, L, 3)
    w = zheng07_np(THETA, mass)
    rb = np.logspace(-1, np.log10(30), 20)
    C = D.weighted_pair_counts(torch.from_numpy(w).cuda(), torch.from_numpy(pos).cuda(), rb, L)
    want = oracle.marked_npairs_3d(pos, pos, rb, 1, period=L, weights1=w, weights2=w,
                                   num_threads=8)
    rel = np.abs(C.cpu().numpy() - want) / np.abs(want)
    assert rel.max() < 1e-6, rel


def test_adjoint_dw_matches_fp64_gradient(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    L = 60.0
    pos, mass, _ = halos(6000, L, 4)
    w = zheng07_np(THETA, mass)
    rb = np.logspace(-1, np.log10(15), 12)
    gbar = np.random.default_rng(5).normal(size=len(rb))
    wt = torch.from_numpy(w).cuda().requires_grad_(True)
    C = D.weighted_pair_counts(wt, torch.from_numpy(pos).cuda(), rb, L)
    (C * torch.from_numpy(gbar).cuda()).sum().backward()
    want = oracle.weighted_adjoint_3d(pos, w, rb, L, gbar)
    got = wt.grad.cpu().numpy()
    scale = np.abs(want).max()
    assert np.max(np.abs(got - want)) / scale < 2e-6
    # spot check one row against the marked-count identity
    m = 123
    c = oracle.marked_npairs_3d(pos[m:m + 1], pos, rb, 1, period=L, weights1=np.ones(1),
                                weights2=w)
    assert abs(got[m] - 2 * np.dot(gbar, c)) <= 2e-6 * scale


def test_hod_gradient_matches_central_differences(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    L = 80.0
    pos, mass, _ = halos(8000, L, 6)
    rb = np.logspace(-1, np.log10(20), 10)
    gbar = np.random.default_rng(7).normal(size=len(rb))
    th = torch.tensor(THETA, dtype=torch.float64, device="cuda", requires_grad=True)
    C = D.hod_pair_counts(th, torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda(), rb, L)
    (C * torch.from_numpy(gbar).cuda()).sum().backward()
    got = th.grad.cpu().numpy()

    def loss(theta):
        w = zheng07_np(theta, mass)
        c = oracle.marked_npairs_3d(pos, pos, rb, 1, period=L, weights1=w, weights2=w,
                                    num_threads=8)
        return float(np.dot(gbar, c))

    h = 1e-4
    fd = np.array([(loss(THETA + h * e) - loss(THETA - h * e)) / (2 * h) for e in np.eye(5)])
    np.testing.assert_allclose(got, fd, rtol=2e-4, atol=1e-6 * np.abs(fd).max())


# ---------------- many parameter draws in one forward and one adjoint pass ----------------
def _thetas(m, seed):
    rng = np.random.default_rng(seed)
    lmin = rng.uniform(11.8, 12.4, m)
    return np.stack([lmin, rng.uniform(0.2, 0.5, m), lmin, lmin + 1.3, rng.uniform(0.9, 1.1, m)],
                    axis=1)


def test_batched_forward_and_dw_match_fp64(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    L = 120.0
    pos, mass, _ = halos(8000, L, 21)
    m_draws = 19  # adjoint groups of 16 (one point per lane) and 3 (two per lane)
    th = _thetas(m_draws, 22)
    W = np.stack([zheng07_np(t, mass) for t in th], axis=1)
    rb = np.logspace(-1, np.log10(15), 10)
    Wt = torch.from_numpy(W).cuda().requires_grad_(True)
    C = D.weighted_pair_counts_batched(Wt, torch.from_numpy(pos).cuda(), rb, L)
    assert C.shape == (m_draws, len(rb))
    gbar = np.random.default_rng(23).normal(size=(m_draws, len(rb)))
    (C * torch.from_numpy(gbar).cuda()).sum().backward()
    got_w = Wt.grad.cpu().numpy()
    for m in range(m_draws):
        want = oracle.marked_npairs_3d(pos, pos, rb, 1, period=L, weights1=W[:, m],
                                       weights2=W[:, m], num_threads=8)
        np.testing.assert_allclose(C[m].detach().cpu().numpy(), want, rtol=1e-6)
        wg = oracle.weighted_adjoint_3d(pos, W[:, m], rb, L, gbar[m])
        assert np.max(np.abs(got_w[:, m] - wg)) / np.abs(wg).max() < 2e-6, m


def test_batched_dw_twelve_channels_on_finer_grids(gpu):
    """12 draws (the one-point-per-lane adjoint with 4 padded channels) against the
    FP64 brute-force gradient, on the automatic grid and on forced finer ones."""
    import torch
    from halotools_gb300 import _native
    from halotools_gb300 import differentiable as D
    L = 90.0
    pos, mass, _ = halos(6000, L, 31)
    th = _thetas(12, 32)
    W = np.stack([zheng07_np(t, mass) for t in th], axis=1)
    rb = np.logspace(-1, np.log10(12), 9)
    gbar = np.random.default_rng(33).normal(size=(12, len(rb)))
    want = [oracle.weighted_adjoint_3d(pos, W[:, m], rb, L, gbar[m]) for m in range(12)]
    plan = _native.default_plan()
    try:
        for reach, block in ((0, 0), (2, 2), (3, 1)):
            plan.set_reach(reach)
            plan.set_block(block)
            Wt = torch.from_numpy(W).cuda().requires_grad_(True)
            C = D.weighted_pair_counts_batched(Wt, torch.from_numpy(pos).cuda(), rb, L)
            (C * torch.from_numpy(gbar).cuda()).sum().backward()
            got = Wt.grad.cpu().numpy()
            for m in range(12):
                err = np.max(np.abs(got[:, m] - want[m])) / np.abs(want[m]).max()
                assert err < 2e-6, (reach, block, m, err)
    finally:
        plan.set_reach(0)
        plan.set_block(0)


def test_batched_theta_gradient_matches_single_draws(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    L = 150.0
    pos, mass, _ = halos(20000, L, 24)
    th = _thetas(5, 25)
    rb = np.logspace(-1, np.log10(20), 12)
    x, m = torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda()
    T = torch.tensor(th, dtype=torch.float64, device="cuda", requires_grad=True)
    gbar = torch.from_numpy(np.random.default_rng(26).normal(size=(5, len(rb)))).cuda()
    C = D.hod_pair_counts_batched(T, x, m, rb, L)
    (C * gbar).sum().backward()
    for k in range(5):
        t1 = torch.tensor(th[k], dtype=torch.float64, device="cuda", requires_grad=True)
        c1 = D.hod_pair_counts(t1, x, m, rb, L)
        (c1 * gbar[k]).sum().backward()
        np.testing.assert_allclose(C[k].detach().cpu().numpy(), c1.detach().cpu().numpy(),
                                   rtol=1e-6)
        g1 = t1.grad.cpu().numpy()
        np.testing.assert_allclose(T.grad[k].cpu().numpy(), g1, rtol=1e-5,
                                   atol=1e-6 * np.abs(g1).max())


def test_batched_zheng07_weights_and_vjp(gpu):
    import torch
    from halotools_gb300 import differentiable as D
    pos, mass, _ = halos(50000, 200.0, 27)
    th = _thetas(6, 28)
    T = torch.tensor(th, dtype=torch.float64, device="cuda", requires_grad=True)
    W = D.zheng07_weights_batched(T, torch.from_numpy(mass).cuda())
    want = np.stack([zheng07_np(t, mass) for t in th], axis=1)
    # FP32 occupations from an FP64 log10 M: 1e-6 relative (absolute near 0)
    np.testing.assert_allclose(W.detach().cpu().numpy(), want, rtol=1e-6, atol=1e-7)
    g = torch.from_numpy(np.random.default_rng(29).normal(size=W.shape)).cuda()
    (W * g).sum().backward()
    for k in range(6):
        t1 = torch.tensor(th[k], dtype=torch.float64, device="cuda", requires_grad=True)
        (D.zheng07_weights(t1, torch.from_numpy(mass).cuda()) * g[:, k]).sum().backward()
        g1 = t1.grad.cpu().numpy()
        np.testing.assert_allclose(T.grad[k].cpu().numpy(), g1, rtol=1e-5,
                                   atol=1e-6 * np.abs(g1).max())
