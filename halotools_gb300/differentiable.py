"""Differentiable occupation-weighted pair counts (PyTorch autograd).

halotools computes HOD clustering by Monte-Carlo populating mocks and counting
pairs (hod_mock_factory.py:196-401, then tpcf); nothing in it has a gradient.
Here the expected pair counts of a Zheng07 HOD are written as an
occupation-weighted count on the halo catalogue,

    C_k(theta) = sum_ij w_i(theta) w_j(theta) [d_ij <= r_k],
    w_i = <Ncen>(M_i) + <Nsat>(M_i)   (zheng07_components.py:149-153, 455-470),

whose forward pass is ``marked_npairs_3d`` with weight function 1 on the GPU
(FP32 compensated sums) and whose reverse pass is a hand-written adjoint
kernel (dC/dw) chained with the Zheng07 vector-Jacobian product (dw/dtheta),
both behind ``torch.autograd.Function``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native
from .pair_counters import _bins, _nonneg, _period, _search_check

__all__ = ("WeightedPairCounts", "Zheng07Weights", "weighted_pair_counts", "zheng07_weights",
           "hod_pair_counts", "WeightedPairCountsBatched", "Zheng07WeightsBatched",
           "weighted_pair_counts_batched", "zheng07_weights_batched", "hod_pair_counts_batched")


def _plan():
    return _native.default_plan()


def _cuda_f64(t: torch.Tensor) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError("tensors must live on a CUDA device")
    return t.detach().to(torch.float64).contiguous()


class WeightedPairCounts(torch.autograd.Function):
    """C = sum_ij w_i w_j [d_ij <= r_k] for one periodic sample; grad w.r.t. w."""

    @staticmethod
    def forward(ctx, w, xyz, rbins, box):
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(w.device).cuda_stream)
        wd, xd = _cuda_f64(w), _cuda_f64(xyz)
        out = np.zeros(len(rbins), dtype=np.float64)
        n = xd.shape[0]
        plan.check(plan.lib.gbp_marked_npairs_3d(
            plan.handle, _native.dptr_int(xd.data_ptr()), n, _native.dptr_int(xd.data_ptr()), n,
            _native.dptr_int(wd.data_ptr()), _native.dptr_int(wd.data_ptr()), 1, 1,
            _native.pd(rbins), len(rbins), _native.pd(box), 1, _native.GBP_MEM_DEVICE,
            _native.pd(out)))
        ctx.save_for_backward(wd, xd)
        ctx.rbins, ctx.box = rbins, box
        return torch.from_numpy(out).to(w.device)

    @staticmethod
    def backward(ctx, gC):
        wd, xd = ctx.saved_tensors
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(wd.device).cuda_stream)
        g = np.ascontiguousarray(gC.detach().to("cpu", torch.float64).numpy())
        grad = torch.empty_like(wd)
        plan.check(plan.lib.gbp_weighted_adjoint_3d(
            plan.handle, _native.dptr_int(xd.data_ptr()), xd.shape[0],
            _native.dptr_int(wd.data_ptr()), _native.pd(ctx.rbins), len(ctx.rbins),
            _native.pd(ctx.box), 1, _native.GBP_MEM_DEVICE, _native.pd(g),
            _native.dptr_int(grad.data_ptr())))
        return grad, None, None, None


class Zheng07Weights(torch.autograd.Function):
    """w_i = <Ncen>(M_i; theta) + <Nsat>(M_i; theta); grad w.r.t. theta (5 values)."""

    @staticmethod
    def forward(ctx, theta, mass):
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(mass.device).cuda_stream)
        md = _cuda_f64(mass)
        th = np.ascontiguousarray(theta.detach().to("cpu", torch.float64).numpy())
        w = torch.empty_like(md)
        plan.check(plan.lib.gbp_zheng07_weights(plan.handle, _native.dptr_int(md.data_ptr()),
                                                md.shape[0], _native.pd(th),
                                                _native.GBP_MEM_DEVICE,
                                                _native.dptr_int(w.data_ptr())))
        ctx.save_for_backward(md)
        ctx.theta = th
        ctx.theta_dtype, ctx.theta_device = theta.dtype, theta.device
        return w

    @staticmethod
    def backward(ctx, gw):
        (md,) = ctx.saved_tensors
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(md.device).cuda_stream)
        g = _cuda_f64(gw)
        out = np.zeros(5, dtype=np.float64)
        plan.check(plan.lib.gbp_zheng07_vjp(plan.handle, _native.dptr_int(md.data_ptr()),
                                            md.shape[0], _native.pd(ctx.theta),
                                            _native.dptr_int(g.data_ptr()),
                                            _native.GBP_MEM_DEVICE, _native.pd(out)))
        return torch.from_numpy(out).to(ctx.theta_device, ctx.theta_dtype), None


def _geometry(rbins, period):
    rbins = _bins(rbins, "Input ``rbins`` must be a monotonically increasing 1D array with at "
                         "least two entries")
    _nonneg(rbins, "rbins")
    box = np.ascontiguousarray(_period(period), dtype=np.float64)
    _search_check([np.max(rbins)] * 3, box)
    return np.ascontiguousarray(rbins, dtype=np.float64), box


def weighted_pair_counts(w, xyz, rbins, period):
    """Differentiable C_k = sum_ij w_i w_j [d_ij <= rbins[k]] (ordered pairs, self-pairs
    included), equal to ``marked_npairs_3d(xyz, xyz, rbins, 1, period, w, w)``."""
    rbins, box = _geometry(rbins, period)
    return WeightedPairCounts.apply(w, xyz, rbins, box)


def zheng07_weights(theta, mass):
    """Per-halo Zheng07 mean occupation <Ncen> + <Nsat>, differentiable in theta."""
    return Zheng07Weights.apply(theta, mass)


def hod_pair_counts(theta, halo_xyz, halo_mass, rbins, period):
    """Expected weighted pair counts of a Zheng07 HOD on a halo catalogue, C(theta)."""
    return weighted_pair_counts(zheng07_weights(theta, halo_mass), halo_xyz, rbins, period)


# ---------------- many parameter draws at once ----------------
_ADJ_CH = 16  # channels of one batched adjoint launch (gbp_weighted_adjoint_3d_channels)


class WeightedPairCountsBatched(torch.autograd.Function):
    """C[m] = sum_ij W_im W_jm [d_ij <= r_k] for the M columns of W (N, M), M <= 32:
    one forward pass over all columns (gbp_marked_npairs_3d_channels) and one
    adjoint pass per 16 columns (gbp_weighted_adjoint_3d_channels)."""

    @staticmethod
    def forward(ctx, W, xyz, rbins, box):
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(W.device).cuda_stream)
        Wd, xd = _cuda_f64(W), _cuda_f64(xyz)
        n, m = Wd.shape
        out = np.zeros((m, len(rbins)), dtype=np.float64)
        plan.check(plan.lib.gbp_marked_npairs_3d_channels(
            plan.handle, _native.dptr_int(xd.data_ptr()), n, _native.dptr_int(xd.data_ptr()), n,
            _native.dptr_int(Wd.data_ptr()), _native.dptr_int(Wd.data_ptr()), m,
            _native.pd(rbins), len(rbins), _native.pd(box), 1, _native.GBP_MEM_DEVICE,
            _native.pd(out)))
        ctx.save_for_backward(Wd, xd)
        ctx.rbins, ctx.box = rbins, box
        return torch.from_numpy(out).to(W.device)

    @staticmethod
    def backward(ctx, gC):
        Wd, xd = ctx.saved_tensors
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(Wd.device).cuda_stream)
        g = gC.detach().to("cpu", torch.float64).numpy()
        n, m = Wd.shape
        grad = torch.empty_like(Wd)
        for c0 in range(0, m, _ADJ_CH):
            c1 = min(m, c0 + _ADJ_CH)
            wg = Wd[:, c0:c1].contiguous()
            gg = torch.empty_like(wg)
            gb = np.ascontiguousarray(g[c0:c1])
            plan.check(plan.lib.gbp_weighted_adjoint_3d_channels(
                plan.handle, _native.dptr_int(xd.data_ptr()), n, _native.dptr_int(wg.data_ptr()),
                c1 - c0, _native.pd(ctx.rbins), len(ctx.rbins), _native.pd(ctx.box), 1,
                _native.GBP_MEM_DEVICE, _native.pd(gb), _native.dptr_int(gg.data_ptr())))
            grad[:, c0:c1] = gg
        return grad, None, None, None


class Zheng07WeightsBatched(torch.autograd.Function):
    """W[:, m] = <Ncen>(M_i; theta_m) + <Nsat>(M_i; theta_m) for thetas (M, 5): one
    launch over (halo, draw) each way (occupations and VJP terms in FP32 from hi/lo
    float splits of log10 M and M; each lane's VJP sums compensated in FP32, the
    lanes reduced in FP64)."""

    @staticmethod
    def forward(ctx, thetas, mass):
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(mass.device).cuda_stream)
        md = _cuda_f64(mass)
        th = np.ascontiguousarray(thetas.detach().to("cpu", torch.float64).numpy())
        W = torch.empty((md.shape[0], len(th)), dtype=torch.float64, device=md.device)
        plan.check(plan.lib.gbp_zheng07_weights_batched(
            plan.handle, _native.dptr_int(md.data_ptr()), md.shape[0], _native.pd(th), len(th),
            _native.GBP_MEM_DEVICE, _native.dptr_int(W.data_ptr())))
        ctx.save_for_backward(md)
        ctx.thetas = th
        ctx.theta_dtype, ctx.theta_device = thetas.dtype, thetas.device
        return W

    @staticmethod
    def backward(ctx, gW):
        (md,) = ctx.saved_tensors
        plan = _plan()
        plan.set_stream(torch.cuda.current_stream(md.device).cuda_stream)
        g = gW.detach().to(torch.float64).contiguous()
        out = np.zeros(ctx.thetas.shape, dtype=np.float64)
        plan.check(plan.lib.gbp_zheng07_vjp_batched(
            plan.handle, _native.dptr_int(md.data_ptr()), md.shape[0], _native.pd(ctx.thetas),
            len(ctx.thetas), _native.dptr_int(g.data_ptr()), _native.GBP_MEM_DEVICE,
            _native.pd(out)))
        return torch.from_numpy(out).to(ctx.theta_device, ctx.theta_dtype), None


def weighted_pair_counts_batched(W, xyz, rbins, period):
    """Differentiable C[m, k] = sum_ij W_im W_jm [d_ij <= rbins[k]] for each column m of
    W (N, M), M <= 32: marked_npairs_3d(xyz, xyz, rbins, 1, period, W[:, m], W[:, m])."""
    rbins, box = _geometry(rbins, period)
    if W.dim() != 2 or W.shape[1] < 1 or W.shape[1] > 32:
        raise ValueError("W must be (N, M) with 1 <= M <= 32 weight columns")
    return WeightedPairCountsBatched.apply(W, xyz, rbins, box)


def zheng07_weights_batched(thetas, mass):
    """Per-halo Zheng07 mean occupations for each parameter vector: (N, M)."""
    return Zheng07WeightsBatched.apply(thetas, mass)


def hod_pair_counts_batched(thetas, halo_xyz, halo_mass, rbins, period):
    """Expected weighted pair counts C(theta_m) of a Zheng07 HOD for M parameter
    vectors at once (M <= 32): (M, nbins), differentiable in thetas (M, 5)."""
    return weighted_pair_counts_batched(zheng07_weights_batched(thetas, halo_mass), halo_xyz,
                                        rbins, period)
