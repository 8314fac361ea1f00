"""Seeded synthetic catalogues with the shapes of the benchmark workloads.

No survey or simulation data ships with this package; these generators stand
in for them.  Functional forms follow halotools:

* satellite radii from the NFW enclosed-mass profile, inverted numerically
  (empirical_models/phase_space_models/analytic_models/satellites/nfw/kernels/
  mass_profile.py:31 and mc_generate_nfw_radial_positions.py:112-130);
* Zheng07 mean occupations, <Ncen> = (1 + erf((log10 M - logMmin)/sigma))/2 and
  <Nsat> = ((M - 10^logM0)/10^logM1)^alpha for M > 10^logM0
  (empirical_models/occupation_models/zheng07_components.py:149-153, 455-470);
* periodic wrap of the final positions (empirical_models/factories/
  model_helpers.py:125).
"""
from __future__ import annotations

import math

import numpy as np


def _nfw_mass(x):
    return np.log1p(x) - x / (1.0 + x)


def nfw_radii(rng, conc, rvir):
    """Radii drawn from an NFW profile of concentration ``conc`` truncated at ``rvir``."""
    conc = np.asarray(conc, dtype=np.float64)
    u = rng.uniform(0, 1, conc.shape)
    target = u * _nfw_mass(conc)
    lo = np.zeros_like(conc)
    hi = conc.copy()
    for _ in range(40):  # bisection on m(x) = target, x = c r / rvir
        mid = 0.5 * (lo + hi)
        below = _nfw_mass(mid) < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return 0.5 * (lo + hi) / conc * rvir


def _isotropic(rng, n):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return d


def clustered_points(npts, lbox, ncen, logm_range=(11.0, 15.0), conc=8.0, rsd_sigma=5.0,
                     seed=0):
    """Centres uniform in the box with log10 M uniform in ``logm_range``;
    Poisson((M/1e12)^0.9) satellites per centre at NFW radii (virial radius
    (M/1e14)^(1/3) Mpc/h, fixed concentration); uniform fill to ``npts``;
    z displaced by N(0, rsd_sigma); wrapped into [0, lbox)."""
    rng = np.random.default_rng(seed)
    cen = rng.uniform(0, lbox, (ncen, 3))
    m = 10.0 ** rng.uniform(logm_range[0], logm_range[1], ncen)
    nsat = rng.poisson((m / 1e12) ** 0.9)
    room = max(npts - ncen, 0)
    host = np.repeat(np.arange(ncen), nsat)
    if len(host) > room:
        host = host[rng.permutation(len(host))[:room]]
    rvir = (m[host] / 1e14) ** (1.0 / 3.0)
    r = nfw_radii(rng, np.full(len(host), conc), rvir)
    sat = cen[host] + _isotropic(rng, len(host)) * r[:, None]
    nfill = npts - ncen - len(host)
    fill = rng.uniform(0, lbox, (max(nfill, 0), 3))
    pts = np.concatenate([cen, sat, fill])[:npts]
    pts[:, 2] += rng.normal(0, rsd_sigma, len(pts))
    return np.mod(pts, lbox)


def halo_table(nhalo, lbox, logm_range=(11.0, 15.0), slope=-0.9, seed=0):
    """Uniform halo positions, log10 M from dN/dlogM ~ M^slope, c = 10 (M/1e12)^-0.1."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, lbox, (nhalo, 3))
    a = slope * math.log(10.0)
    lo, hi = logm_range
    u = rng.uniform(0, 1, nhalo)
    # inverse CDF of p(logM) ~ exp(a logM) on [lo, hi]
    logm = np.log(np.exp(a * lo) + u * (np.exp(a * hi) - np.exp(a * lo))) / a
    mass = 10.0 ** logm
    conc = 10.0 * (mass / 1e12) ** -0.1
    return pos, mass, conc


def zheng07_mean_ncen(logm, logMmin, sigma_logM):
    from scipy.special import erf
    return 0.5 * (1.0 + erf((logm - logMmin) / sigma_logM))


def zheng07_mean_nsat(mass, logM0, logM1, alpha):
    m0, m1 = 10.0 ** logM0, 10.0 ** logM1
    out = np.zeros_like(mass, dtype=np.float64)
    ok = mass > m0
    out[ok] = ((mass[ok] - m0) / m1) ** alpha
    return out


def hod_mock(pos, mass, conc, lbox, theta, seed=0):
    """One Zheng07 realisation: Bernoulli centrals, Poisson satellites on NFW radii."""
    logMmin, sigma, logM0, logM1, alpha = theta
    rng = np.random.default_rng(seed)
    logm = np.log10(mass)
    ncen = zheng07_mean_ncen(logm, logMmin, sigma)
    nsat = zheng07_mean_nsat(mass, logM0, logM1, alpha)
    cen = pos[rng.uniform(0, 1, len(mass)) < ncen]
    ns = rng.poisson(nsat)
    host = np.repeat(np.arange(len(mass)), ns)
    rvir = (mass[host] / 1e14) ** (1.0 / 3.0)
    r = nfw_radii(rng, conc[host], rvir)
    sat = pos[host] + _isotropic(rng, len(host)) * r[:, None]
    return np.mod(np.concatenate([cen, sat]), lbox)


def hod_mocks_gpu(pos, mass, conc, lbox, thetas, seed=0, rvir=None, plan=None):
    """Many Zheng07 realisations drawn by the GPU kernels (``gbp_hod_mocks``).

    pos (N, 3), mass, conc (and optionally rvir, default (M / 1e14)^(1/3) as the
    other generators here) as numpy arrays or CUDA tensors; thetas (M, 5) of
    (logMmin, sigma_logM, logM0, logM1, alpha).  Returns (xyz, offsets): a float32
    CUDA tensor (total, 3) with mock m in rows [offsets[m], offsets[m+1]), and the
    numpy int64 offsets.  The draws are fixed by (seed, halo, mock, draw index).
    """
    import torch
    from . import _native
    dev = torch.device("cuda")

    def col(a):
        return torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()

    P, M, C = col(pos), col(mass), col(conc)
    R = col(rvir) if rvir is not None else (M / 1e14) ** (1.0 / 3.0)
    th = np.ascontiguousarray(np.atleast_2d(np.asarray(thetas, dtype=np.float64)))
    n = int(M.numel())
    plan = plan or _native.default_plan()
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    offs = np.zeros(len(th) + 1, dtype=np.int64)
    args = (plan.handle, _native.dptr_int(P.data_ptr()), _native.dptr_int(M.data_ptr()),
            _native.dptr_int(C.data_ptr()), _native.dptr_int(R.data_ptr()), n, _native.pd(th),
            len(th), float(lbox), int(seed) & 0xFFFFFFFFFFFFFFFF, _native.GBP_MEM_DEVICE)
    plan.check(plan.lib.gbp_hod_mocks(*args, None, 0, _native.pi64(offs)))
    out = torch.empty((max(int(offs[-1]), 1), 3), dtype=torch.float32, device=dev)
    if offs[-1] > 0:
        plan.check(plan.lib.gbp_hod_mocks(*args, _native.dptr_int(out.data_ptr()), int(offs[-1]),
                                          _native.pi64(offs)))
    return out[:int(offs[-1])], offs
