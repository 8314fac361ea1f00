"""Benchmark of the GB300 pair-counting engines.

One JSON line on stdout (rank 0).  Metric: in-range ordered pair evaluations
per second (pairs whose separation passes the outermost bin, read exactly
from the counts), on the configuration named in ``config.workload``:

  3d10m   (default) npairs_3d, 10,000,000 clustered points, L = 2000,
          30 log bins 0.5-50 (the largest single-GPU configuration)
  xyz2m   npairs_xy_z, 2,000,000 clustered points, L = 1000,
          20 log rp bins 0.1-30 x 40 linear pi bins 0-40
  3d100k  npairs_3d, 100,000 uniform points, L = 250, 15 log bins 0.1-20

A step is one full engine call (cell-list build + count + readback) on
device-resident inputs; L2 is flushed (256 MiB write) between steps outside
the timed events.  ``e2e`` repeats the step through the public drop-in API
from pinned host memory.

``--impl reference`` times halotools' own compiled engine
(``npairs_3d_engine`` / ``npairs_xy_z_engine``, through
``oracle/ref_driver.py``) on all host cores over the full periodic workload:
the K timed steps count K contiguous slabs of cell1 ids, together the whole
workload exactly once, with the mesh build added once.  Where the compiled
engines are missing, the C restatement of the engines (``oracle``) stands in
and the line says ``kind: "port"``.

The default run also measures the other configurations (``paths``) and
checks every one against the oracle at its full size (``parity``): integer
counts bit-exact, weighted sums and gradients as the relative error of each
bin against FP64.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "3d10m": dict(kind="3d", n=10_000_000, L=2000.0, ncen=1_000_000, logm=(11.0, 15.5),
                  bins=np.logspace(np.log10(0.5), np.log10(50), 30),
                  desc="npairs_3d, 10,000,000 clustered points, periodic L = 2000, "
                       "30 log bins 0.5-50"),
    "xyz2m": dict(kind="xyz", n=2_000_000, L=1000.0, ncen=200_000, logm=(11.0, 15.0),
                  bins=np.logspace(-1, np.log10(30), 20), bins2=np.linspace(0, 40, 40),
                  desc="npairs_xy_z, 2,000,000 clustered points, periodic L = 1000, "
                       "20 log rp bins 0.1-30 x 40 linear pi bins 0-40"),
    "3d100k": dict(kind="3d", n=100_000, L=250.0, ncen=0, bins=np.logspace(-1, np.log10(20), 15),
                   desc="npairs_3d, 100,000 uniform points, periodic L = 250, "
                        "15 log bins 0.1-20"),
}
REF_ORACLE = "oracle (C restatement of the reference engines, pinned to their golden vectors)"


def make_points(w, seed=2):
    from halotools_gb300 import mocks
    if w["ncen"] == 0:
        return np.random.default_rng(0).uniform(0, w["L"], (w["n"], 3))
    return mocks.clustered_points(w["n"], w["L"], w["ncen"], logm_range=w["logm"], seed=seed)


def in_range(kind, out):
    return int(out[-1] if kind == "3d" else out[-1, -1])


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def call_device(plan, kind, xd, n, w, box, out):
    """One engine call on device-resident positions (sample2 is sample1)."""
    from halotools_gb300 import _native as N
    ptr = xd.data_ptr()
    if kind == "3d":
        rc = plan.lib.gbp_npairs_3d(plan.handle, ptr, n, ptr, n, N.pd(w["bins"]), len(w["bins"]),
                                    N.pd(box), 1, N.GBP_MEM_DEVICE, N.pi64(out))
    else:
        rc = plan.lib.gbp_npairs_xy_z(plan.handle, ptr, n, ptr, n, N.pd(w["bins"]),
                                      len(w["bins"]), N.pd(w["bins2"]), len(w["bins2"]),
                                      N.pd(box), 1, N.GBP_MEM_DEVICE, N.pi64(out))
    plan.check(rc)


def replica_throughput(units_per_rank, seconds, device=None):
    """Whole-job throughput of N independent replicas (no data-path collective):
    every rank processed ``units_per_rank`` units and the job took the slowest
    rank's time.  Returns (units per second over all ranks, max seconds)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    if world > 1:
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device or "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return units_per_rank * world / seconds, seconds


# ---------------------------------------------------------------------------
# the CPU reference (halotools' compiled engines) -- also the CPU leg's source
# ---------------------------------------------------------------------------

def reference_run(w, x, steps, warmup, nslabs, threads, full_call):
    """Time the reference engine over ``steps`` slabs of the workload (after
    ``warmup`` untimed slabs).  Returns a dict: rate, seconds, counts of the
    whole workload when the timed slabs covered it whole, and what was run."""
    from oracle import ref_driver as R
    kind, bins, bins2, L = w["kind"], w["bins"], w.get("bins2"), w["L"]
    nslabs = max(1, int(nslabs))
    res = {"cores": threads}
    if R.engines_available():
        sc = R.SlabCounter(kind, x, x, bins, bins2, L, threads, nslabs)
        nslabs = sc.nslabs
        try:
            for k in range(warmup):
                sc.count(k)
            tot, t = None, 0.0
            for k in range(steps):
                c, dt = sc.count(k)
                tot = c if tot is None else tot + c
                t += dt
        finally:
            sc.close()
        setup = sc.setup_s * min(1.0, steps / nslabs)
        res.update(kind="reference", setup_s=sc.setup_s,
                   sample=("full periodic workload (%d points): halotools' compiled %s on %d "
                           "processes; the %d timed steps count %d contiguous slabs of the %d "
                           "cell1 ids%s, mesh build and sort (%.2f s) added %s" %
                           (len(x), "npairs_3d_engine" if kind == "3d" else "npairs_xy_z_engine",
                            threads, steps, min(steps, nslabs), sc.ncells,
                            " (the whole workload once)" if steps == nslabs else "",
                            sc.setup_s, "once" if steps >= nslabs else "pro rata")))
    else:
        from oracle import oracle
        edges = np.linspace(0.0, L, nslabs + 1)
        edges[-1] = np.inf

        def slab(k):
            k %= nslabs
            sub = np.ascontiguousarray(x[(x[:, 0] >= edges[k]) & (x[:, 0] < edges[k + 1])])
            t0 = time.perf_counter()
            c = (oracle.npairs_3d(sub, x, bins, period=L, num_threads=threads) if kind == "3d"
                 else oracle.npairs_xy_z(sub, x, bins, bins2, period=L, num_threads=threads))
            return c, time.perf_counter() - t0
        for k in range(warmup):
            slab(k)
        tot, t = None, 0.0
        for k in range(steps):
            c, dt = slab(k)
            tot = c if tot is None else tot + c
            t += dt
        setup = 0.0
        res.update(kind="port", sample=(
            "full periodic workload (%d points): the C restatement of the engines on %d threads "
            "(the reference's compiled engines are not available here); the %d timed steps count "
            "%d x-slabs of sample 1 against all of sample 2" % (len(x), threads, steps,
                                                                min(steps, nslabs))))
    pairs = in_range(kind, tot)
    seconds = t + setup
    res.update(value=pairs / seconds, seconds=seconds, pairs=pairs, nslabs=nslabs)
    if steps % nslabs == 0:
        res["counts"] = tot // (steps // nslabs)
    if full_call and res["kind"] == "reference":
        t0 = time.perf_counter()
        c = R.full_call(kind, x, x, bins, bins2, L, threads)
        dt = time.perf_counter() - t0
        res["full_call"] = {"seconds": dt, "pairs_per_s": in_range(kind, c) / dt,
                            "what": "one call structured as the reference front-end (mesh, "
                                    "partial over the caller's columns, Pool(%d).map over the "
                                    "cell1 ranges)" % threads,
                            "same_counts_as_slabs": bool("counts" in res and
                                                         np.array_equal(c, res["counts"]))}
    return res


def cpu_leg(args, w, x, steps=16):
    """The reference engine on the whole workload in a fresh process (no fork
    after CUDA initialisation): its rate and its counts."""
    tmp = tempfile.mkdtemp(prefix="gbp_cpu_")
    try:
        pf, cf = os.path.join(tmp, "points.npy"), os.path.join(tmp, "counts.npy")
        np.save(pf, x)
        cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload",
               args.workload, "--steps", str(steps), "--warmup", "0", "--slabs", str(steps),
               "--no-full-call", "--points-file", pf, "--counts-file", cf]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=1800)
        if r.returncode != 0:
            raise RuntimeError("CPU reference leg failed: " + r.stderr[-400:])
        line = json.loads(r.stdout.strip().splitlines()[-1])
        counts = np.load(cf) if os.path.exists(cf) else None
        return line, counts
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


# ---------------------------------------------------------------------------
# the other configurations, each timed on the GPU and checked at full size
# ---------------------------------------------------------------------------

def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_gpu(stream, fn, reps=3):
    import torch
    fn()
    t = []
    for _ in range(reps):
        a, b = _events()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        t.append(a.elapsed_time(b) / 1e3)
    return float(np.median(t))


def extra_small(dev, threads, check, name):
    """A plain workload (3d100k: config 1; xyz2m: config 2) timed on device-resident
    inputs and compared with the oracle over the whole workload."""
    import torch
    from halotools_gb300 import _native as N
    w = WORKLOADS[name]
    x = make_points(w)
    xd = torch.from_numpy(x).cuda(dev)
    plan = N.Plan(dev)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    box = np.array([w["L"]] * 3)
    shape = len(w["bins"]) if w["kind"] == "3d" else (len(w["bins"]), len(w["bins2"]))
    out = np.zeros(shape, dtype=np.int64)
    t = _time_gpu(stream, lambda: call_device(plan, w["kind"], xd, len(x), w, box, out))
    pairs = in_range(w["kind"], out)
    res = {"workload": w["desc"], "gpu_ms": t * 1e3, "gpu_pairs_per_s": pairs / t,
           "in_range_pairs": pairs}
    if check:
        from oracle import oracle, parity
        t0 = time.perf_counter()
        want = (oracle.npairs_3d(x, x, w["bins"], period=w["L"], num_threads=threads)
                if w["kind"] == "3d" else
                oracle.npairs_xy_z(x, x, w["bins"], w["bins2"], period=w["L"],
                                   num_threads=threads))
        res["cpu_oracle_pairs_per_s"] = in_range(w["kind"], want) / (time.perf_counter() - t0)
        res["parity"] = dict(parity.exact(out, want), vs=REF_ORACLE, size="full")
    return res


def extra_batched(dev, threads, check, reps=3, nhalo=1_000_000, check_mocks=None):
    """Config 3: 64 Zheng07 mocks on a 1M-halo table (L = 1000, float32), npairs_3d
    15 log bins 0.1-20: one batched launch vs one plain call per mock.  The mocks are
    drawn on the GPU (gbp_hod_mocks) straight into the batched counter's input; the
    draw time is reported beside the counts.  ``nhalo`` scales the halo table (same
    mass function and box); ``check_mocks`` limits the oracle check to that many
    mocks, spread over the 64."""
    import torch
    from halotools_gb300 import BatchedCounter, mocks
    from halotools_gb300 import _native as N
    L = 1000.0
    pos, mass, conc = mocks.halo_table(nhalo, L, seed=11)
    rng = np.random.default_rng(12)
    lmin = rng.uniform(11.8, 12.4, 64)
    thetas = np.stack([lmin, rng.uniform(0.2, 0.5, 64), lmin, lmin + 1.3,
                       rng.uniform(0.9, 1.1, 64)], axis=1)
    xyz, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, thetas, seed=13)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xyz, offs = mocks.hod_mocks_gpu(pos, mass, conc, L, thetas, seed=13)
    torch.cuda.synchronize()
    t_pop = time.perf_counter() - t0
    rb = np.logspace(-1, np.log10(20), 15)
    bc = BatchedCounter(dev, graph=True, autotune=True)
    stream = torch.cuda.current_stream(dev)
    bc.plan.set_stream(stream.cuda_stream)
    for _ in range(2):
        out = bc.count_device(xyz, offs, rb, L)
    pairs = int(out[:, -1].sum())
    t = []
    for _ in range(reps):
        a, b = _events()
        a.record(stream)
        bc.count_device(xyz, offs, rb, L)
        b.record(stream)
        torch.cuda.synchronize()
        t.append(a.elapsed_time(b) / 1e3)
    tb = float(np.median(t))
    st = bc.stats()
    # plain path: one npairs_3d call per mock (FP64 positions on the device)
    plan = N.Plan(dev)
    plan.set_stream(stream.cuda_stream)
    x64 = xyz.double()
    box = np.array([L] * 3)
    o1 = np.zeros(len(rb), dtype=np.int64)

    def plain_all():
        tot = 0
        for m in range(len(offs) - 1):
            lo, hi = int(offs[m]), int(offs[m + 1])
            ptr = x64.data_ptr() + lo * 24
            plan.check(plan.lib.gbp_npairs_3d(plan.handle, N.dptr_int(ptr), hi - lo, N.dptr_int(ptr),
                                              hi - lo, N.pd(rb), len(rb), N.pd(box), 1,
                                              N.GBP_MEM_DEVICE, N.pi64(o1)))
            tot += int(o1[-1])
        return tot
    plain_all()
    a, b = _events()
    a.record(stream)
    tot = plain_all()
    b.record(stream)
    torch.cuda.synchronize()
    tp = a.elapsed_time(b) / 1e3
    assert tot == pairs
    res = {"mocks": len(offs) - 1, "galaxies": int(offs[-1]),
           "galaxies_per_mock": [int(np.min(np.diff(offs))), int(np.max(np.diff(offs)))],
           "in_range_pairs": pairs, "batched_pairs_per_s": pairs / tb, "batched_ms": tb * 1e3,
           "plain_pairs_per_s": pairs / tp, "plain_ms": tp * 1e3, "speedup_vs_plain": tp / tb,
           "reach": st["reach"], "graph": True, "autotune": True,
           "population_ms": t_pop * 1e3,
           "population": "64 Zheng07 draws on the GPU from host halo arrays (two passes)"}
    res["halos"] = nhalo
    if check:
        from oracle import oracle
        xs = xyz.cpu().numpy().astype(np.float64)  # float32 upcast exactly, as the engine does
        nm = len(offs) - 1
        which = list(range(nm)) if not check_mocks else \
            sorted(set(np.linspace(0, nm - 1, check_mocks).round().astype(int).tolist()))
        bad = [m for m in which
               if not np.array_equal(out[m], oracle.npairs_3d(
                   xs[offs[m]:offs[m + 1]], xs[offs[m]:offs[m + 1]], rb, period=L,
                   num_threads=threads))]
        res["parity"] = {"exact": not bad, "mocks_checked": which, "mismatched_mocks": bad,
                         "vs": REF_ORACLE + ", per mock",
                         "size": "full" if len(which) == nm else "full mocks, %d of %d" % (
                             len(which), nm)}
    return res


def _hod_theta_draws(m, seed=31):
    rng = np.random.default_rng(seed)
    lmin = rng.uniform(11.8, 12.4, m)
    return np.stack([lmin, rng.uniform(0.2, 0.5, m), lmin, lmin + 1.3, rng.uniform(0.9, 1.1, m)],
                    axis=1)


def _fp64_hod(pos, mass, theta, rb, L, threads):
    """FP64 C_k and dC_k/dtheta (nb, 5) of the Zheng07-weighted auto count."""
    from oracle import oracle, parity
    w = parity.zheng07_fp64(theta, mass)
    S = oracle.weighted_per_object_3d(pos, w, rb, L, threads)
    return parity.weighted_counts_and_jacobian(S, w, parity.zheng07_jacobian_fp64(theta, mass))


def _jac_summary(got, want):
    """Per bin: the largest |dC_k/dtheta_p| error over the 5 parameters relative
    to the bin's largest |dC_k/dtheta_p|."""
    got, want = np.asarray(got), np.asarray(want)
    scale = np.maximum(np.abs(want).max(axis=-1), 1e-300)
    r = np.abs(got - want).max(axis=-1) / scale
    return [float(v) for v in r.reshape(-1)]


def extra_differentiable(dev, threads, check, reps=3):
    """Config 4: 2M halos in L = 1000, Zheng07 weights at theta = (12, 0.3, 12, 13.3, 1),
    weighted npairs_3d over 20 log bins 0.1-30, forward + hand-written backward."""
    import torch
    from halotools_gb300 import differentiable as D, mocks
    L = 1000.0
    pos, mass, _ = mocks.halo_table(2_000_000, L, seed=21)
    rb = np.logspace(-1, np.log10(30), 20)
    xd = torch.from_numpy(pos).cuda(dev)
    md = torch.from_numpy(mass).cuda(dev)
    gbar = torch.ones(len(rb), dtype=torch.float64, device=f"cuda:{dev}")
    stream = torch.cuda.current_stream(dev)
    theta = np.array([12.0, 0.3, 12.0, 13.3, 1.0])

    def step():
        th = torch.tensor(theta, dtype=torch.float64, device=f"cuda:{dev}", requires_grad=True)
        C = D.hod_pair_counts(th, xd, md, rb, L)
        (C * gbar).sum().backward()
        return C, th.grad
    step()
    t = []
    for _ in range(reps):
        a, b = _events()
        a.record(stream)
        C, g = step()
        b.record(stream)
        torch.cuda.synchronize()
        t.append(a.elapsed_time(b) / 1e3)
    tfb = float(np.median(t))
    import halotools_gb300 as H
    pairs = int(H.npairs_3d(pos, pos, rb, period=L)[-1])
    res = {"halos": len(pos), "in_range_pairs": pairs, "fwd_bwd_ms": tfb * 1e3,
           "pair_evals_per_s": 2 * pairs / tfb, "passes": 2}
    if check:
        from oracle import parity
        th = torch.tensor(theta, dtype=torch.float64, device=f"cuda:{dev}", requires_grad=True)
        C = D.hod_pair_counts(th, xd, md, rb, L)
        jac = np.stack([torch.autograd.grad(C[k], th, retain_graph=True)[0].cpu().numpy()
                        for k in range(len(rb))])
        C64, J64 = _fp64_hod(pos, mass, theta, rb, L, threads)
        fw = parity.rel_summary(C.detach().cpu().numpy(), C64, 1e-6)
        jr = _jac_summary(jac, J64)
        res["parity"] = {"forward": fw,
                         "dC_dtheta": {"max_rel_err": max(jr), "tol": 1e-5, "ok": max(jr) <= 1e-5,
                                       "rel_err_per_bin": jr,
                                       "what": "per bin, max over the 5 parameters of "
                                               "|GPU - FP64| / max |FP64| (20 backward passes)"},
                         "vs": "FP64 oracle: per-halo neighbour weight sums over the cell walk "
                               "(oracle.weighted_per_object_3d) with the analytic Zheng07 "
                               "Jacobian", "size": "full"}
        res["parity"]["ok"] = bool(fw["ok"] and res["parity"]["dC_dtheta"]["ok"])
    return res


def extra_batched_adjoint(dev, threads, check, reps=3, m=16):
    """Batched + adjoint (the configurations' target): 16 Zheng07 parameter draws on the
    config-4 halo table (2M halos, L = 1000; draws as config 3: logMmin ~ U[11.8, 12.4],
    sigma_logM ~ U[0.2, 0.5], logM0 = logMmin, logM1 = logMmin + 1.3, alpha ~ U[0.9, 1.1]),
    weighted npairs_3d over 20 log bins 0.1-30 and dC/dtheta for every draw: one forward
    pass over all draws and one adjoint pass per 8 draws, against the same 16 forward +
    backward steps run one draw at a time on the same GPU."""
    import torch
    from halotools_gb300 import differentiable as D, mocks
    L = 1000.0
    pos, mass, _ = mocks.halo_table(2_000_000, L, seed=21)
    rb = np.logspace(-1, np.log10(30), 20)
    th = _hod_theta_draws(m)
    xd = torch.from_numpy(pos).cuda(dev)
    md = torch.from_numpy(mass).cuda(dev)
    gbar = torch.ones((m, len(rb)), dtype=torch.float64, device=f"cuda:{dev}")
    stream = torch.cuda.current_stream(dev)

    def batched():
        T = torch.tensor(th, dtype=torch.float64, device=f"cuda:{dev}", requires_grad=True)
        C = D.hod_pair_counts_batched(T, xd, md, rb, L)
        (C * gbar).sum().backward()
        return C, T.grad

    def single():
        out = []
        for k in range(m):
            t1 = torch.tensor(th[k], dtype=torch.float64, device=f"cuda:{dev}",
                              requires_grad=True)
            c1 = D.hod_pair_counts(t1, xd, md, rb, L)
            (c1 * gbar[k]).sum().backward()
            out.append(t1.grad)
        return out

    def timed(fn):
        fn()
        t = []
        for _ in range(reps):
            a, b = _events()
            a.record(stream)
            r = fn()
            b.record(stream)
            torch.cuda.synchronize()
            t.append(a.elapsed_time(b) / 1e3)
        return float(np.median(t)), r
    tb, (C, G) = timed(batched)
    ts, g1 = timed(single)

    def forward_only():
        with torch.no_grad():
            T = torch.tensor(th, dtype=torch.float64, device=f"cuda:{dev}")
            return D.hod_pair_counts_batched(T, xd, md, rb, L)
    tf, _ = timed(forward_only)
    import halotools_gb300 as H
    pairs = int(H.npairs_3d(pos, pos, rb, period=L)[-1])
    gerr = max(float(np.max(np.abs(G[k].cpu().numpy() - g1[k].cpu().numpy()) /
                            np.abs(g1[k].cpu().numpy()).max())) for k in range(m))
    res = {"halos": len(pos), "draws": m, "in_range_pairs_per_draw": pairs,
           "batched_ms": tb * 1e3, "batched_forward_ms": tf * 1e3, "single_draws_ms": ts * 1e3,
           "speedup": ts / tb,
           "batched_pair_evals_per_s": 2 * m * pairs / tb,
           "single_pair_evals_per_s": 2 * m * pairs / ts,
           "max_rel_dtheta_diff_vs_single": gerr, "adjoint_passes": -(-m // D._ADJ_CH)}
    if check:
        from oracle import parity
        Cn, Gn = C.detach().cpu().numpy(), G.cpu().numpy()
        per = {}
        for k in (0, m - 1):  # two of the draws against FP64 (a full FP64 pass each)
            C64, J64 = _fp64_hod(pos, mass, th[k], rb, L, threads)
            g64 = J64.sum(axis=0)  # the bench's loss: sum over bins (gbar = 1)
            per["draw_%d" % k] = {
                "forward": parity.rel_summary(Cn[k], C64, 1e-6),
                "dL_dtheta_rel_err": [float(v) for v in np.abs(Gn[k] - g64) / np.abs(g64).max()]}
        ok = all(v["forward"]["ok"] and max(v["dL_dtheta_rel_err"]) <= 1e-5 for v in per.values())
        res["parity"] = dict(per, ok=ok, vs="FP64 oracle (oracle.weighted_per_object_3d + "
                                             "analytic Zheng07 Jacobian), draws 0 and 15",
                             size="full")
    return res


def batched_step_only(k, m=16):
    """The batched step of batched_adjoint_2m alone, ``k`` times: 16 Zheng07 draws
    on 2M halos, forward over all draws and dC/dtheta; CUDA-event times of the
    weights, the forward and the backward of each step."""
    import torch
    from halotools_gb300 import differentiable as D, mocks
    L = 1000.0
    pos, mass, _ = mocks.halo_table(2_000_000, L, seed=21)
    rb = np.logspace(-1, np.log10(30), 20)
    th = _hod_theta_draws(m)
    xd = torch.from_numpy(pos).cuda()
    md = torch.from_numpy(mass).cuda()
    gbar = torch.ones((m, len(rb)), dtype=torch.float64, device="cuda")
    steps = []
    for _ in range(k):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record()
        T = torch.tensor(th, dtype=torch.float64, device="cuda", requires_grad=True)
        W = D.zheng07_weights_batched(T, md)
        e[1].record()
        C = D.weighted_pair_counts_batched(W, xd, rb, L)
        e[2].record()
        (C * gbar).sum().backward()
        e[3].record()
        torch.cuda.synchronize()
        steps.append({"weights_ms": e[0].elapsed_time(e[1]), "forward_ms": e[1].elapsed_time(e[2]),
                      "backward_ms": e[2].elapsed_time(e[3]), "step_ms": e[0].elapsed_time(e[3])})
    return {"path": "batched_adjoint_2m step", "draws": m, "steps": steps}


_POINTS_10M = []


def points_10m():
    """The 10M-point clustered sample of config 5 (generated once per process)."""
    if not _POINTS_10M:
        _POINTS_10M.append(make_points(WORKLOADS["3d10m"]))
    return _POINTS_10M[0]


def extra_marked_10m(dev, threads, check):
    """Config 5: marked counts with the product weight function (id 1), 30 log bins
    0.5-50, on 10M clustered points (L = 2000).  Marks: a lognormal(0, 0.5) and a
    uniform[0, 1) component, both channels in one launch; then 8 random-mark draws
    (permutations of the lognormal component, as marked_tpcf's randomisation) in one
    launch against 8 single-channel calls.  Parity: both components against the FP64
    oracle over the whole sample."""
    import torch
    from halotools_gb300 import _native as N
    w = WORKLOADS["3d10m"]
    x = points_10m()
    n = len(x)
    rng = np.random.default_rng(51)
    comp = np.stack([rng.lognormal(0.0, 0.5, n), rng.uniform(0.0, 1.0, n)], axis=1)
    draws = np.stack([rng.permutation(comp[:, 0]) for _ in range(8)], axis=1)
    xd = torch.from_numpy(x).cuda(dev)
    cd = torch.from_numpy(np.ascontiguousarray(comp)).cuda(dev)
    dd = torch.from_numpy(np.ascontiguousarray(draws)).cuda(dev)
    cols = [dd[:, c].contiguous() for c in range(8)]
    plan = N.Plan(dev)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    box = np.array([w["L"]] * 3)
    rb = w["bins"]
    o2 = np.zeros((2, len(rb)))
    o8 = np.zeros((8, len(rb)))
    o1 = np.zeros(len(rb))

    def channels(wt, out):
        plan.check(plan.lib.gbp_marked_npairs_3d_channels(
            plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, wt.data_ptr(), wt.data_ptr(),
            wt.shape[1], N.pd(rb), len(rb), N.pd(box), 1, N.GBP_MEM_DEVICE, N.pd(out)))

    def separate():
        for col in cols:
            plan.check(plan.lib.gbp_marked_npairs_3d(
                plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, col.data_ptr(), col.data_ptr(), 1,
                1, N.pd(rb), len(rb), N.pd(box), 1, N.GBP_MEM_DEVICE, N.pd(o1)))
    t2 = _time_gpu(stream, lambda: channels(cd, o2))
    t8 = _time_gpu(stream, lambda: channels(dd, o8))
    t8s = _time_gpu(stream, separate, reps=1)
    np.testing.assert_allclose(o8[-1], o1, rtol=1e-6)  # last draw: one launch == separate call
    ones = np.zeros(len(rb), dtype=np.int64)
    call_device(plan, "3d", xd, n, w, box, ones)
    pairs = int(ones[-1])
    res = {"points": n, "in_range_pairs": pairs, "weight_func_id": 1,
           "two_components_one_launch_ms": t2 * 1e3,
           "two_components_pair_evals_per_s": 2 * pairs / t2,
           "eight_draws_one_launch_ms": t8 * 1e3, "eight_draws_separate_ms": t8s * 1e3,
           "eight_draws_speedup": t8s / t8, "eight_draws_pair_evals_per_s": 8 * pairs / t8}
    if check:
        from oracle import oracle, parity
        per = {}
        t0 = time.perf_counter()
        for c in range(2):
            want = oracle.marked_npairs_3d(x, x, rb, 1, period=w["L"], weights1=comp[:, c],
                                           weights2=comp[:, c], num_threads=threads)
            per["component_%d" % c] = parity.rel_summary(o2[c], want, 1e-6)
        res["cpu_oracle_pair_evals_per_s"] = 2 * pairs / (time.perf_counter() - t0)
        res["parity"] = dict(per, ok=all(v["ok"] for v in per.values()),
                             vs="FP64 oracle marked_npairs_3d(id 1) per component", size="full")
    return res


def extra_s_mu_10m(dev, threads, check):
    """Config 5: npairs_s_mu, 30 log s bins 0.5-50 x 20 linear mu bins (21 edges 0-1),
    line of sight z, on 10M clustered points (L = 2000); exact against the oracle."""
    import torch
    from halotools_gb300 import _native as N
    w = WORKLOADS["3d10m"]
    x = points_10m()
    n = len(x)
    sb = w["bins"]
    mu = np.linspace(0.0, 1.0, 21)
    mup = np.sort(np.sin(np.arccos(mu)))
    xd = torch.from_numpy(x).cuda(dev)
    plan = N.Plan(dev)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    box = np.array([w["L"]] * 3)
    out = np.zeros((len(sb), len(mu)), dtype=np.int64)

    def run():
        plan.check(plan.lib.gbp_npairs_s_mu(plan.handle, xd.data_ptr(), n, xd.data_ptr(), n,
                                            N.pd(sb), len(sb), N.pd(mup), len(mup), N.pd(box), 1,
                                            N.GBP_MEM_DEVICE, N.pi64(out)))
    tg = _time_gpu(stream, run)
    pairs = int(out[-1, -1])
    res = {"points": n, "gpu_ms": tg * 1e3, "gpu_pairs_per_s": pairs / tg,
           "recheck_fraction": plan.stats()["recheck_pairs"] / pairs,
           "stats": {k: plan.stats()[k] for k in ("ms_build", "ms_count", "block", "reach",
                                                  "recheck_pairs")}}
    if check:
        from oracle import oracle, parity
        t0 = time.perf_counter()
        want = oracle.npairs_s_mu(x, x, sb, mu, period=w["L"], num_threads=threads)
        res["cpu_oracle_pairs_per_s"] = pairs / (time.perf_counter() - t0)
        res["parity"] = dict(parity.exact(out, want), vs=REF_ORACLE, size="full")
    return res


def extra_siblings_10m(dev, threads, check):
    """The sibling engines on the config-5 sample (10M clustered points, L = 2000):
    marked_npairs_xy_z (id 1, lognormal marks; rp 30 log bins 0.5-50 x pi 26 linear
    edges 0-50) and weighted_npairs_s_mu (30 x 21 edges) through the C ABI on device
    memory; counts_in_cylinders (rp 2, pi 10) and spherical_isolation (r 1) through
    their host-memory front-ends (the count kernel's own time reported beside the
    call).  Parity for these is in the test suite (golden vectors of halotools' own
    engines, and the oracle); this path only times them."""
    import torch
    import halotools_gb300 as H
    from halotools_gb300 import _native as N
    w = WORKLOADS["3d10m"]
    x = points_10m()
    n = len(x)
    rng = np.random.default_rng(5)
    mk = rng.lognormal(0.0, 0.5, n)
    rp = w["bins"]
    pi = np.linspace(0.0, 50.0, 26)
    mu = np.linspace(0.0, 1.0, 21)
    mup = np.sort(np.sin(np.arccos(mu)))
    xd = torch.from_numpy(x).cuda(dev)
    wd = torch.from_numpy(np.ascontiguousarray(mk)).cuda(dev)
    plan = N.Plan(dev)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    box = np.array([w["L"]] * 3)
    res = {"points": n}
    out = np.zeros((len(rp), len(pi)))

    def mxyz():
        plan.check(plan.lib.gbp_marked_npairs_xy_z(
            plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, wd.data_ptr(), wd.data_ptr(), 1, 1,
            N.pd(rp), len(rp), N.pd(pi), len(pi), N.pd(box), 1, N.GBP_MEM_DEVICE, N.pd(out)))
    t = _time_gpu(stream, mxyz)
    cnt = np.zeros((len(rp), len(pi)), dtype=np.int64)
    plan.check(plan.lib.gbp_npairs_xy_z(plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, N.pd(rp),
                                        len(rp), N.pd(pi), len(pi), N.pd(box), 1,
                                        N.GBP_MEM_DEVICE, N.pi64(cnt)))
    pairs = int(cnt[-1, -1])
    res["marked_xy_z"] = {"ms": t * 1e3, "in_range_pairs": pairs, "pairs_per_s": pairs / t}
    c2 = np.zeros((len(rp), len(mup)), dtype=np.int64)
    w2 = np.zeros((len(rp), len(mup)))

    def wsmu():
        plan.check(plan.lib.gbp_weighted_npairs_s_mu(
            plan.handle, xd.data_ptr(), n, xd.data_ptr(), n, wd.data_ptr(), wd.data_ptr(),
            N.pd(rp), len(rp), N.pd(mup), len(mup), N.pd(box), 1, N.GBP_MEM_DEVICE, N.pi64(c2),
            N.pd(w2)))
    t = _time_gpu(stream, wsmu)
    res["weighted_s_mu"] = {"ms": t * 1e3, "in_range_pairs": int(c2[-1, -1]),
                            "pairs_per_s": int(c2[-1, -1]) / t,
                            "recheck_pairs": plan.stats()["recheck_pairs"]}
    # host-memory front-ends: wall time of the call, and the kernel's event time
    dp = H.default_plan(dev)
    for name, fn in (("counts_in_cylinders", lambda: H.counts_in_cylinders(x, x, 2.0, 10.0,
                                                                            period=w["L"])),
                     ("spherical_isolation", lambda: H.spherical_isolation(x, x, 1.0,
                                                                            period=w["L"]))):
        fn()
        t0 = time.perf_counter()
        r = fn()
        dt = time.perf_counter() - t0
        st = dp.stats()
        res[name] = {"call_ms": dt * 1e3, "ms_count": st["ms_count"], "ms_build": st["ms_build"],
                     "points_per_s": n / dt, "result_sum": int(np.sum(r))}
    return res


EXTRAS = {
    "3d100k": lambda dev, threads, check: extra_small(dev, threads, check, "3d100k"),
    "xyz2m": lambda dev, threads, check: extra_small(dev, threads, check, "xyz2m"),
    "batched_hod64": extra_batched,
    # the same 64 draws on a 10M-halo table: 0.5-3M galaxies per mock, the counts
    # the configuration quotes (the stated 1M-halo table gives 0.08-0.31M)
    "batched_hod64_10mhalos": lambda dev, threads, check: extra_batched(
        dev, threads, check, nhalo=10_000_000, check_mocks=4),
    "differentiable_2m": extra_differentiable,
    "batched_adjoint_2m": extra_batched_adjoint,
    "marked_10m": extra_marked_10m,
    "s_mu_10m": extra_s_mu_10m,
    "siblings_10m": extra_siblings_10m,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="3d10m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other configurations (paths)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size oracle checks")
    ap.add_argument("--only-path", choices=sorted(EXTRAS),
                    help="run one comparison path alone and print its JSON (profiling)")
    ap.add_argument("--batched-step", type=int, default=0, metavar="K",
                    help="run only the batched + adjoint step of batched_adjoint_2m K times "
                         "and print its timings (profiling)")
    # the reference arm's own options
    ap.add_argument("--slabs", type=int, default=0,
                    help="reference arm: slabs of cell1 ids (default: --steps, at most 64)")
    ap.add_argument("--no-full-call", action="store_true",
                    help="reference arm: skip the one reference-structured full call")
    ap.add_argument("--points-file", help="reference arm: read the points from this .npy")
    ap.add_argument("--counts-file", help="reference arm: save the whole workload's counts")
    args = ap.parse_args()
    threads = os.cpu_count() or 1
    if args.batched_step:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(batched_step_only(args.batched_step)))
        return 0
    if args.only_path:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"path": args.only_path,
                          **EXTRAS[args.only_path](0, threads, not args.no_parity)},
                         default=lambda o: o.tolist()))
        return 0
    w = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cfg = {"workload": args.workload, "desc": w["desc"],
           "engine": "npairs_" + ("3d" if w["kind"] == "3d" else "xy_z"),
           "points": w["n"], "box": w["L"], "bins": len(w["bins"]),
           "bins2": len(w["bins2"]) if "bins2" in w else None, "autocorr": True, "periodic": True,
           "l2": "flushed between steps (256 MiB write, outside the timed events)"}
    metric = "pair evals/s (in-range ordered pairs, exact counts)"

    if args.impl == "reference":
        if rank != 0:
            return 0
        x = np.load(args.points_file) if args.points_file else make_points(w)
        nslabs = args.slabs or max(1, min(args.steps, 64))
        r = reference_run(w, x, args.steps, args.warmup, nslabs, threads,
                          full_call=not args.no_full_call)
        if args.counts_file and "counts" in r:
            np.save(args.counts_file, r["counts"])
        line = {"impl": "reference", "metric": metric, "value": r["value"], "unit": "pairs/s",
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": r["seconds"] / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg,
                "cpu_baseline": {"value": r["value"], "unit": "pairs/s", "cores": threads,
                                 "kind": r["kind"], "sample": r["sample"]},
                "e2e": {"value": r["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "pairs_counted": r["pairs"], "slabs": r["nslabs"]}
        if "full_call" in r:
            line["full_call"] = r["full_call"]
        print(json.dumps(line))
        return 0

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    import halotools_gb300 as H
    from halotools_gb300 import _native as N

    x = make_points(w)
    box = np.array([w["L"]] * 3)
    n = len(x)
    xd = torch.from_numpy(x).to(f"cuda:{dev}")
    plan = N.Plan(dev)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    out = np.zeros(len(w["bins"]) if w["kind"] == "3d" else (len(w["bins"]), len(w["bins2"])),
                   dtype=np.int64)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    for _ in range(max(args.warmup, 3)):
        call_device(plan, w["kind"], xd, n, w, box, out)
    pairs_step = in_range(w["kind"], out)
    counts_gpu = out.copy()
    fp32_peak = plan.fp32_peak_tflops()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    count_ms = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            call_device(plan, w["kind"], xd, n, w, box, out)
            ev[k][1].record(stream)
            count_ms.append(plan.stats()["ms_count"])
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1e3
    value, total_s = replica_throughput(pairs_step * args.steps, total_s, device=f"cuda:{dev}")
    st = plan.stats()
    assert np.array_equal(out, counts_gpu), "counts changed between steps"

    # e2e: public drop-in API from pinned host memory, result back on the host
    xp = torch.from_numpy(x).pin_memory().numpy()
    f = (lambda: H.npairs_3d(xp, xp, w["bins"], period=w["L"])) if w["kind"] == "3d" else \
        (lambda: H.npairs_xy_z(xp, xp, w["bins"], w["bins2"], period=w["L"]))
    for _ in range(2):
        f()
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = f()
        e2e_t.append(time.perf_counter() - t0)
    assert np.array_equal(r, counts_gpu)
    st_e2e = H.default_plan(dev).stats()
    e2e = {"value": pairs_step / float(np.mean(e2e_t)), "unit": "pairs/s",
           "h2d_bytes_per_step": int(st_e2e["h2d_bytes"]),
           "d2h_bytes_per_step": int(st_e2e["d2h_bytes"]),
           "ms_per_step": float(np.mean(e2e_t)) * 1e3}

    cnt_ms = float(np.mean(count_ms))
    achieved = 8.0 * pairs_step / (cnt_ms * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak if fp32_peak else None, "traffic": None,
                "kernel": "k_count<%d>" % (0 if w["kind"] == "3d" else 1),
                "flops_per_unit": 8, "unit_of_work": "in-range ordered pair",
                "peak_source": "measured live: FFMA-chain probe kernel (gbp_measure_fp32_peak); "
                               "MEASURED_PEAKS.json holds no FP32 figure",
                "count_ms": cnt_ms,
                "candidate_pairs": st["candidate_pairs"], "recheck_pairs": st["recheck_pairs"],
                "grid_cells": st["cells"], "reach": st["reach"], "block": st["block"],
                "stencil_cells": st["stencil_cells"]}
    # figures of one ncu capture of the count kernel per workload (profiles/*.md)
    tf = os.path.join(ROOT, "profiles", "k_count_ncu.json")
    ncu_fig = {}
    if os.path.exists(tf):
        try:
            ncu_fig = json.load(open(tf)).get(args.workload) or {}
        except Exception:
            ncu_fig = {}
    roofline["traffic"] = ncu_fig.get("dram_bytes")
    # diagnostics: the FP64 recheck rate, and the count kernel's DRAM rate from the
    # ncu traffic figure over its live time (far below HBM: the kernel is issue-bound)
    roofline["recheck_fraction"] = st["recheck_pairs"] / pairs_step if pairs_step else None
    if roofline["traffic"]:
        roofline["hbm_gbs"] = roofline["traffic"] / (cnt_ms * 1e-3) / 1e9
    # the limit the kernel actually meets: instruction issue (one warp instruction
    # per scheduler per cycle, 4 schedulers per SM, at the SM clock sampled during
    # the timed region); warp instructions per launch from the ncu capture
    sm_mhz = clk.summary().get("sm_mhz")
    wi = ncu_fig.get("warp_instructions")
    if wi and sm_mhz:
        nsm = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_issue = nsm * 4 * sm_mhz * 1e6
        roofline["issue"] = {"warp_instructions_per_launch": wi,
                             "achieved": wi / (cnt_ms * 1e-3), "peak": peak_issue,
                             "unit": "warp instructions/s",
                             "frac": wi / (cnt_ms * 1e-3) / peak_issue,
                             "source": "smsp__inst_executed.sum of one ncu capture "
                                       "(profiles/k_count_ncu.json)"}

    line = {"metric": metric, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded; shapes of the named configuration)", "config": cfg,
            "roofline": roofline, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": int(st["kernel_launches"]) * args.steps,
            "ms_build": st["ms_build"], "ms_count": cnt_ms, "pairs_per_step": pairs_step,
            "recheck_pairs_per_step": int(st["recheck_pairs"])}
    parity = {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the reference engine over the whole workload (also the headline's parity)
        try:
            ref, ref_counts = cpu_leg(args, w, x)
            line["cpu_baseline"] = dict(ref["cpu_baseline"], seconds=ref["ms_per_step"] *
                                        ref["steps"] / 1e3)
            if ref_counts is not None:
                from oracle import parity as P
                parity[args.workload] = dict(P.exact(counts_gpu, ref_counts), size="full",
                                             vs="halotools' compiled engine"
                                             if ref["cpu_baseline"]["kind"] == "reference"
                                             else REF_ORACLE)
            cpu = line["cpu_baseline"]["value"]
            line["target_plain_over_host"] = {
                "value": e2e["value"] / cpu, "device_resident": value / cpu, "target": 50,
                "config": w["desc"],
                "gpu": "e2e: the public npairs_3d from pinned host arrays, copies timed",
                "host": line["cpu_baseline"]["sample"]}
        except Exception as exc:  # report, never hide
            line["cpu_baseline"] = {"error": repr(exc)[:400]}
    if rank == 0 and world == 1 and not args.no_extras:
        extras = {}
        for name, fn in EXTRAS.items():
            try:
                extras[name] = fn(dev, threads, not args.no_parity)
            except Exception as exc:  # report, never hide
                extras[name] = {"error": repr(exc)[:300]}
            if "parity" in extras[name]:
                parity[name] = extras[name]["parity"]
        line["paths"] = extras
        ba = extras.get("batched_adjoint_2m", {})
        if "speedup" in ba:
            line["target_batched_adjoint_over_plain"] = {
                "value": ba["speedup"], "target": 5,
                "config": "16 Zheng07 draws on 2,000,000 halos (L = 1000), weighted npairs_3d "
                          "20 log bins 0.1-30, forward + dC/dtheta per draw",
                "batched_ms": ba["batched_ms"], "plain_ms": ba["single_draws_ms"]}
    if parity:
        line["parity"] = parity
        line["parity_ok"] = all(bool(p.get("exact", p.get("ok", False))) for p in parity.values())
    if rank == 0:
        print(json.dumps(line, default=lambda o: o.tolist() if hasattr(o, "tolist") else str(o)))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
