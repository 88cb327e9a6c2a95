"""Benchmark: independent samples/s of GPU MGMC on the 3D 256^3 posterior.

Workload (synthetic, seeded): Q = h^3(-Delta_h + kappa^2) on 256^3 cells
(255^3 = 16,581,375 unknowns, kappa^2 = 10), 64 ball measurements of radius
0.05 with centres uniform in [0.1, 0.9]^3 (seed 1), Sigma = 1e-4 I, values
y ~ N(0, 1) (seed 1), right hand side f = B Sigma^{-1} y; V(1,1) cycle with
SSOR (omega = 1) on 5 levels and the dense FP64 Cholesky sampler on the
16^3-cell coarse level (3,375 unknowns).

A step is one MGMC V-cycle (one sample).  value = steps/s / IACT of the
FP32-mixed chain, IACT from the observable z = b^T x (ball average at the
centre of the domain, radius 0.05) with the reference's tau_int estimator
(window 50).  The FP64 chain is timed the same way and reported beside it.

Run:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun every rank runs an independent chain on its own GPU
(replicas; no collective on the data path).
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (256, 256, 256)
KAPPA_SQ = 10.0
M_MEAS = 64
RADIUS = 0.05
VARIANCE = 1e-4
NLEVEL = 5
IACT_WINDOW = 50
# DRAM bytes (read + write) of one fine colour-pass launch at 256^3 -- a
# constant taken from one ncu capture, not measured in the run
RB_VEC_DRAM_BYTES = 110.47e6
RB_VEC_TRAFFIC_SOURCE = ("constant: ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, capture of "
                         "`python bench.py --profile-steps 1` (profiles/k_sweep_rb_vec_256cubed.md, launch 1): "
                         "100.68 MB read + 9.79 MB written")
RB_VEC_KERNEL = ("k_sweep_rb_vec<1, 0, 1, 1> (one colour pass of the fine-level red-black SOR sweep: FP32, Philox "
                 "noise, 256-bit spans, colour-split f)")
METRIC = "indep. samples/s (rate/IACT), 3D 256³ posterior: mixed vs FP64 plain, 1 GB300"
UNIT = "indep_samples/s"
WORKLOAD = ("3D 256^3 posterior MGMC V(1,1) SSOR omega=1, 5 levels, coarse dense Cholesky 16^3, "
            "64 measurements r=0.05 Sigma=1e-4, kappa^2=10")
PUBLISHED_MGMC_IACT = 1.28  # python/plot_summary.py:28-29, MGMC at 64^3


def problem():
    """The seeded 256^3 posterior: (LinearOperator, f, observable)."""
    import multigridmc_gb300 as M
    rng = np.random.default_rng(1)
    loc = rng.uniform(0.1, 0.9, size=(M_MEAS, 3))
    y = rng.standard_normal(M_MEAS)
    op = M.LinearOperator.shifted_laplace_fd(SHAPE, KAPPA_SQ).with_measurements(
        loc, np.ones(M_MEAS), variance_scaling=VARIANCE, radius=RADIUS)
    f = np.zeros(op.n)
    for j in range(op.m):
        sl = slice(op.B_ptr[j], op.B_ptr[j + 1])
        f[op.B_idx[sl]] += op.B_val[sl] * (y[j] / op.Sigma[j])
    bidx, bval = M.measurement_vector(SHAPE, [0.5, 0.5, 0.5], RADIUS)
    return op, f, (bidx, bval), loc, y


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def replica_max(values, dist, device):
    """Max over the ranks of per-rank times (the slowest replica sets the
    job's time); `dist` is torch.distributed or None for one process."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_rate(world, seconds_per_step, iact):
    """Whole-job independent samples/s of `world` replica chains, each taking
    `seconds_per_step` (the max over ranks) per step."""
    return world / seconds_per_step / iact


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def time_chain(M, torch, op, f, obs, precision, steps, warmup, iact_extra, dist, seed):
    """Timed K steps with the state and f resident on the GPU."""
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), ordering=M.MULTICOLOUR,
                             precision=precision, noise=M.PHILOX, seed=seed)
    s.fix_rhs(f)
    s.set_observable(obs[0], obs[1], capacity=warmup + steps + iact_extra + 8)
    s.step(warmup)
    s.synchronize()
    st = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(st)
    s.step(steps)
    e1.record(st)
    s.synchronize()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(e1) / steps
    if iact_extra > 0:
        s.step(iact_extra)
    z = s.read_observations(warmup + steps + iact_extra + 8)[warmup:]
    return s, ms, z


def sweep_roofline(M, torch, s, precision, peak):
    """Fine-level red-black SOR colour pass (``k_sweep_rb_vec`` in FP32,
    ``k_sweep_rb_pass`` in FP64; Philox noise, no low-rank update) timed on
    the sampler's stream.  One sweep is two launches, one per colour.  The
    algorithmic bytes of a sweep are 3 n s (x read, f read, x written once
    each; in-kernel noise costs none), so one colour launch is charged
    1.5 n s."""
    n = s.level_size(0)
    sz = 4 if precision == M.FP32_MIXED else 8
    s.sweep_device(0, nrepeat=5, with_lowrank=False)
    s.synchronize()
    st = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rep = 40
    e0.record(st)
    s.sweep_device(0, nrepeat=rep, with_lowrank=False)
    e1.record(st)
    s.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / (2 * rep)   # seconds per colour-pass launch
    bytes_per_launch = 1.5 * n * sz
    achieved = bytes_per_launch / t / 1e9
    return achieved, bytes_per_launch, t


def kernel_table(M, torch, s, precision, peak, sweep_launch_s):
    """Achieved GB/s of the other fine-level kernel families on the
    sampler's stream, algorithmic bytes per launch as for the sweep:
    residual-restriction 2 n s + n_1 s (x and f read, f_1 written; the
    low-rank term adds nnz(B)(4 + 2 s)), prolongation n_1 s + 2 n s, and the
    low-rank correction of one sweep (the difference between sweeps with
    and without it, reported as a time): nnz(B)(4 + 2 s) for B^T x (32-bit
    index, value, gathered state) and rows(C)(8 + 3 s) for x += C z (32-bit
    row and column, value, state read and written; nearly every support row
    of C has one entry)."""
    n, n1 = s.level_size(0), s.level_size(1)
    sz = 4 if precision == M.FP32_MIXED else 8
    st = torch.cuda.ExternalStream(s.stream)

    def timed(fn, rep):
        fn(3)
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn(rep)
        e1.record(st)
        s.synchronize()
        return e0.elapsed_time(e1) / 1e3 / rep

    out = {}
    t = timed(lambda r: s.transfer_device(0, 0, r), 40)
    b = 2 * n * sz + n1 * sz
    out["resid_restrict"] = {"s": t, "algorithmic_bytes": b, "gbs": b / t / 1e9, "frac": b / t / 1e9 / peak}
    t = timed(lambda r: s.transfer_device(0, 1, r), 40)
    b = n1 * sz + 2 * n * sz
    out["prolong_add"] = {"s": t, "algorithmic_bytes": b, "gbs": b / t / 1e9, "frac": b / t / 1e9 / peak}
    t_full = timed(lambda r: s.sweep_device(0, nrepeat=r, with_lowrank=True), 20)
    t_lr = t_full - 2 * sweep_launch_s
    out["lowrank_per_sweep"] = {"s": t_lr, "note": "sweep with the low-rank correction minus its two colour passes"}
    out["sweep_with_lowrank_s"] = t_full
    return out


def time_e2e(M, torch, op, f, precision, steps, seed, iact, fixed=True):
    """The same metric through Sampler::apply with host buffers, as the
    reference's measure_sampling_time drives it (sampling_time.cc:28-41):
    fix_rhs(f) once, then apply(f, x) per step with the fixed f, so x goes
    host->device (pinned) and comes back device->host every step.  With
    fixed=False every step also sends f (apply without fix_rhs)."""
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), ordering=M.MULTICOLOUR,
                             precision=precision, noise=M.PHILOX, seed=seed + 7)
    fh = torch.empty(op.n, dtype=torch.float64, pin_memory=True).numpy()
    xh = torch.empty(op.n, dtype=torch.float64, pin_memory=True).numpy()
    fh[:] = f
    xh[:] = 0.0
    if fixed:
        s.fix_rhs(fh)
    fa = None if fixed else fh
    for _ in range(3):
        s.apply(fa, xh)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.apply(fa, xh)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    s.close()
    return 1.0 / dt / iact, dt, (1 if fixed else 2) * op.n * 8, op.n * 8


def cpu_reference(seconds_budget=25.0, nsteps=None, warmup=1):
    """The oracle's restatement of the reference MGMC (lexicographic SOR,
    dense B-bar, CLCG noise) on the host cores, one chain, OpenMP threads in
    the dense products; `warmup` untimed steps, then `nsteps` timed steps
    (or as many as fit in `seconds_budget` when nsteps is None)."""
    import oracle as O
    import multigridmc_gb300 as M
    rng = np.random.default_rng(1)
    loc = rng.uniform(0.1, 0.9, size=(M_MEAS, 3))
    y = rng.standard_normal(M_MEAS)
    t0 = time.perf_counter()
    op = O.Operator.fd(list(SHAPE), KAPPA_SQ)
    op.add_measurements(loc, np.ones(M_MEAS), variance_scaling=VARIANCE, radius=RADIUS)
    Bd_ptr, Brow, Bval, sig = op.B()
    f = np.zeros(op.n)
    for j in range(M_MEAS):
        f[Brow[Bd_ptr[j]:Bd_ptr[j + 1]]] += Bval[Bd_ptr[j]:Bd_ptr[j + 1]] * (y[j] / sig[j])
    s = O.mgmc_sampler(op, O.Source(), NLEVEL, ordering=0)
    setup = time.perf_counter() - t0
    x = np.zeros(op.n)
    s.apply(f, x, max(1, warmup))  # untimed steps (the first touches every array)
    times = []
    t_start = time.perf_counter()
    while True:
        t1 = time.perf_counter()
        s.apply(f, x, 1)
        times.append(time.perf_counter() - t1)
        if nsteps is not None and len(times) >= nsteps:
            break
        if nsteps is None and time.perf_counter() - t_start > seconds_budget:
            break
    per_step = float(np.mean(times))
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"per_step_s": per_step, "steps": len(times), "setup_s": setup, "threads": threads, "host": host_cpu()}


def host_cpu():
    """CPU model and core count of this host (as lscpu reports them)."""
    model = platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip() + f" ({platform.machine()})"
                break
    except Exception:
        pass
    return f"{model}, {os.cpu_count()} cores"


def coupled_run(s, probes, nsamples):
    """`nsamples` further steps of sampler `s` recording every probe b_p^T x
    after each step; returns the (nsamples, nprobe) observations."""
    s.set_probes(probes, nsamples + 8)
    s.step(nsamples)
    s.synchronize()
    return s.read_observations(nsamples + 8)


def covariance_figures(M, op, f, pts, Z32, Z64, iact32, iact64, exact=True):
    """The precision target of the 256^3 posterior: relative Frobenius
    difference of the probe-point sample covariances of the coupled
    FP32-mixed and FP64 chains (identical Philox normals, so the difference
    is the FP32 chain's rounding, not Monte Carlo noise), and each chain
    against the exact probe covariance within its Monte Carlo error."""
    nprobe = len(pts)
    C32 = np.cov(Z32[:, :nprobe].T)
    C64 = np.cov(Z64[:, :nprobe].T)
    out = {"fp32_vs_fp64_cov_rel_frobenius": float(np.linalg.norm(C32 - C64) / np.linalg.norm(C64)),
           "fp32_vs_fp64_mean_rel": float(np.linalg.norm(Z32[:, :nprobe].mean(0) - Z64[:, :nprobe].mean(0))
                                          / np.linalg.norm(Z64[:, :nprobe].mean(0))),
           "nprobe": nprobe, "nsamples": int(Z32.shape[0]), "target": 1e-3,
           "probes": "256 interior vertices drawn uniformly without replacement (seed 2)"}
    if not exact:
        return out
    Cx, mu, solve_s = exact_probe_moments(op, f, pts)
    for name, Z, tau in (("fp32", Z32, iact32), ("fp64", Z64, iact64)):
        Zp = Z[:, :nprobe]
        N = Zp.shape[0]
        C = np.cov(Zp.T)
        cov_se = np.sqrt(tau * np.sum(Cx ** 2 + np.outer(np.diag(Cx), np.diag(Cx))) / N)
        mean_se = np.sqrt(tau * np.sum(np.diag(Cx)) / N)
        out[name + "_vs_exact"] = {"cov_rel_frobenius": float(np.linalg.norm(C - Cx) / np.linalg.norm(Cx)),
                                   "cov_mc_expected": float(cov_se / np.linalg.norm(Cx)),
                                   "mean_rel": float(np.linalg.norm(Zp.mean(0) - mu) / np.linalg.norm(mu)),
                                   "mean_mc_expected": float(mean_se / np.linalg.norm(mu))}
    out["exact"] = ("probe covariances e_p^T Q^-1 e_q and the mean Q^-1 f by multigrid-preconditioned loop "
                    f"solves on the GPU to rtol 1e-10 ({solve_s:.1f} s)")
    return out


def covariance_study(nsamples, nprobe=256, warmup=50, seed=1000):
    """Coupled FP32-mixed and FP64 chains on the 256^3 posterior: the same
    Philox streams (the FP64 chain widens the FP32 normals), so the two
    chains see identical noise.  Reports the relative Frobenius difference of
    the nprobe x nprobe probe-point sample covariances and each chain's
    IACT."""
    import multigridmc_gb300 as M
    op, f, obs, _, _ = problem()
    rng = np.random.default_rng(2)
    pts = rng.choice(op.n, size=nprobe, replace=False)
    probes = [(np.array([p], np.int64), np.array([1.0])) for p in pts] + [obs]
    res = {}
    Z = {}
    for name, prec in (("fp32", M.FP32_MIXED), ("fp64", M.FP64)):
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), ordering=M.MULTICOLOUR,
                                 precision=prec, noise=M.PHILOX, seed=seed)
        s.fix_rhs(f)
        s.step(warmup)
        s.set_probes(probes, nsamples)
        t0 = time.perf_counter()
        s.step(nsamples)
        s.synchronize()
        dt = time.perf_counter() - t0
        Z[name] = s.read_observations(nsamples)
        res[name] = {"ms_per_step": dt / nsamples * 1e3, "iact": M.statistics.tau_int(Z[name][:, -1], IACT_WINDOW)}
        s.close()
    C32 = np.cov(Z["fp32"][:, :nprobe].T)
    C64 = np.cov(Z["fp64"][:, :nprobe].T)
    res["cov_rel_frobenius"] = float(np.linalg.norm(C32 - C64) / np.linalg.norm(C64))
    # each chain against the exact posterior: mean Q^{-1} f and the probe
    # covariances e_p^T Q^{-1} e_q, by multigrid solves on the GPU
    Cx, mu, solve_s = exact_probe_moments(op, f, pts)
    for name in ("fp32", "fp64"):
        Zp = Z[name][:, :nprobe]
        C = np.cov(Zp.T)
        tau = res[name]["iact"]
        # Monte Carlo standard errors for nsamples draws with integrated
        # autocorrelation time tau: Var(C^_pq) ~ tau (C_pq^2 + C_pp C_qq) / N,
        # Var(mean_p) ~ tau C_pp / N
        cov_se = np.sqrt(tau * np.sum(Cx ** 2 + np.outer(np.diag(Cx), np.diag(Cx))) / nsamples)
        mean_se = np.sqrt(tau * np.sum(np.diag(Cx)) / nsamples)
        res[name]["cov_vs_exact_rel_frobenius"] = float(np.linalg.norm(C - Cx) / np.linalg.norm(Cx))
        res[name]["cov_vs_exact_mc_expected"] = float(cov_se / np.linalg.norm(Cx))
        res[name]["mean_vs_exact_rel"] = float(np.linalg.norm(Zp.mean(0) - mu) / np.linalg.norm(mu))
        res[name]["mean_vs_exact_mc_expected"] = float(mean_se / np.linalg.norm(mu))
    res["exact_moments"] = {"method": "MG-preconditioned loop solves on the GPU (FP32-mixed cycle, FP64 "
                                      "refinement, rtol 1e-10), one per probe plus one for the mean",
                            "seconds": solve_s}
    res["mean_rel_diff"] = float(np.linalg.norm(Z["fp32"][:, :nprobe].mean(0) - Z["fp64"][:, :nprobe].mean(0))
                                 / np.linalg.norm(Z["fp64"][:, :nprobe].mean(0)))
    res["pathwise_rel_diff_last"] = float(np.linalg.norm(Z["fp32"][-1, :nprobe] - Z["fp64"][-1, :nprobe])
                                          / np.linalg.norm(Z["fp64"][-1, :nprobe]))
    res["nsamples"] = nsamples
    res["nprobe"] = nprobe
    return res


def exact_probe_moments(op, f, pts, rtol=1e-10):
    """Exact posterior mean at the probe points, (Q^{-1} f)[pts], and the
    probe covariance matrix (Q^{-1})[pts, pts], by LoopSolver solves with the
    multigrid preconditioner on the GPU (the reference's Woodbury + loop
    solve comparator of cholesky_solver.cc / loop_solver.cc at sizes where a
    factorisation does not fit)."""
    import torch
    import multigridmc_gb300 as M
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), precision=M.FP32_MIXED)
    b = torch.zeros(op.n, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    idx = torch.as_tensor(np.asarray(pts, np.int64), device="cuda")
    t0 = time.perf_counter()
    C = np.zeros((len(pts), len(pts)))
    for k, p in enumerate(pts):
        b.zero_()
        b[int(p)] = 1.0
        torch.cuda.synchronize()
        _, _, conv = s.solve_device(b.data_ptr(), x.data_ptr(), rtol, 1e30, 100)
        if not conv:
            raise RuntimeError("probe solve did not converge")
        C[:, k] = x[idx].cpu().numpy()
    b.copy_(torch.from_numpy(np.asarray(f, np.float64)))
    torch.cuda.synchronize()
    _, _, conv = s.solve_device(b.data_ptr(), x.data_ptr(), rtol, 1e30, 100)
    if not conv:
        raise RuntimeError("mean solve did not converge")
    mu = x[idx].cpu().numpy()
    dt = time.perf_counter() - t0
    s.close()
    return 0.5 * (C + C.T), mu, dt


def adjoint_study(nsteps=200, every=10, nfd=4, seed=7, fd2=True):
    """Differentiation: 3D 128^3 posterior (kappa^2 = 10, 32 measurements,
    centres U[0.1, 0.9]^3, radius 0.05, Sigma = 1e-4, values N(0, 1)),
    J = mean over 200 MGMC steps from x = 0 of ||x on the sub-cube
    [0.25, 0.75]^3||^2 with the Philox noise fixed by the seed; gradients
    with respect to kappa^2, the measurement values y and log Sigma by the
    parameter adjoint with a checkpoint every 10 steps (each segment
    recomputed from its checkpoint), FP64 and FP32-mixed; the FP64 gradient
    against central differences (step 1e-6 relative) for kappa^2 and the
    first nfd entries of y and log Sigma."""
    import torch
    import scipy.sparse as sp
    import multigridmc_gb300 as M
    shape, m = (128, 128, 128), 32
    rng = np.random.default_rng(1)
    loc = rng.uniform(0.1, 0.9, size=(m, 3))
    y0 = rng.standard_normal(m)
    cols = [M.measurement_vector(shape, x0, RADIUS) for x0 in loc]
    k20, ls0 = KAPPA_SQ, np.full(m, np.log(VARIANCE))

    def make_op(k2, ls):
        return M.LinearOperator.shifted_laplace_fd(shape, k2).with_lowrank(cols, np.exp(ls))

    op0 = make_op(k20, ls0)
    n = op0.n
    B = sp.csc_matrix((op0.B_val, op0.B_idx, op0.B_ptr), shape=(n, m))
    hd = 1.0 / float(np.prod(shape))
    N = [c - 1 for c in shape]
    ax = [(np.arange(k) + 1.0) / c for k, c in zip(N, shape)]
    inside = ((ax[2][:, None, None] >= 0.25) & (ax[2][:, None, None] <= 0.75) &
              (ax[1][None, :, None] >= 0.25) & (ax[1][None, :, None] <= 0.75) &
              (ax[0][None, None, :] >= 0.25) & (ax[0][None, None, :] <= 0.75))
    mask = torch.from_numpy(inside.reshape(-1).astype(np.float64)).cuda()
    prm = M.MultigridParameters(nlevel=5)

    def sampler(op, prec):
        return M.MultigridMCSampler(op, prm, precision=prec, noise=M.PHILOX, seed=seed)

    def forward(s, ls, yv, keep=False):
        s.fix_rhs(B @ (yv / np.exp(ls)))
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        s.set_state_device(x.data_ptr())
        s.step_counter = 0
        J = torch.zeros((), dtype=torch.float64, device="cuda")
        cps = {0: x.clone()}
        for t in range(nsteps):
            s.step(1)
            s.get_state_device(x.data_ptr())
            J += (mask * x * x).sum()
            if keep and (t + 1) % every == 0 and t + 1 < nsteps:
                cps[t + 1] = x.clone()
        return float(J) / nsteps, cps

    def gradient(prec):
        s = sampler(op0, prec)
        for _ in range(2):  # warm-up: graphs, tape buffers, lazy allocations, the torch kernels of J
            x = torch.zeros(n, dtype=torch.float64, device="cuda")
            lam = torch.ones_like(x)
            fb = torch.zeros_like(x)
            torch.cuda.synchronize()
            s.set_state_device(x.data_ptr())
            s.step(3)
            s.get_state_device(x.data_ptr())
            w = (mask * x * x).sum() + (2.0 / nsteps) * (mask * x).sum()
            lam += (2.0 / nsteps) * mask * x
            x2 = x.clone()
            torch.cuda.synchronize()
            s.adjoint_params_device(x2.data_ptr(), lam.data_ptr(), fb.data_ptr(), step_index=0)
            float(w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, cps = forward(s, ls0, y0, keep=True)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        lam = torch.zeros(n, dtype=torch.float64, device="cuda")
        fbar = torch.zeros_like(lam)
        gc, gs = 0.0, np.zeros(m)
        t0 = time.perf_counter()
        for a in reversed(range(0, nsteps, every)):
            b = min(nsteps, a + every)
            x = cps[a].clone()
            torch.cuda.synchronize()
            s.set_state_device(x.data_ptr())
            s.step_counter = a
            xs = [cps[a]]
            for _ in range(a, b):
                s.step(1)
                xt = torch.empty_like(x)
                s.get_state_device(xt.data_ptr())
                xs.append(xt)
            for t in range(b - 1, a - 1, -1):  # lam: adjoint of x_{t+1}
                lam += (2.0 / nsteps) * mask * xs[t + 1 - a]
                torch.cuda.synchronize()
                c, g = s.adjoint_params_device(xs[t - a].data_ptr(), lam.data_ptr(), fbar.data_ptr(), step_index=t)
                gc += c
                gs += g
        torch.cuda.synchronize()
        t_rev = time.perf_counter() - t0
        Btf = B.T @ fbar.cpu().numpy()
        sig = np.exp(ls0)
        grads = {"kappa_sq": hd * gc, "y": Btf / sig, "log_sigma": gs - Btf * y0 / sig}
        return s, J, grads, {"forward_ms_per_step": t_fwd * 1e3 / nsteps, "reverse_ms_per_step": t_rev * 1e3 / nsteps}

    out = {}
    s64, J64, g64, tm64 = gradient(M.FP64)
    s32, J32, g32, tm32 = gradient(M.FP32_MIXED)
    s32.close()
    out["fp64"] = {"J": J64, **tm64}
    out["fp32_mixed"] = {"J": J32, **tm32}
    out["fp32_vs_fp64_rel"] = {k: float(np.linalg.norm(np.atleast_1d(g32[k]) - np.atleast_1d(g64[k])) /
                                        np.linalg.norm(np.atleast_1d(g64[k]))) for k in g64}
    # finite differences of the FP64 chain: central, step 1e-6 (relative for
    # kappa^2 and y, absolute for log Sigma), and fourth order with step 1e-4
    # (J ~ 1e7 here, so the two-point difference carries eps J / h ~ 1e-3 of
    # rounding; the fourth-order one, with its larger step, ~1e-5)
    checks = []

    def J_with(k2=k20, ls=ls0, yv=y0, reuse=None):
        s = reuse or sampler(make_op(k2, ls), M.FP64)
        J, _ = forward(s, ls, yv)
        if reuse is None:
            s.close()
        return J

    def J_dir(kind, k, t):
        if kind == "kappa_sq":
            return J_with(k2=k20 * (1.0 + t))
        e = np.zeros(m)
        if kind == "log_sigma":
            e[k] = t
            return J_with(ls=ls0 + e)
        e[k] = t * max(1.0, abs(y0[k]))
        return J_with(yv=y0 + e, reuse=s64)

    params = [("kappa_sq", 0, g64["kappa_sq"], k20, abs(g64["kappa_sq"]))]
    for k in range(nfd):
        params.append(("log_sigma", k, float(g64["log_sigma"][k]), 1.0, np.abs(g64["log_sigma"]).max()))
        params.append(("y", k, float(g64["y"][k]), max(1.0, abs(y0[k])), np.abs(g64["y"]).max()))
    for kind, k, g, unit, scale in params:
        c = {"param": kind if kind == "kappa_sq" else f"{kind}[{k}]", "adjoint": g}
        if fd2:
            h = 1e-6
            d2 = (J_dir(kind, k, h) - J_dir(kind, k, -h)) / (2 * h * unit)
            c.update(fd2=d2, rel_err_fd2=abs(g - d2) / max(abs(d2), 0.1 * scale))
        h = 1e-4
        fd4 = (8 * (J_dir(kind, k, h) - J_dir(kind, k, -h)) - (J_dir(kind, k, 2 * h) - J_dir(kind, k, -2 * h))) / (12 * h * unit)
        c.update(fd4=fd4, rel_err_fd4=abs(g - fd4) / max(abs(fd4), 0.1 * scale))
        checks.append(c)
    s64.close()
    out["fd_checks_fp64"] = checks
    if fd2:
        out["max_rel_err_fd2"] = max(c["rel_err_fd2"] for c in checks)
    out["max_rel_err_fd4"] = max(c["rel_err_fd4"] for c in checks)
    out["problem"] = ("3D 128^3 posterior, 32 measurements, V(1,1) SSOR, 5 levels, coarse Cholesky 8^3, Philox noise, "
                      f"{nsteps} steps, checkpoints every {every}")
    return out


def config1_figures(nsamples=10000, burnin=100, seed=31):
    """Config 1: 2D prior on 64^2 cells (63^2 = 3,969 unknowns), kappa^2 = 10,
    V(1,1) SSOR omega = 1 on 4 levels, Cholesky sampler on the 8^2-cell coarse
    level, FP64 chain with Philox noise; 10^4 samples after 100 burn-in steps.
    IACT of the centre ball average (window 50) and every vertex's sample
    mean and variance against the exact mean mu and covariance (dense inverse
    of the precision the library assembles; f = Q mu with mu uniform in
    [0, 1]): z-scores with an integrated autocorrelation time of 1.5 in the
    error model, and the covariance's relative Frobenius error against its
    Monte Carlo expectation."""
    import multigridmc_gb300 as M
    shape = (64, 64)
    op = M.LinearOperator.shifted_laplace_fd(shape, KAPPA_SQ)
    Q = op.to_scipy().toarray()
    C = np.linalg.inv(Q)
    mu = np.random.default_rng(1342517).uniform(0.0, 1.0, op.n)
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=4), precision=M.FP64, seed=seed)
    s.fix_rhs(Q @ mu)
    s.step(burnin)
    bidx, bval = M.measurement_vector(shape, [0.5, 0.5], RADIUS)
    probes = [(np.array([p], np.int64), np.array([1.0])) for p in range(op.n)] + [(bidx, bval)]
    s.set_probes(probes, nsamples + 8)
    s.step(nsamples)
    s.synchronize()
    Z = s.read_observations(nsamples + 8)
    s.close()
    X = Z[:, :op.n]
    N, tau_b = X.shape[0], 1.5
    d = np.diag(C)
    zm = (X.mean(0) - mu) / np.sqrt(tau_b * d / N)
    zv = (X.var(0) - d) / (d * np.sqrt(2.0 * tau_b / N))
    Ch = np.cov(X.T, bias=True)
    expected = np.sqrt(tau_b * np.sum(C ** 2 + np.outer(d, d)) / N) / np.linalg.norm(C)
    return {"workload": "2D prior 64^2 cells, kappa^2=10, V(1,1) SSOR, 4 levels, coarse Cholesky 8^2, FP64",
            "samples": int(N), "burnin": burnin, "iact": M.statistics.tau_int(Z[:, -1], IACT_WINDOW),
            "mean_z_max": float(np.abs(zm).max()), "mean_z_rms": float(np.sqrt(np.mean(zm ** 2))),
            "var_z_max": float(np.abs(zv).max()), "var_z_rms": float(np.sqrt(np.mean(zv ** 2))),
            "cov_rel_frobenius": float(np.linalg.norm(Ch - C) / np.linalg.norm(C)),
            "cov_rel_frobenius_mc_expected": float(expected)}


def configs_section():
    """The other configurations of the benchmark suite, compactly, each
    guarded so that a failure is recorded instead of losing the line:
    config 1 (2D 64^2 prior: IACT, variances vs exact), config 2 (128^3 FP64
    posterior, 32 measurements: MGMC against the one-level SSOR Gibbs sampler
    and the exact sampler), config 4 (512 batched chains), config 5 (128^3
    differentiation, 200 steps, checkpoints every 10: the FP64 gradient
    against fourth-order differences for kappa^2, y_0 and log Sigma_0, and the
    FP32-mixed gradient against the FP64 one)."""
    out = {}
    for name, fn in (("config1_2d_prior_64", lambda: config1_figures()),
                     ("config2_posterior_128_fp64", lambda: summary_study(sizes=(128,), gibbs_steps=40000,
                                                                          fp32=False, verbose=False)[0]),
                     ("config4_batch_512", lambda: batch_study(512, 100, compare=False)),
                     ("config5_adjoint_128", lambda: adjoint_study(nfd=1, fd2=False))):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:  # recorded, never fatal to the benchmark line
            out[name] = {"failed": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


def summary_study(sizes=(16, 32, 48, 64, 128), m=32, seed=1, lrchol_max=48, gibbs_steps=None, fp32=True,
                  verbose=True):
    """The reference's published comparison (python/plot_summary.py:23-33:
    IACT and time per independent sample of the Cholesky, Gibbs and MGMC
    samplers on a 3D posterior at 16^3 .. 64^3 cells) on the GPU, plus
    128^3: posterior kappa^2 = 10 with m ball measurements (centres
    U[0.1, 0.9]^3, radius 0.05, Sigma = 1e-4, values N(0, 1)), observable
    b^T x with b the measurement vector at the centre (sampling_time.cc:22-40).
    MGMC: V(1,1) SSOR down to 8^3 cells (6^3 at 48^3); Gibbs: the one-level
    SSOR sampler; exact: x = Q^{-1}(f + eta), one multigrid solve to 1e-10
    per independent draw; the reference's LowRankCholeskySampler (factor of
    A_0 on the host, samples on the GPU) up to lrchol_max^3 cells.  Time per
    independent sample = ms per step x IACT; IACT windows grow to 10 IACT."""
    import multigridmc_gb300 as M
    levels = {16: 2, 32: 3, 48: 4, 64: 4, 96: 4, 128: 5}
    rows = []
    for N in sizes:
        shape = (N, N, N)
        rng = np.random.default_rng(seed)
        loc = rng.uniform(0.1, 0.9, size=(m, 3))
        y = rng.standard_normal(m)
        op = M.LinearOperator.shifted_laplace_fd(shape, KAPPA_SQ).with_measurements(
            loc, np.ones(m), variance_scaling=VARIANCE, radius=RADIUS)
        f = np.zeros(op.n)
        for j in range(op.m):
            sl = slice(op.B_ptr[j], op.B_ptr[j + 1])
            f[op.B_idx[sl]] += op.B_val[sl] * (y[j] / op.Sigma[j])
        bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], RADIUS)
        row = {"cells": N, "unknowns": op.n}

        def chain(params, prec, nsteps, warm):
            s = M.MultigridMCSampler(op, params, precision=prec, seed=seed + 100)
            s.fix_rhs(f)
            s.step(warm)
            s.set_observable(bidx, bval, nsteps + 8)
            s.synchronize()
            t0 = time.perf_counter()
            s.step(nsteps)
            s.synchronize()
            dt = (time.perf_counter() - t0) / nsteps
            z = s.read_observations(nsteps + 8)[:nsteps]
            s.close()
            K = 50
            tau = M.statistics.tau_int(z, K)
            while K < 10 * tau and 10 * tau < len(z) / 20:
                K = int(10 * tau) + 1
                tau = M.statistics.tau_int(z, K)
            return {"ms_per_step": dt * 1e3, "iact": tau, "window": K, "steps": nsteps,
                    "ms_per_indep": dt * 1e3 * max(tau, 1.0)}

        mg = M.MultigridParameters(nlevel=levels[N])
        gibbs = M.MultigridParameters(nlevel=1, coarse_solver="SSOR", ncoarsesmooth=1)
        row["mgmc_fp64"] = chain(mg, M.FP64, 4000, 100)
        if fp32:
            row["mgmc_fp32"] = chain(mg, M.FP32_MIXED, 4000, 100)
        gsteps = gibbs_steps or (100000 if N >= 128 else 50000)
        row["gibbs_fp64"] = chain(gibbs, M.FP64, gsteps, 2000)
        if N < 128 and fp32:
            row["gibbs_fp32"] = chain(gibbs, M.FP32_MIXED, gsteps, 2000)
        import torch
        fd = torch.from_numpy(np.asarray(f, np.float64)).cuda()
        xd = torch.empty_like(fd)
        torch.cuda.synchronize()
        for name, prec in (("exact_fp32", M.FP32_MIXED), ("exact_fp64", M.FP64))[(0 if fp32 else 1):]:
            s = M.MultigridMCSampler(op, mg, precision=prec, seed=seed + 200)
            for _ in range(3):
                s.exact_sample_device(fd.data_ptr(), xd.data_ptr())
            ns = 40
            its = 0
            t0 = time.perf_counter()
            for _ in range(ns):
                its += s.exact_sample_device(fd.data_ptr(), xd.data_ptr())
            dt = (time.perf_counter() - t0) / ns
            s.close()
            row[name] = {"ms_per_sample": dt * 1e3, "iterations": its / ns, "ms_per_indep": dt * 1e3}
        if N <= lrchol_max:
            # the reference's LowRankCholeskySampler: factor of A_0 on the
            # host (set-up timed apart), FP64 samples on the GPU
            t0 = time.perf_counter()
            s = M.LowRankCholeskySampler(op, seed=seed + 300)
            setup = time.perf_counter() - t0
            s.fix_rhs(f)
            for _ in range(3):
                s.apply_device(0, xd.data_ptr())
            torch.cuda.synchronize()
            ns = 40
            t0 = time.perf_counter()
            for _ in range(ns):
                s.apply_device(0, xd.data_ptr())
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / ns
            s.close()
            row["lowrank_cholesky_fp64"] = {"ms_per_sample": dt * 1e3, "ms_per_indep": dt * 1e3, "setup_s": setup}
        rows.append(row)
        if verbose:
            print(json.dumps({"summary_row": row}), flush=True)
    return rows


def variable_study(N=256, nsteps=4000, Lambda_min=0.12, Lambda_max=0.23, seed=1):
    """Variable coefficients at the benchmark's size: the 256^3 posterior
    (64 measurements, radius 0.05, Sigma = 1e-4) with the periodic
    correlation length (correlationlength_model.hh:83-112) instead of the
    constant kappa^2 = 10; per-vertex centre weights on the fine level,
    per-point Galerkin 27-point stencils below.  ms per step (graph, host
    clock over nsteps), IACT of b^T x, independent samples/s, FP32-mixed and
    FP64, and the constant-coefficient chain of the same run."""
    import multigridmc_gb300 as M
    shape = (N, N, N)
    rng = np.random.default_rng(seed)
    loc = rng.uniform(0.1, 0.9, size=(M_MEAS, 3))
    y = rng.standard_normal(M_MEAS)
    bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], RADIUS)
    out = {}
    for label, base in (("periodic", M.LinearOperator.shifted_laplace_fd_periodic(shape, Lambda_min, Lambda_max)),
                        ("constant", M.LinearOperator.shifted_laplace_fd(shape, KAPPA_SQ))):
        op = base.with_measurements(loc, np.ones(M_MEAS), variance_scaling=VARIANCE, radius=RADIUS)
        f = np.zeros(op.n)
        for j in range(op.m):
            sl = slice(op.B_ptr[j], op.B_ptr[j + 1])
            f[op.B_idx[sl]] += op.B_val[sl] * (y[j] / op.Sigma[j])
        for pname, prec in (("fp32", M.FP32_MIXED), ("fp64", M.FP64)):
            t0 = time.perf_counter()
            s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), precision=prec, seed=seed + 10)
            setup = time.perf_counter() - t0
            s.fix_rhs(f)
            s.step(50)
            s.set_observable(bidx, bval, nsteps + 8)
            s.synchronize()
            t0 = time.perf_counter()
            s.step(nsteps)
            s.synchronize()
            dt = (time.perf_counter() - t0) / nsteps
            z = s.read_observations(nsteps + 8)[:nsteps]
            s.close()
            tau = M.statistics.tau_int(z, IACT_WINDOW)
            out[f"{label}_{pname}"] = {"ms_per_step": dt * 1e3, "iact": tau, "indep_per_s": 1.0 / (dt * tau),
                                       "setup_s": setup}
    out["problem"] = (f"3D {N}^3 posterior, {M_MEAS} measurements; periodic Lambda in [{Lambda_min}, {Lambda_max}] "
                      f"vs constant kappa^2 = {KAPPA_SQ}; V(1,1) SSOR, {NLEVEL} levels")
    return out


def solve_study(rtol=1e-10, repeats=3):
    """The reference's deterministic multigrid solve (driver_mg: LoopSolver
    with MultigridPreconditioner) of Q x = f on the 256^3 posterior: FP64
    cycle and FP32-mixed cycle with FP64 refinement; device-resident
    vectors, host clock around the whole solve (it synchronises once per
    iteration for the convergence test)."""
    import torch
    import multigridmc_gb300 as M
    op, f, _, _, _ = problem()
    b = torch.from_numpy(np.asarray(f, np.float64)).cuda()
    x = torch.zeros_like(b)
    out = {}
    for name, prec in (("fp32_mixed", M.FP32_MIXED), ("fp64", M.FP64)):
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), precision=prec)
        s.solve_device(b.data_ptr(), x.data_ptr(), rtol, 1e30, 100)  # graphs and solver buffers
        best = None
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it, rn, conv = s.solve_device(b.data_ptr(), x.data_ptr(), rtol, 1e30, 100)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        # residual of the returned x, checked through the FP64 operator apply
        xh = x.cpu().numpy()
        r = f - s.level_apply(0, xh) if prec == M.FP64 else None
        s.close()
        out[name] = {"iterations": it, "converged": conv, "ms": best * 1e3, "ms_per_iteration": best * 1e3 / max(it, 1),
                     "rel_residual": rn / float(np.linalg.norm(f))}
        if r is not None:
            out[name]["rel_residual_host_check"] = float(np.linalg.norm(r) / np.linalg.norm(f))
    out["rtol"] = rtol
    out["problem"] = "3D 256^3 posterior, 64 measurements, V(1,1) SSOR, 5 levels, coarse Cholesky 16^3"
    return out


def batch_study(nchain, steps, warmup=5, seed=3, compare=True):
    """Batching: nchain independent chains, cubic lattices drawn from
    {32,48,64,96,128}^3 cells, kappa^2 log-uniform in [1, 100], 0-64
    measurements (centres U[0.1,0.9]^3, radius 0.05, variance 1e-4, values
    N(0,1)), FP32-mixed precision, V(1,1) SSOR, 5 levels, all
    stepped by one CUDA graph launch per step: the chains of each lattice
    size through the batched kernels, and, for comparison, every chain as
    its own child graph.  Reports aggregate samples/s and the per-chain IACT
    distribution (steps >= 60 for the IACT)."""
    import torch
    import multigridmc_gb300 as M
    rng = np.random.default_rng(seed)
    sizes = rng.choice([32, 48, 64, 96, 128], size=nchain)
    ksq = np.exp(rng.uniform(np.log(1.0), np.log(100.0), size=nchain))
    ms = rng.integers(0, 65, size=nchain)
    chains = []
    t0 = time.perf_counter()
    unknowns = 0
    for i in range(nchain):
        shape = (int(sizes[i]),) * 3
        op = M.LinearOperator.shifted_laplace_fd(shape, float(ksq[i]))
        m = int(ms[i])
        y = rng.standard_normal(m)
        if m > 0:
            op = op.with_measurements(rng.uniform(0.1, 0.9, size=(m, 3)), np.ones(m), VARIANCE, RADIUS)
        f = np.zeros(op.n)
        for j in range(op.m):
            sl = slice(op.B_ptr[j], op.B_ptr[j + 1])
            f[op.B_idx[sl]] += op.B_val[sl] * (y[j] / op.Sigma[j])
        s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), precision=M.FP32_MIXED, seed=10000 + i)
        s.fix_rhs(f)
        bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], RADIUS)
        s.set_observable(bidx, bval, warmup + steps + 8)
        chains.append(s)
        unknowns += op.n
    setup = time.perf_counter() - t0

    def timed_batch():
        batch = M.MultigridMCBatch(chains)
        groups = batch.groups
        batch.step(warmup)
        batch.synchronize()
        st = torch.cuda.ExternalStream(batch.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        batch.step(steps)
        e1.record(st)
        batch.synchronize()
        ms = e0.elapsed_time(e1) / steps
        taus = []
        for s in chains:
            z = s.read_observations(warmup + steps + 8)[warmup:]
            if len(z) > 60 and np.std(z) > 0:
                taus.append(M.statistics.tau_int(z, 20))
        batch.close()
        return ms, groups, taus

    # batched kernels: one launch per kernel of the step for all chains of a
    # lattice size; then the same chains as one child graph per chain
    ms_step, groups, taus = timed_batch()
    graphs = None
    if compare:
        os.environ["MGMC_BATCH_KERNELS"] = "0"
        try:
            ms_graphs, _, _ = timed_batch()
        finally:
            del os.environ["MGMC_BATCH_KERNELS"]
        graphs = {"ms_per_batched_step": ms_graphs, "samples_per_s": nchain * 1000.0 / ms_graphs}
    for ch in chains:
        ch.close()
    return {"nchain": nchain, "ms_per_batched_step": ms_step, "samples_per_s": nchain * 1000.0 / ms_step,
            "groups": groups[0], "chains_in_groups": groups[1],
            "graph_of_graphs": graphs,
            "unknowns_total": int(unknowns), "setup_s": setup, "iact_median": float(np.median(taus)) if taus else None,
            "iact_p90": float(np.percentile(taus, 90)) if taus else None, "iact_window": 20, "steps": steps}


def convergence_study(nchain, nsteps, seed=5000):
    """measure_convergence (convergence.cc:4-161) as batched GPU chains: a
    32^3 posterior (kappa^2 = 10, 8 measurements r = 0.1 Sigma = 1e-4),
    FP32-mixed, nchain chains from x = 0; per step |E[z^k] - E[z]| and
    |Var[z^k] - Var[z]| with their statistical errors, against the exact
    moments of z = b^T x (CG on the assembled operator, FP64)."""
    import multigridmc_gb300 as M
    from multigridmc_gb300.measurements import exact_observable_moments, measure_convergence
    shape = (32, 32, 32)
    rng = np.random.default_rng(seed)
    m = 8
    op = M.LinearOperator.shifted_laplace_fd(shape, KAPPA_SQ).with_measurements(
        rng.uniform(0.1, 0.9, size=(m, 3)), np.ones(m), VARIANCE, 0.1)
    y = rng.standard_normal(m)
    f = op.B_dense() @ (y / op.Sigma)
    bidx, bval = M.measurement_vector(shape, [0.5, 0.5, 0.5], RADIUS)
    mu, var = exact_observable_moments(op, f, bidx, bval)
    t0 = time.perf_counter()
    res = measure_convergence(op, M.MultigridParameters(nlevel=4), f, bidx, bval, nchain, nsteps, seed=seed,
                              precision=M.FP32_MIXED)
    dt = time.perf_counter() - t0
    dm = np.abs(res["mean"] - mu)
    dv = np.abs(res["variance"] - var)
    return {"nchain": nchain, "nsteps": nsteps, "exact_mean": mu, "exact_variance": var,
            "mean_diff": dm.tolist(), "mean_err": res["err_mean"].tolist(),
            "variance_diff": dv.tolist(), "variance_err": res["err_variance"].tolist(), "wall_s": dt}


def profile_steps(nsteps, warmup, precision):
    """The benchmark chain for a profiler: warm-up steps, then `nsteps` steps
    inside the NVTX range "timed"."""
    import torch
    import multigridmc_gb300 as M
    op, f, _, _, _ = problem()
    prec = M.FP32_MIXED if precision == "fp32" else M.FP64
    s = M.MultigridMCSampler(op, M.MultigridParameters(nlevel=NLEVEL), ordering=M.MULTICOLOUR, precision=prec,
                             noise=M.PHILOX, seed=1)
    s.fix_rhs(f)
    s.step(warmup)
    s.synchronize()
    torch.cuda.nvtx.range_push("timed")
    s.step(nsteps)
    s.synchronize()
    torch.cuda.nvtx.range_pop()
    print(f"profiled {nsteps} steps, {s.launches_per_step} launches per step", flush=True)
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--iact-samples", type=int, default=20000,
                    help="samples of the coupled FP32-mixed / FP64 run after the timed steps: IACT and the "
                         "probe covariances")
    ap.add_argument("--cov-probes", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the compact runs of configs 1, 2, 4 and 5 after the headline measurement")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--covariance-study", type=int, default=0, metavar="NSAMPLES",
                    help="run the coupled FP32/FP64 covariance comparison instead of the benchmark")
    ap.add_argument("--batch-chains", type=int, default=0, metavar="N",
                    help="run the batched-chains study (N chains of mixed sizes) instead of the benchmark")
    ap.add_argument("--convergence-study", type=int, default=0, metavar="NCHAIN",
                    help="run measure_convergence over NCHAIN batched chains (--steps steps) instead of the benchmark")
    ap.add_argument("--adjoint-study", action="store_true",
                    help="run the 128^3 differentiation study (parameter adjoint with checkpoints, FD checks)")
    ap.add_argument("--summary-study", action="store_true",
                    help="MGMC vs Gibbs vs exact sampler at 16^3 .. 128^3 (the reference's summary comparison)")
    ap.add_argument("--variable-study", action="store_true",
                    help="the 256^3 posterior with the periodic correlation length (variable coefficients)")
    ap.add_argument("--solve-study", action="store_true",
                    help="time the deterministic multigrid solve of Q x = f instead of the benchmark")
    ap.add_argument("--profile-steps", type=int, default=0, metavar="K",
                    help="profiling mode: K steps of the benchmark chain inside an NVTX range 'timed' "
                         "(after --warmup steps), for ncu --nvtx-include timed/; prints no JSON")
    ap.add_argument("--profile-precision", default="fp32", choices=["fp32", "fp64"])
    args = ap.parse_args()
    if args.profile_steps > 0:
        profile_steps(args.profile_steps, max(3, args.warmup), args.profile_precision)
        return
    if args.batch_chains > 0:
        print(json.dumps({"batch_study": batch_study(args.batch_chains, args.steps)}), flush=True)
        return
    if args.convergence_study > 0:
        print(json.dumps({"convergence_study": convergence_study(args.convergence_study, args.steps)}), flush=True)
        return
    if args.adjoint_study:
        print(json.dumps({"adjoint_study": adjoint_study()}), flush=True)
        return
    if args.summary_study:
        print(json.dumps({"summary_study": summary_study()}), flush=True)
        return
    if args.variable_study:
        print(json.dumps({"variable_study": variable_study()}), flush=True)
        return
    if args.solve_study:
        print(json.dumps({"solve_study": solve_study()}), flush=True)
        return
    if args.covariance_study > 0:
        print(json.dumps({"covariance_study": covariance_study(args.covariance_study)}), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        r = cpu_reference(nsteps=args.steps, warmup=args.warmup)
        val = 1.0 / r["per_step_s"] / PUBLISHED_MGMC_IACT
        sample = (f"{r['steps']} MGMC steps (after {args.warmup} untimed) of the oracle's reference restatement at "
                  f"256^3, m=64 (lexicographic SOR, dense B-bar, CLCG), one chain, {r['threads']} OpenMP threads "
                  f"in the dense products; IACT {PUBLISHED_MGMC_IACT} = the reference's published MGMC IACT at "
                  f"64^3 (python/plot_summary.py:28), not measured at 256^3 on the CPU; setup "
                  f"{r['setup_s']:.1f} s untimed; host {r['host']}")
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": args.warmup, "ms_per_step": r["per_step_s"] * 1e3,
                "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "unknowns": int(np.prod([n - 1 for n in SHAPE])),
                           "precision": "fp64", "ordering": "lexicographic (the reference's sweep order)"},
                "cpu_baseline": {"value": val, "unit": UNIT, "cores": r["threads"], "kind": "port", "sample": sample},
                "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        dist = tdist
    import multigridmc_gb300 as M

    op, f, obs, _, _ = problem()
    peak, peak_kind = measured_peaks()
    clocks = ClockSampler(local)
    rng = np.random.default_rng(2)
    probe_pts = rng.choice(op.n, size=args.cov_probes, replace=False)
    probes = [(np.array([p], np.int64), np.array([1.0])) for p in probe_pts] + [obs]

    # FP32-mixed headline chain (clocks sampled during its timed region),
    # then the coupled covariance run on the same chain
    clocks.start()
    s32, ms32, _ = time_chain(M, torch, op, f, obs, M.FP32_MIXED, args.steps, args.warmup, 0, dist, 1000 + rank)
    clk = clocks.stop()
    launches = s32.launches_per_step
    Z32 = coupled_run(s32, probes, args.iact_samples)
    ach, bpl, tl = sweep_roofline(M, torch, s32, M.FP32_MIXED, peak)
    kernels = kernel_table(M, torch, s32, M.FP32_MIXED, peak, tl)
    s32.close()
    # FP64 chain: same seed, so it draws the FP32 chain's normals (coupled
    # chains): the two IACT estimates share their Monte Carlo noise, the ratio
    # of the two values is the cost ratio of equal-quality samples, and the
    # sample covariances differ only by the FP32 chain's rounding
    s64, ms64, _ = time_chain(M, torch, op, f, obs, M.FP64, args.steps, args.warmup, 0, dist, 1000 + rank)
    Z64 = coupled_run(s64, probes, args.iact_samples)
    ach64, bpl64, tl64 = sweep_roofline(M, torch, s64, M.FP64, peak)
    s64.close()
    iact32 = M.statistics.tau_int(Z32[:, -1], IACT_WINDOW)
    iact64 = M.statistics.tau_int(Z64[:, -1], IACT_WINDOW)
    cov = covariance_figures(M, op, f, probe_pts, Z32, Z64, iact32, iact64, exact=(rank == 0 and world == 1))

    ms32, ms64 = replica_max([ms32, ms64], dist, "cuda")
    value = replica_rate(world, ms32 / 1000.0, iact32)
    value64 = replica_rate(world, ms64 / 1000.0, iact64)

    e2e_val, e2e_dt, h2d, d2h = time_e2e(M, torch, op, f, M.FP32_MIXED, args.e2e_steps, 1000 + rank, iact32)
    e2e64_val, e2e64_dt, _, _ = time_e2e(M, torch, op, f, M.FP64, args.e2e_steps, 1000 + rank, iact64)
    _, e2eu_dt, h2du, d2hu = time_e2e(M, torch, op, f, M.FP32_MIXED, args.e2e_steps, 1000 + rank, iact32, fixed=False)
    e2e_dt, e2e64_dt, e2eu_dt = replica_max([e2e_dt, e2e64_dt, e2eu_dt], dist, "cuda")
    e2e_val = replica_rate(world, e2e_dt, iact32)
    e2e64_val = replica_rate(world, e2e64_dt, iact64)
    e2eu_val = replica_rate(world, e2eu_dt, iact32)
    fma = {"fp64_tflops": M.device_fma_rate(M.FP64), "fp32_tflops": M.device_fma_rate(M.FP32_MIXED),
           "how": "mgmc_device_fma_rate: 8 independent FMA chains per thread, 8 CTAs x 256 threads per SM, "
                  "~20 ms per launch, best of 3, CUDA events"}

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        try:
            r = cpu_reference(seconds_budget=args.cpu_seconds)
            cv = 1.0 / r["per_step_s"] / PUBLISHED_MGMC_IACT
            cpu = {"value": cv, "unit": UNIT, "cores": r["threads"], "kind": "port",
                   "sample": (f"{r['steps']} oracle MGMC steps at 256^3 m=64 (reference algorithm: lexicographic "
                              f"SOR, dense B-bar, CLCG), {r['per_step_s']:.2f} s/step; IACT {PUBLISHED_MGMC_IACT} "
                              f"= the reference's published MGMC IACT at 64^3 (python/plot_summary.py:28), not "
                              f"measured at 256^3 on the CPU; host {r['host']}")}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}

    configs = configs_section() if (world == 1 and not args.no_configs) else None

    n = int(op.n)
    sweep_bytes = 3 * n * 4
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 Cholesky factorisation; m x m low-rank system in float-float)", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "unknowns": n, "ordering": "multicolour (red-black fine, 8-colour coarse)",
                   "noise": "in-kernel Philox4x32-10", "parallelism": f"replicas x{world}",
                   "l2": "per-step working set > L2 (x and f alone 134 MB FP32 / 268 MB FP64)",
                   "iact_window": IACT_WINDOW, "iact_samples": int(Z32.shape[0])},
        "iact": iact32, "steps_per_s": 1000.0 / ms32,
        "covariance_rel_err": cov["fp32_vs_fp64_cov_rel_frobenius"],
        "covariance": cov,
        "fp64": {"value": value64, "ms_per_step": ms64, "iact": iact64, "steps_per_s": 1000.0 / ms64,
                 "sweep_gbs": ach64, "sweep_launch_s": tl64,
                 "e2e": {"value": e2e64_val, "unit": UNIT, "ms_per_step": e2e64_dt * 1e3,
                         "api": "mgmc_sampler_fix_rhs once, then mgmc_sampler_apply(NULL, x) per step"}},
        "kernels_fp32": kernels,
        "mixed_vs_fp64": value / value64,
        "fma_peaks": fma,
        "clocks": clk,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_dt * 1e3,
                "api": "mgmc_sampler_fix_rhs once, then mgmc_sampler_apply(NULL, x) per step with pinned host x "
                       "(measure_sampling_time's fix_rhs + apply loop)",
                "unfixed": {"value": e2eu_val, "ms_per_step": e2eu_dt * 1e3, "h2d_bytes_per_step": h2du,
                            "d2h_bytes_per_step": d2hu, "api": "mgmc_sampler_apply(f, x) per step, pinned host f, x"}},
        "gpu_launches": int(launches * args.steps),
        "launches_per_step": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "traffic": RB_VEC_DRAM_BYTES,
                     "traffic_source": RB_VEC_TRAFFIC_SOURCE,
                     "kernel": RB_VEC_KERNEL,
                     "algorithmic_bytes": "3 n s per sweep (x read, f read, x written), 1.5 n s per colour launch",
                     "algorithmic_bytes_per_launch": bpl, "launch_s": tl, "sweep_s": 2 * tl,
                     "sweep_gbs": sweep_bytes / (2 * tl) / 1e9, "peak_kind": peak_kind},
        "cpu_baseline": cpu,
        "configs": configs,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
