"""Benchmark: batched HMC on Bayesian logistic regression.

Workload (the multi-chain HMC configuration): X 10,000 x 50 fp32 iid N(0,1),
w ~ N(0,1)^50, b ~ N(0,1), y ~ Bernoulli(sigmoid(Xw + b)); priors N(0,1);
4,096 independent chains started from N(0,1); 10 leapfrog steps of size
0.005; FP32 state, FP64 accept ratio.  One "step" = one HMC iteration of all
chains (10 leapfrog steps + Metropolis test each), i.e. one launch of the
persistent HMC kernel.  Metric: chain-leapfrog-steps per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference-structured CPU restatement (one
chain per inference, GEMV per leapfrog gradient, as edward/inferences/hmc.py
runs it) on all host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_ROWS, N_FEAT, N_CHAINS, N_LEAP, STEP = 10_000, 50, 4096, 10, 0.005
METRIC = "HMC leapfrog chain-steps/s (Bayesian logistic regression, batched chains)"
UNIT = "chain-steps/s"
CONFIG = {"workload": "hmc_logreg_N10000_D50_C4096_L10", "N": N_ROWS, "D": N_FEAT,
          "chains": N_CHAINS, "leapfrog_steps": N_LEAP, "step_size": STEP,
          "state_dtype": "fp32", "ratio_dtype": "fp64"}


def make_data(seed=0):
    import numpy as np
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N_ROWS, N_FEAT)).astype(np.float32)
    w = rng.standard_normal(N_FEAT)
    b = rng.standard_normal()
    p = 1.0 / (1.0 + np.exp(-(X.astype(np.float64) @ w + b)))
    y = (rng.random(N_ROWS) < p).astype(np.float32)
    z0 = rng.standard_normal((N_CHAINS, N_FEAT + 1)).astype(np.float32)
    return X, y, z0


# ------------------------------------------------------------------ CPU baseline

def _cpu_worker(args):
    chains, n_iter, seed = args
    import numpy as np
    from oracle.cpu_baseline import hmc_logreg_chain
    X, y, z0 = make_data()
    P = N_FEAT + 1
    t0 = time.perf_counter()
    for c in chains:
        hmc_logreg_chain(X, y, z0[c], n_iter, STEP, N_LEAP, seed, c,
                         np.zeros(P, np.float32), np.ones(P, np.float32))
    return time.perf_counter() - t0


def cpu_baseline(budget_s=10.0, procs=None):
    """Reference-structured CPU HMC on all host cores (one process per core,
    chains split across processes); returns a cpu_baseline dict."""
    import multiprocessing as mp
    ncores = len(os.sched_getaffinity(0))
    procs = procs or ncores
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    ctx = mp.get_context("spawn")
    # calibrate: one chain, 2 iterations
    t = _cpu_worker(([0], 2, 1))
    per_chain_iter = max(t / 2, 1e-4)
    n_iter = 2
    chains_per_proc = max(1, int(budget_s / (per_chain_iter * n_iter)))
    chains_per_proc = min(chains_per_proc, N_CHAINS // procs if N_CHAINS >= procs else 1)
    work = [(list(range(p * chains_per_proc, (p + 1) * chains_per_proc)), n_iter, 1)
            for p in range(procs)]
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        pool.map(_cpu_worker, work)
        wall = time.perf_counter() - t0
    total = procs * chains_per_proc * n_iter * N_LEAP
    return {"value": total / wall, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{procs * chains_per_proc} chains x {n_iter} HMC iterations x {N_LEAP} "
                      f"leapfrog steps, one chain at a time per process (GEMV per gradient, "
                      f"NumPy FP32, BLAS 1 thread/process), {wall:.1f} s wall"}


def _cpu_mc_worker(args):
    """Reference-structured SGLD or random-walk MH chains of the 10,000 x 50
    logistic regression (one chain at a time); returns the seconds taken."""
    kind, chains, n_iter, seed = args
    import numpy as np
    from oracle.cpu_baseline import mh_logreg_chain, sgld_logreg_chain
    X, y, z0 = make_data()
    P = N_FEAT + 1
    loc, sc = np.zeros(P, np.float32), np.ones(P, np.float32)
    t0 = time.perf_counter()
    for c in chains:
        if kind == "sgld":
            sgld_logreg_chain(X, y, z0[c], n_iter, 1e-4, seed, c, loc, sc)
        else:
            mh_logreg_chain(X, y, z0[c], n_iter, 0.01 * np.ones(P, np.float32), seed, c, loc, sc)
    return time.perf_counter() - t0


def cpu_mc_baseline(kind, budget_s=10.0):
    """SGLD / MH chains on all host cores (one process per core, chains split
    across processes, NumPy FP32, BLAS one thread per process); a
    cpu_baseline dict in chain-iterations/s."""
    import multiprocessing as mp
    procs = len(os.sched_getaffinity(0))
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    t = _cpu_mc_worker((kind, [0], 4, 1))
    per = max(t / 4, 1e-5)  # seconds per chain-iteration
    chains_per_proc = max(1, N_CHAINS // procs)
    n_iter = int(min(max(budget_s / (per * chains_per_proc), 4), 200))
    work = [(kind, list(range(p * chains_per_proc, (p + 1) * chains_per_proc)), n_iter, 1)
            for p in range(procs)]
    with mp.get_context("spawn").Pool(procs) as pool:
        t0 = time.perf_counter()
        pool.map(_cpu_mc_worker, work)
        wall = time.perf_counter() - t0
    total = procs * chains_per_proc * n_iter
    what = "gradient (2 GEMVs)" if kind == "sgld" else "two log joints (1 GEMV each)"
    return {"value": total / wall, "unit": "chain-iterations/s", "cores": procs, "kind": "port",
            "sample": f"{procs * chains_per_proc} chains x {n_iter} iterations, one chain at a "
                      f"time per process ({what} per iteration, NumPy FP32, BLAS 1 thread/"
                      f"process), {wall:.1f} s wall"}


def _cpu_hier_worker(units):
    """Reference-structured HMC iterations (one chain each) on hierarchical
    instances given as (X_i, y_i, global chain row); returns the seconds taken."""
    import numpy as np
    from oracle.cpu_baseline import hier_chain
    t0 = time.perf_counter()
    for X, y, row in units:
        hier_chain(X, y, np.zeros(X.shape[1] + 2, np.float32), 1, 0.01, 10, 1, row)
    return time.perf_counter() - t0


def cpu_hier_baseline(Xs, ys, C, L, budget_s=10.0):
    """One HMC iteration of single chains on instances drawn at random
    (seeded) from the ragged batch, on all host cores; projected to the whole
    batch by its work (sum of N_i * D_i per chain), in chain-steps/s."""
    import multiprocessing as mp
    import numpy as np
    procs = len(os.sched_getaffinity(0))
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    work = np.array([x.shape[0] * x.shape[1] for x in Xs], np.float64)
    rng = np.random.default_rng(5)
    # calibrate on a few instances
    probe = rng.integers(0, len(Xs), 4)
    t = _cpu_hier_worker([(Xs[i], ys[i], int(i) * C) for i in probe])
    per_work = max(t / work[probe].sum(), 1e-12)
    n_units = max(procs, int(procs * budget_s / (per_work * work.mean())))
    pick = rng.integers(0, len(Xs), n_units)
    groups = [[(Xs[i], ys[i], int(i) * C) for i in pick[p::procs]] for p in range(procs)]
    with mp.get_context("spawn").Pool(procs) as pool:
        t0 = time.perf_counter()
        pool.map(_cpu_hier_worker, groups)
        wall = time.perf_counter() - t0
    t_full = wall * C * work.sum() / work[pick].sum()
    return {"value": float(len(Xs) * C * L / t_full), "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{n_units} (instance, chain) pairs drawn at random, one HMC iteration "
                      f"of {L} leapfrog steps each (GEMV pair per gradient, NumPy FP32, BLAS 1 "
                      f"thread/process), {wall:.1f} s wall, projected to the whole batch by "
                      f"sum(N_i D_i)"}


# ------------------------------------------------------------------ KLqp workload (the ELBO-gradient half)

KLQP_S, KLQP_ITERS, KLQP_SEED = 5, 1000, 1
KLQP_METRIC = "KLqp ELBO-grad evals/s (Bayesian logistic regression, S=5)"
KLQP_UNIT = "evals/s"


def klqp_init():
    """q initialisation shared by the GPU run and the CPU leg: mu = 0 and
    rho ~ N(0, 1) (seed 2), so both optimise from the same point with the
    same Philox draws (seed 1)."""
    import numpy as np
    P = N_FEAT + 1
    return np.zeros(P, np.float32), np.random.default_rng(2).standard_normal(P).astype(np.float32)


def _cpu_klqp_worker(n_steps):
    import numpy as np
    from oracle.cpu_baseline import klqp_logreg_step
    from oracle.klqp import default_learning_rate
    X, y, _ = make_data()
    P = N_FEAT + 1
    mu, rho = klqp_init()
    m = np.zeros(2 * P, np.float32)
    v = np.zeros(2 * P, np.float32)
    loc, scale = np.zeros(P, np.float32), np.ones(P, np.float32)
    losses = []
    t0 = time.perf_counter()
    for t in range(n_steps):
        losses.append(klqp_logreg_step(X, y, mu, rho, m, v, t, KLQP_S, KLQP_SEED, loc, scale,
                                       default_learning_rate(t)))
    return time.perf_counter() - t0, losses


def cpu_klqp_baseline(n_steps=KLQP_ITERS):
    """The reference-structured CPU KLqp (one model copy per Monte Carlo
    sample, GEMV forward + GEMV backward each, analytic KL, unfused TF Adam;
    NumPy FP32) for the whole 1,000-step optimisation, in one spawned process
    whose BLAS uses every host core (the reference's TF intra-op pool).
    Returns the cpu_baseline dict and the final ELBO per datum (mean of the
    last 100 losses / N)."""
    import multiprocessing as mp
    import numpy as np
    ncores = len(os.sched_getaffinity(0))
    keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = str(ncores)
    try:
        with mp.get_context("spawn").Pool(1) as pool:
            dt, losses = pool.apply(_cpu_klqp_worker, (n_steps,))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    elbo = -float(np.mean(losses[-100:])) / N_ROWS
    cb = {"value": n_steps / dt, "unit": KLQP_UNIT, "cores": ncores, "kind": "port",
          "sample": f"the full {n_steps}-step optimisation (S={KLQP_S}, analytic KL, TF Adam, "
                    f"staircase lr), one process, BLAS on {ncores} threads, {dt:.1f} s wall"}
    return cb, elbo


def _cpu_net_worker(kind, n_steps):
    """Times n_steps of the reference-structured CPU step of a network
    workload (after one untimed step); returns (seconds, steps)."""
    import numpy as np
    from oracle import cpu_baseline as cb
    if kind == "bnn":
        N, D, H1, H2, M, S = 100000, 32, 256, 256, 4096, 64
        X, y = bnn_data(N, D, H1, H2)
        X, y = X[:M], y[:M]
        P = D * H1 + H1 + H1 * H2 + H2 + H2 + 1
        rng = np.random.default_rng(1)
        mu = (rng.standard_normal(P) * 0.1).astype(np.float32)
        rho = np.full(P, -3.0, np.float32)
        m, v = np.zeros(2 * P, np.float32), np.zeros(2 * P, np.float32)
        step = lambda t: cb.bnn_klqp_step(X, y, mu, rho, m, v, t, S, 1, 0.1, N / M,  # noqa: E731
                                          D, H1, H2, 1e-3)
    else:
        V, H0, H1, B, S = 784, 200, 200, 1024, 16
        X = sbn_data(V=V, H0=H0, H1=H1)[:B].astype(np.float32)
        P = (V + 1) * H0 + (H0 + 1) * H1 + (H1 + 1) * H0 + (H0 + 1) * V
        theta = (np.random.default_rng(1).standard_normal(P) * 0.05).astype(np.float32)
        m, v = np.zeros(P, np.float32), np.zeros(P, np.float32)
        step = lambda t: cb.sbn_score_step(X, theta, m, v, t, S, 1, V, H0, H1, 1e-3)  # noqa: E731
    step(0)
    t0 = time.perf_counter()
    for t in range(1, n_steps + 1):
        step(t)
    return time.perf_counter() - t0, n_steps


def cpu_net_baseline(kind, n_steps, what):
    """cpu_baseline record for a network workload: the reference-structured
    CPU step (one model copy per Monte Carlo sample, NumPy FP32) in one spawned
    process whose BLAS uses every host core."""
    import multiprocessing as mp
    ncores = len(os.sched_getaffinity(0))
    keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = str(ncores)
    try:
        with mp.get_context("spawn").Pool(1) as pool:
            dt, n = pool.apply(_cpu_net_worker, (kind, n_steps))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return {"value": n / dt, "unit": "evals/s", "cores": ncores, "kind": "port",
            "sample": f"{n} steps of {what} after one untimed step, one process, BLAS on "
                      f"{ncores} threads, {dt:.1f} s wall"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cb = None
    steps = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(budget_s=max(2.0, 20.0 / max(1, args.steps + args.warmup)))
        if i >= args.warmup:
            steps.append(r)
        cb = r
    val = statistics.median(s["value"] for s in steps)
    cb = dict(cb)
    cb["value"] = val
    kcb, kelbo = cpu_klqp_baseline()
    klqp = {"metric": KLQP_METRIC, "value": kcb["value"], "unit": KLQP_UNIT,
            "higher_is_better": True, "config": {"workload": "klqp_logreg_N10000_D50_S5_T1000"},
            "cpu_baseline": kcb, "final_elbo_per_datum": kelbo,
            "e2e": {"value": kcb["value"], "unit": KLQP_UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * N_CHAINS * N_LEAP / val, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(CONFIG, l2_flush="n/a (CPU)"), "impl": "reference",
            "cpu_baseline": cb,
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "klqp": klqp}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ clocks

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        else:
            self.out = ""

    def summary(self):
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxes.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes),
                "reasons": sorted(reasons), "samples": len(sms)}


# ------------------------------------------------------------------ GPU arm

def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # CPU baseline first (spawned pool before heavy GPU work), rank 0 at N=1 only
    cb = cpu_klqp = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(budget_s=args.cpu_budget)
        if not args.no_extras:
            cpu_klqp = cpu_klqp_baseline()

    import edward_gb300 as ed
    from edward_gb300 import _lib
    from edward_gb300.models import Bernoulli, Empirical, Normal

    X, y, z0 = make_data()
    tf32 = None if args.no_extras else measure_tf32_peak(dev)
    T = args.warmup + args.steps
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yrv = Bernoulli(logits=ed.dot(X, w) + b)
    qw_init = np.zeros((T, N_CHAINS, N_FEAT), np.float32)
    qb_init = np.zeros((T, N_CHAINS), np.float32)
    qw_init[0] = z0[:, :N_FEAT]
    qb_init[0] = z0[:, N_FEAT]
    qw = Empirical(ed.Variable(qw_init, trainable=False), n_chains=N_CHAINS)
    qb = Empirical(ed.Variable(qb_init, trainable=False), n_chains=N_CHAINS)
    inf = ed.HMC({w: qw, b: qb}, data={yrv: y}, n_chains=N_CHAINS)
    inf.initialize(step_size=STEP, n_steps=N_LEAP, n_print=0, engine=args.engine,
                   chains_per_block=args.ct)
    kernel_name = ("hmc_glm_tc_kernel (tcgen05 3xTF32, one CTA cluster per 128 chains)"
                   if inf.engine == "tc"
                   else "hmc_glm_kernel<%d> (SIMT FP32)" % inf._cfg.chains_per_block)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        inf.run_iterations(1)
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))               # L2 flush (256 MB write), outside the events
            ev[i][0].record(stream)
            inf.run_iterations(1)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if world > 1:
        dist.barrier()
    per_step = [a.elapsed_time(bb) for a, bb in ev]
    t_ms = sum(per_step)
    if world > 1:
        tt = torch.tensor([t_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    units = N_CHAINS * N_LEAP * args.steps
    value = world * units / (t_ms / 1e3)

    # accept-rate sanity (posterior moves, chains not stuck)
    acc = float(inf._n_accept.sum().item()) / (N_CHAINS * T)

    # end-to-end through the C ABI with host buffers (copies inside the timed region)
    e2e = run_e2e(args, inf, X, y, z0, dev)

    # roofline of the dominant kernel (the persistent HMC kernel is the only launch per step)
    P = N_FEAT + 1
    flops_per_launch = 4.0 * N_ROWS * P * N_CHAINS * N_LEAP
    avg_launch_ms = statistics.mean(per_step)
    achieved = flops_per_launch / (avg_launch_ms / 1e3) / 1e12
    peak, psrc = tensor_peak(tf32)
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": read_traffic(inf.engine),
            "kernel": kernel_name, "peak_source": psrc,
            "tf32_tflops_measured": tf32,
            "algorithmic_flops_per_launch": flops_per_launch}

    extras = {}
    if not args.no_extras and rank == 0:
        extras["klqp"] = run_klqp_record(args, dev, X, y, cpu_klqp, flush, tf32)
        posterior, target_hmc = run_hmc_posterior_and_target(args, dev, X, y, z0)
        extras["posterior"] = posterior
        extras["target"] = {"hmc": target_hmc, "klqp": run_klqp_target(X, y, dev)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": dict(CONFIG,
                               l2_flush="256 MB write before each step, outside the timed events"),
                "parallelism": f"replicas{world}", "engine": inf.engine,
                "accept_rate": round(acc, 4),
                "e2e": e2e, "gpu_launches": args.steps, "roofline": roof,
                "cpu_baseline": cb, "clocks": clk.summary(),
                "wall_s_timed_region": wall}
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_e2e(args, inf, X, y, z0, dev):
    """Same metric through the C ABI with host buffers: every step copies X, y
    and the chain state (z, cached gradient and log joint) from pinned host
    memory, re-lays X for the engine when it needs it, runs one iteration with
    the engine the inference selected, and copies the state and the kept
    sample back.  The step's buffers are packed into one pinned host buffer
    mirrored by one device buffer, [X | y | state record | z | g | lj |
    sample], so that each step makes one host->device copy (X .. lj) and one
    device->host copy (z .. sample); the host copy of the state record
    (iteration t = 0) is never overwritten, so every step starts at t = 0 while
    the chain state held on the host advances."""
    import ctypes
    import torch
    from edward_gb300 import _lib
    P = N_FEAT + 1
    sizes = [("X", X.size * 4), ("y", y.size * 4), ("st", ctypes.sizeof(_lib.EdgState)),
             ("z", N_CHAINS * P * 4), ("g", N_CHAINS * P * 4), ("lj", N_CHAINS * 8),
             ("s", N_CHAINS * P * 4)]
    off, o = {}, 0
    for name, nbytes in sizes:
        off[name] = (o, nbytes)
        o += (nbytes + 255) // 256 * 256
    total = o
    h_buf = torch.zeros(total, dtype=torch.uint8).pin_memory()

    def hview(name, dtype):
        o0, nb = off[name]
        return h_buf[o0:o0 + nb].view(dtype)

    hview("X", torch.float32).copy_(torch.as_tensor(X).reshape(-1))
    hview("y", torch.float32).copy_(torch.as_tensor(y).reshape(-1))
    hview("z", torch.float32).copy_(torch.as_tensor(z0).reshape(-1))
    st0 = _lib.EdgState()
    st0.beta1_power, st0.beta2_power = 0.9, 0.999
    hview("st", torch.uint8).copy_(torch.frombuffer(bytearray(bytes(st0)), dtype=torch.uint8))
    d_buf = torch.empty(total, dtype=torch.uint8, device=dev)
    base = d_buf.data_ptr()

    def dptr(name):
        return ctypes.c_void_p(base + off[name][0])

    in_end = off["lj"][0] + off["lj"][1]
    out_begin = off["z"][0]
    out_end = off["s"][0] + off["s"][1]
    glm = _lib.EdgGLM()
    glm.X, glm.y, glm.N, glm.D, glm.bias, glm.lik, glm.lik_scale = (
        base + off["X"][0], base + off["y"][0], N_ROWS, N_FEAT, 1, 0, 1.0)
    glm.prior_loc = inf._glm.prior_loc.data_ptr()
    glm.prior_scale = inf._glm.prior_scale.data_ptr()
    cfg = inf._cfg
    stream = torch.cuda.current_stream()
    sp = _lib.stream_ptr(stream)
    lib = _lib.load()
    tc = inf.engine == "tc"
    if tc:
        nb = lib.edg_hmc_glm_tc_tiles_bytes(ctypes.byref(glm))
        tiles = torch.empty(nb, dtype=torch.uint8, device=dev)
    h_in, d_in = h_buf[:in_end], d_buf[:in_end]
    h_out, d_out = h_buf[out_begin:out_end], d_buf[out_begin:out_end]

    def step(cache_valid):
        d_in.copy_(h_in, non_blocking=True)
        if tc:
            _lib.call("edg_hmc_glm_tc_prepare", ctypes.byref(glm), _lib.ptr(tiles), nb, sp)
            _lib.call("edg_hmc_glm_tc_run", ctypes.byref(glm), ctypes.byref(cfg), N_CHAINS, 1,
                      _lib.ptr(tiles), dptr("z"), dptr("g"), dptr("lj"), cache_valid,
                      None, dptr("st"), dptr("s"), 1, None, None, None, None, sp)
        else:
            _lib.call("edg_hmc_glm_run", ctypes.byref(glm), ctypes.byref(cfg), N_CHAINS, 1,
                      dptr("z"), dptr("g"), dptr("lj"), cache_valid, None,
                      dptr("st"), dptr("s"), 1, None, None, None, None, sp)
        h_out.copy_(d_out, non_blocking=True)
        stream.synchronize()

    step(0)  # builds the gradient cache for the host-held state
    for _ in range(max(0, args.warmup - 1)):
        step(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(1)
    dt = time.perf_counter() - t0
    name = "edg_hmc_glm_tc_prepare + edg_hmc_glm_tc_run" if tc else "edg_hmc_glm_run"
    return {"value": N_CHAINS * N_LEAP * args.steps / dt, "unit": UNIT,
            "h2d_bytes_per_step": int(in_end), "d2h_bytes_per_step": int(out_end - out_begin),
            "path": f"{name} (C ABI), one packed pinned host buffer, one copy each way per step, "
                    "wall clock"}


def measure_tf32_peak(dev, n=8192, reps=10):
    """Dense TF32 tensor-core rate of this GPU, measured here: cuBLAS FP32 GEMM
    with TF32 math (torch.matmul with allow_tf32), n^3, best of `reps` after
    warm-up, CUDA events.  The 3xTF32 kernels' roofline is this rate / 3."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        c = torch.empty(n, n, device=dev)
        for _ in range(3):
            torch.matmul(a, b, out=c)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def tensor_peak(tf32_tflops):
    """(3xTF32 peak, source) from the TF32 rate measured in this run, else from
    MEASURED_PEAKS.json's bf16 rate / 2."""
    if tf32_tflops:
        return tf32_tflops / 3.0, (f"cuBLAS TF32 GEMM 8192^3 measured in this run: "
                                   f"{tf32_tflops:.0f} TFLOP/s / 3 (3xTF32 passes), of measured")
    p, src = _peak_3xtf32()
    return p, src


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs, of measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s, of fallback"


def _klqp_inference(X, y):
    import torch
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Normal
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    inf = ed.KLqp([w, b], data={yv: y})
    inf.initialize(n_samples=KLQP_S, n_iter=KLQP_ITERS, n_print=0)
    inf._cfg.seed = KLQP_SEED
    mu0, rho0 = klqp_init()

    def restart():
        inf.reset()
        inf._graphs = {}
        inf._mu.copy_(torch.as_tensor(mu0))
        inf._rho.copy_(torch.as_tensor(rho0))
    restart()
    return inf, restart


def run_klqp_record(args, dev, X, y, cpu_klqp, flush, tf32):
    """The KLqp half of the metric on the S = 5 logistic regression: ELBO-grad
    evals/s of the fused step (one launch per step: Philox eps, X z for all
    samples, log-likelihood + adjoint, analytic KL, Adam), device-timed with an
    L2 flush before every step; the whole 1,000-step run and its final ELBO;
    the same step end to end through the C ABI with host buffers."""
    import ctypes
    import numpy as np
    import torch
    from edward_gb300 import _lib
    inf, restart = _klqp_inference(X, y)
    stream = torch.cuda.current_stream()
    # the full optimisation: 900 steps from CUDA graphs, the last 100 read one by one
    t0 = time.perf_counter()
    for _ in range(18):
        inf.steps(50)
    losses = []
    for _ in range(100):
        inf._step(apply=True)
        losses.append(float(inf._read_state().loss))
    torch.cuda.synchronize()
    run_wall = time.perf_counter() - t0
    final_elbo = -float(np.mean(losses)) / N_ROWS
    assert inf.t == KLQP_ITERS
    # device-timed steps, L2 flushed before each (outside the events)
    restart()
    for _ in range(5):
        inf._step(apply=True)
    torch.cuda.synchronize()
    K = args.klqp_steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    with ClockSampler(dev.index or 0) as clk:
        for i in range(K):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            inf._step(apply=True)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    per = [a.elapsed_time(b) for a, b in ev]
    ms = sum(per) / K
    # the same steps replayed back to back from a CUDA graph (X L2-resident)
    restart()
    inf.steps(50)
    inf.steps(50)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(10):
        inf.steps(50)
    b.record()
    b.synchronize()
    ms_graph = a.elapsed_time(b) / 500
    # end to end through the C ABI: X, y and the optimiser state copied in from
    # pinned host memory and the state copied back every step
    P = N_FEAT + 1
    sizes = [("X", X.size * 4), ("y", y.size * 4), ("mu", P * 4), ("rho", P * 4),
             ("slots", 4 * P * 4), ("st", ctypes.sizeof(_lib.EdgState))]
    off, o = {}, 0
    for name, nbytes in sizes:
        off[name] = (o, nbytes)
        o += (nbytes + 255) // 256 * 256
    h = torch.zeros(o, dtype=torch.uint8).pin_memory()

    def hview(name, dtype):
        o0, nb = off[name]
        return h[o0:o0 + nb].view(dtype)
    mu0, rho0 = klqp_init()
    hview("X", torch.float32).copy_(torch.as_tensor(X).reshape(-1))
    hview("y", torch.float32).copy_(torch.as_tensor(y).reshape(-1))
    hview("mu", torch.float32).copy_(torch.as_tensor(mu0))
    hview("rho", torch.float32).copy_(torch.as_tensor(rho0))
    hview("st", torch.uint8).copy_(_lib.new_state("cpu"))
    d = torch.empty(o, dtype=torch.uint8, device=dev)
    base = d.data_ptr()
    glm = _lib.EdgGLM()
    glm.X, glm.y, glm.N, glm.D, glm.bias, glm.lik, glm.lik_scale = (
        base + off["X"][0], base + off["y"][0], N_ROWS, N_FEAT, 1, 0, 1.0)
    glm.prior_loc = inf._glm.prior_loc.data_ptr()
    glm.prior_scale = inf._glm.prior_scale.data_ptr()
    out0 = off["mu"][0]
    sp = _lib.stream_ptr(stream)

    def e2e_step():
        d.copy_(h, non_blocking=True)
        _lib.call("edg_klqp_glm_step", ctypes.byref(glm), ctypes.byref(inf._cfg),
                  ctypes.byref(inf._opt), ctypes.c_void_p(base + off["mu"][0]),
                  ctypes.c_void_p(base + off["rho"][0]), ctypes.c_void_p(base + off["slots"][0]),
                  ctypes.c_void_p(base + off["st"][0]), None, None, 1, _lib.ptr(inf._ws),
                  inf._ws_bytes, sp)
        h[out0:].copy_(d[out0:], non_blocking=True)
        stream.synchronize()
    for _ in range(5):
        e2e_step()
    hview("mu", torch.float32).copy_(torch.as_tensor(mu0))
    hview("rho", torch.float32).copy_(torch.as_tensor(rho0))
    hview("slots", torch.float32).zero_()
    hview("st", torch.uint8).copy_(_lib.new_state("cpu"))
    t0 = time.perf_counter()
    for _ in range(K):
        e2e_step()
    e2e_dt = time.perf_counter() - t0
    st_h = _lib.EdgState.from_buffer_copy(bytes(hview("st", torch.uint8).numpy().tobytes()))
    assert st_h.t == K and np.isfinite(st_h.loss)
    hbm, hsrc = hbm_peak()
    alg_bytes = 4.0 * N_ROWS * N_FEAT + 4.0 * N_ROWS
    achieved = alg_bytes / (ms / 1e3) / 1e9
    rec = {"metric": KLQP_METRIC, "value": 1e3 / ms, "unit": KLQP_UNIT, "steps": K,
           "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
           "config": {"workload": "klqp_logreg_N10000_D50_S5_T1000", "n_samples": KLQP_S,
                      "n_iter": KLQP_ITERS, "optimizer": "Adam, lr 0.1 * 0.9^(t/100) staircase",
                      "l2_flush": "256 MB write before each timed step, outside the events"},
           "value_graph_l2_resident": 1e3 / ms_graph,
           "e2e": {"value": K / e2e_dt, "unit": KLQP_UNIT,
                   "h2d_bytes_per_step": int(o), "d2h_bytes_per_step": int(o - out0),
                   "path": "edg_klqp_glm_step (C ABI), one packed pinned host buffer "
                           "[X | y | mu | rho | slots | state] copied in and the optimiser "
                           "state copied out every step, wall clock"},
           "gpu_launches": K,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "traffic": read_traffic_file(
                            "klqp_glm_kernel_logreg_S5.txt"),
                        "kernel": "klqp_glm_kernel<8> (fused step, 79 blocks of 128 rows)",
                        "peak_source": hsrc, "algorithmic_bytes_per_launch": alg_bytes,
                        "note": "2 MB of X per step: launch- and latency-bound by construction"},
           "final_elbo_per_datum": final_elbo, "run_wall_s_1000_steps": run_wall,
           "cpu_baseline": cpu_klqp[0] if cpu_klqp else None,
           "cpu_final_elbo_per_datum": cpu_klqp[1] if cpu_klqp else None,
           "clocks": clk.summary()}
    if cpu_klqp:
        rec["final_elbo_abs_diff_vs_cpu"] = abs(final_elbo - cpu_klqp[1])
    return rec


def plain_klqp_torch(X, y, n_iter, dev):
    """The plain GPU method for KLqp: the reference's execution on a GPU one op
    at a time, as TF runs its graph there -- per Monte Carlo sample a copy of
    the model (GEMV over X, Bernoulli log-likelihood), the analytic KL,
    autodiff, and an unfused Adam with the staircase learning rate.  Eager
    torch ops; a comparison arm only (nothing of the library runs in it).
    Returns (wall seconds, losses)."""
    import torch
    import torch.nn.functional as F
    mu0, rho0 = klqp_init()
    Xd = torch.as_tensor(X, device=dev)
    yd = torch.as_tensor(y, device=dev)
    mu = torch.tensor(mu0, device=dev, requires_grad=True)
    rho = torch.tensor(rho0, device=dev, requires_grad=True)
    opt = torch.optim.Adam([mu, rho], lr=0.1, betas=(0.9, 0.999), eps=1e-8)
    gen = torch.Generator(device=dev)
    gen.manual_seed(KLQP_SEED)
    losses = torch.empty(n_iter, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(n_iter):
        for grp in opt.param_groups:
            grp["lr"] = 0.1 * 0.9 ** (t // 100)
        sig = F.softplus(rho)
        ll = 0.0
        for _ in range(KLQP_S):
            z = mu + sig * torch.randn(N_FEAT + 1, device=dev, generator=gen)
            eta = Xd @ z[:N_FEAT] + z[N_FEAT]
            ll = ll + (yd * eta - F.softplus(eta)).sum()
        kl = (0.5 * mu * mu + 0.5 * (sig * sig - 1.0) - torch.log(sig)).sum()
        loss = -(ll / KLQP_S - kl)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        losses[t] = loss.detach()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, losses.cpu().numpy()


def run_klqp_target(X, y, dev, chunk=10):
    """Spec target for KLqp: wall time for the fused step to come within
    0.1 nat/datum of the plain GPU method's final ELBO (mean of its last 100
    losses after 1,000 steps), against the plain method's 1,000-step time.
    The fused run reads the loss after every `chunk` steps (replayed from a
    CUDA graph) and stops at the first chunk whose ELBO estimate (mean of the
    last 5 chunk-end losses) is there; the reads count in its time."""
    import numpy as np
    import torch
    plain_wall, plain_losses = plain_klqp_torch(X, y, KLQP_ITERS, dev)
    plain_elbo = -float(np.mean(plain_losses[-100:])) / N_ROWS
    inf, restart = _klqp_inference(X, y)
    inf.steps(chunk)
    torch.cuda.synchronize()
    restart()
    torch.cuda.synchronize()
    recent, steps, reached = [], 0, None
    t0 = time.perf_counter()
    while steps < KLQP_ITERS:
        inf.steps(chunk)
        steps += chunk
        recent.append(float(inf._read_state().loss))
        est = -float(np.mean(recent[-5:])) / N_ROWS
        if len(recent) >= 5 and est >= plain_elbo - 0.1:
            reached = time.perf_counter() - t0
            break
    # the fused run's whole 1,000 steps, for the same-work comparison
    restart()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(KLQP_ITERS // 50):
        inf.steps(50)
    torch.cuda.synchronize()
    full_wall = time.perf_counter() - t1
    return {"plain_method": "eager per-op GPU form (per-sample GEMV copies, autodiff, "
                            "unfused Adam), 1,000 steps",
            "fused_wall_s_1000_steps": full_wall,
            "wall_time_ratio_1000_steps": plain_wall / full_wall,
            "plain_wall_s": plain_wall, "plain_final_elbo_per_datum": plain_elbo,
            "fused_steps_to_within_0.1_nat": steps if reached is not None else None,
            "fused_wall_s": reached, "fused_elbo_per_datum_at_stop": est,
            "wall_time_ratio": (plain_wall / reached) if reached else None}


def _hmc_glm(X, y, dev):
    """Device copy of the logistic-regression model for direct C-ABI runs."""
    import numpy as np
    from edward_gb300.compile import GLMSpec
    from edward_gb300.ops import GLMDevice
    P = N_FEAT + 1
    spec = GLMSpec(X=X, y=y, bias=True, lik=0, lik_scale=1.0,
                   prior_loc=np.zeros(P, np.float32), prior_scale=np.ones(P, np.float32))
    return GLMDevice(spec, dev)


def _hmc_launch(g, tiles, engine, z, gr, lj, cache, n_iter, st, seed, samples=None,
                moments=None, nacc=None):
    import ctypes
    from edward_gb300 import _lib
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed = STEP, N_LEAP, seed
    C = z.shape[0]
    T = samples.shape[0] if samples is not None else 0
    if engine == "tc":
        _lib.call("edg_hmc_glm_tc_run", g.ref(), ctypes.byref(cfg), C, n_iter, _lib.ptr(tiles),
                  _lib.ptr(z), _lib.ptr(gr), _lib.ptr(lj), cache, _lib.ptr(nacc), _lib.ptr(st),
                  _lib.ptr(samples), T, _lib.ptr(moments), None, None, None, _lib.stream_ptr())
    else:
        cfg.chains_per_block = 8
        _lib.call("edg_hmc_glm_run", g.ref(), ctypes.byref(cfg), C, n_iter, _lib.ptr(z),
                  _lib.ptr(gr), _lib.ptr(lj), cache, _lib.ptr(nacc), _lib.ptr(st),
                  _lib.ptr(samples), T, _lib.ptr(moments), None, None, None, _lib.stream_ptr())


def run_hmc_posterior_and_target(args, dev, X, y, z0):
    """Posterior error of the batched sampler and the spec wall-time
    comparison for HMC on the 10,000 x 50 logistic regression.

    * truth: the batched tensor-core run, 4,096 chains, 200 burn-in
      iterations, then 300 iterations of running moments (1.2 M draws);
    * long single-chain run (one chain, one launch):
      1,000 burn-in + args.long_chain_iters iterations, its mean and variance
      against the truth, with its batch-means standard error;
    * plain GPU method: one chain, one launch per iteration, the
      configuration's 2,000 iterations from an N(0, 1) start, mean over the
      second half; batched form: 4,096 chains, one tensor-core launch per
      iteration from N(0, 1) starts, mean over the second half of the
      iterations run so far at checkpoints k = 2, 4, ..., 512; the wall time
      of the first checkpoint whose posterior-mean error (max over
      coordinates of |mean - truth| / posterior sd) is at most the plain
      method's is compared with the plain method's wall time."""
    import numpy as np
    import torch
    from edward_gb300 import _lib
    P = N_FEAT + 1
    g = _hmc_glm(X, y, dev)
    lib = _lib.load()
    nb = lib.edg_hmc_glm_tc_tiles_bytes(g.ref())
    tiles = torch.empty(nb, dtype=torch.uint8, device=dev)
    _lib.call("edg_hmc_glm_tc_prepare", g.ref(), _lib.ptr(tiles), nb, _lib.stream_ptr())

    def fresh(C, start):
        z = torch.as_tensor(start, device=dev).reshape(C, P).clone()
        return (z, torch.zeros(C, P, device=dev), torch.zeros(C, dtype=torch.float64, device=dev),
                _lib.new_state(dev), torch.zeros(C, dtype=torch.int32, device=dev))
    # truth
    C = N_CHAINS
    z, gr, lj, st, nacc = fresh(C, z0)
    _hmc_launch(g, tiles, "tc", z, gr, lj, 0, 200, st, 11, nacc=nacc)
    mom = torch.zeros(2, C, P, dtype=torch.float64, device=dev)
    _hmc_launch(g, tiles, "tc", z, gr, lj, 1, 300, st, 11, moments=mom, nacc=nacc)
    torch.cuda.synchronize()
    n_t = 300 * C
    m_true = (mom[0].sum(0) / n_t).cpu().numpy()
    v_true = (mom[1].sum(0) / n_t).cpu().numpy() - m_true ** 2
    sd_true = np.sqrt(v_true)
    acc_true = float(nacc.double().mean().item()) / 500
    # long single chain (one launch; the tensor-core engine is the faster one
    # for a single chain: 0.55 ms against 1.9 ms per iteration on the SIMT one)
    T_long = args.long_chain_iters
    z, gr, lj, st, nacc = fresh(1, z0[0])
    _hmc_launch(g, tiles, "tc", z, gr, lj, 0, 1000, st, 12, nacc=nacc)
    samp = torch.zeros(T_long + 1000, 1, P, device=dev)
    t0 = time.perf_counter()
    _hmc_launch(g, tiles, "tc", z, gr, lj, 1, T_long, st, 12, samples=samp, nacc=nacc)
    torch.cuda.synchronize()
    long_wall = time.perf_counter() - t0
    s1 = samp[1000:1000 + T_long, 0].double().cpu().numpy()
    m1, v1 = s1.mean(0), s1.var(0)
    nbat = 20
    bm = s1[: T_long // nbat * nbat].reshape(nbat, -1, P).mean(1)
    se1 = bm.std(0, ddof=1) / np.sqrt(nbat)
    posterior = {
        "truth": f"batched tensor-core run, {C} chains x 300 iterations after 200 of burn-in "
                 f"(acceptance {acc_true:.3f})",
        "long_single_chain": f"tensor-core engine, 1 chain, {T_long} iterations after 1,000 of "
                             f"burn-in, {long_wall:.2f} s",
        "long_chain_mean_err_max_over_sd": float(np.max(np.abs(m1 - m_true) / sd_true)),
        "long_chain_mean_err_max_over_se": float(np.max(np.abs(m1 - m_true) / se1)),
        "long_chain_var_rel_err_max": float(np.max(np.abs(v1 - v_true) / v_true)),
        "posterior_sd_range": [float(sd_true.min()), float(sd_true.max())]}
    # plain GPU method: one chain, one launch per iteration (the reference's
    # one-chain update per sess.run), on each engine; the faster one is the
    # comparison point
    T_plain = 2000
    plain = {}
    for eng, tl in (("tc", tiles), ("simt", None)):
        z, gr, lj, st, nacc = fresh(1, z0[0])
        samp = torch.zeros(T_plain, 1, P, device=dev)
        _hmc_launch(g, tl, eng, z.clone(), gr.clone(), lj.clone(), 0, 1, _lib.new_state(dev), 13)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(T_plain):
            _hmc_launch(g, tl, eng, z, gr, lj, 1 if i else 0, 1, st, 13, samples=samp, nacc=nacc)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        sp_ = samp[T_plain // 2:, 0].double().cpu().numpy()
        plain[eng] = (wall, float(np.max(np.abs(sp_.mean(0) - m_true) / sd_true)))
    plain_eng = min(plain, key=lambda e: plain[e][0])
    plain_wall, err_plain = plain[plain_eng]
    # batched form: 4,096 chains, one launch per iteration, checkpoints
    Kmax = 512
    z, gr, lj, st, nacc = fresh(C, z0)
    samp = torch.zeros(Kmax, C, P, device=dev)
    zw, gw, ljw, stw = z.clone(), gr.clone(), lj.clone(), _lib.new_state(dev)
    _hmc_launch(g, tiles, "tc", zw, gw, ljw, 0, 1, stw, 14)
    torch.cuda.synchronize()
    marks, t_mark = [2 ** k for k in range(1, 10)], {}
    t0 = time.perf_counter()
    for i in range(Kmax):
        _hmc_launch(g, tiles, "tc", z, gr, lj, 1 if i else 0, 1, st, 14, samples=samp, nacc=nacc)
        if i + 1 in marks:
            torch.cuda.synchronize()
            t_mark[i + 1] = time.perf_counter() - t0
    errs = {}
    reached = None
    mt = torch.as_tensor(m_true, device=dev)
    sdt = torch.as_tensor(sd_true, device=dev)
    for k in marks:
        mk = samp[k // 2:k].double().mean(dim=(0, 1))
        errs[k] = float(((mk - mt).abs() / sdt).max().item())
        if reached is None and errs[k] <= err_plain:
            reached = k
    target = {
        "plain_method": f"one chain, one launch per iteration, {T_plain} iterations, mean over "
                        f"the second half; engine: {plain_eng} (the faster for one chain)",
        "plain_wall_s": plain_wall, "plain_mean_err_max_over_sd": err_plain,
        "plain_by_engine": {e: {"wall_s": w, "mean_err_max_over_sd": er}
                            for e, (w, er) in plain.items()},
        "batched_method": f"{C} chains, one tensor-core launch per iteration, mean over the "
                          f"second half of the iterations so far",
        "batched_mean_err_max_over_sd_at": {str(k): v for k, v in errs.items()},
        "batched_wall_s_at": {str(k): v for k, v in t_mark.items()},
        "batched_iterations_to_plain_error": reached,
        "batched_wall_s": t_mark.get(reached) if reached else None,
        "wall_time_ratio": (plain_wall / t_mark[reached]) if reached else None}
    return posterior, target


def read_traffic(engine):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (a line 'dram_bytes_per_launch: <int>'), else None."""
    name = "hmc_glm_tc_kernel_logreg_C4096.txt" if engine == "tc" else \
        "hmc_glm_kernel_logreg_C4096.txt"
    return read_traffic_file(name)


def read_traffic_file(name, key="dram_bytes_per_launch"):
    """The integer after '<key>:' in a committed ncu summary under profiles/, else None."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


def graph_of(fn):
    """fn captured into a CUDA graph (run once first, outside the capture)."""
    import torch
    fn()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    return g


def flush_timed(fn, k, dev):
    """Mean device time in ms of k calls of fn, each preceded by a 256 MB write
    that flushes L2; CUDA events on the launching stream bracket fn only."""
    import torch
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(k)]
    torch.cuda.synchronize()
    for i in range(k):
        flush.fill_(float(i))
        ev[i][0].record(st)
        fn()
        ev[i][1].record(st)
    torch.cuda.synchronize()
    del flush
    return sum(a.elapsed_time(b) for a, b in ev) / k


# ------------------------------------------------------------------ secondary workloads

def _peak_3xtf32():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
        src = "MEASURED_PEAKS.json bf16_tflops"
    except (OSError, KeyError, ValueError):
        bf16, src = 1900.0, "fallback 1.9 PFLOP/s bf16"
    return bf16 / 6.0, f"{src} {bf16:g} / 2 (TF32 rate) / 3 (3xTF32 passes), of measured"


def hier_data(I=2048, seed=0):
    """Ragged hierarchical logistic regressions: N_i log-uniform in [50, 20000],
    D_i uniform in {8..128}, X ~ N(0,1), w_i ~ N(mu_i, tau_i^2), mu_i ~ N(0,1),
    tau_i ~ HalfNormal(1), y ~ Bernoulli(sigmoid(X w_i))."""
    import numpy as np
    rng = np.random.default_rng(seed)
    Ns = np.exp(rng.uniform(np.log(50), np.log(20000), I)).astype(np.int64)
    Ds = rng.integers(8, 129, I)
    Xs, ys = [], []
    for N, D in zip(Ns, Ds):
        X = rng.standard_normal((N, D), dtype=np.float32)
        w = rng.standard_normal() + abs(rng.standard_normal()) * rng.standard_normal(D)
        eta = X @ w.astype(np.float32)
        y = (rng.random(N) < 1.0 / (1.0 + np.exp(-np.clip(eta, -60, 60)))).astype(np.float32)
        Xs.append(X)
        ys.append(y)
    return Xs, ys


def run_hier(args):
    """All 2,048 instances x 64 chains, 10 leapfrog steps per iteration, one
    launch per iteration, timed for both engines (edg_hmc_hier_tc_run: tcgen05
    3xTF32, 64 chains x 128 rows per tile; edg_hmc_hier_run: SIMT in two tile
    shapes, 32 chains x 64 rows and 16 chains x 128 rows) and both launch forms
    (the persistent work-queue grid and one CTA per (instance, chain tile));
    the fastest form is then replayed from a CUDA graph, which is the value."""
    import ctypes
    import numpy as np
    import torch
    from edward_gb300 import _lib
    from edward_gb300.ops import HierDevice
    C, L = 64, 10
    Xs, ys = hier_data(I=args.hier_instances)
    hd = HierDevice(Xs, ys)
    dev = torch.device("cuda")
    n = hd.I * C
    z = torch.zeros(n, hd.SP, device=dev)
    g = torch.zeros_like(z)
    lj = torch.zeros(n, dtype=torch.float64, device=dev)
    nacc = torch.zeros(n, dtype=torch.int32, device=dev)
    st = _lib.new_state(dev)
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed = 0.01, L, 1
    state = {"cache": 0, "fn": "edg_hmc_hier_run"}

    def step():
        lead = (_lib.ptr(hd.order),)
        if state["fn"] == "edg_hmc_hier_tc_run":
            tiles, toff = hd.tc_tiles()
            lead = lead + (_lib.ptr(tiles), _lib.ptr(toff))
        _lib.call(state["fn"], hd.ref(), ctypes.byref(cfg), C, 1, *lead,
                  _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), state["cache"], _lib.ptr(nacc),
                  _lib.ptr(st), None, 0, None, None, None, None, _lib.stream_ptr())
        state["cache"] = 1

    def timed(fn, k):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(k):
            fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / k

    forms, shape = {}, {}
    tc_ok = hd.max_D <= 128
    for engine in (("tc", "simt") if tc_ok else ("simt",)):
        for launch, lname in ((0, "persistent"), (1, "one_cta_per_item")):
            for ct in ((64,) if engine == "tc" else (32, 16)):
                rows = 128 if engine == "tc" else 2048 // ct
                name = f"{engine}_{lname}_{ct}x{rows}"
                cfg.launch, cfg.chains_per_block = launch, (ct if engine == "simt" else 0)
                state["fn"] = "edg_hmc_hier_tc_run" if engine == "tc" else "edg_hmc_hier_run"
                for _ in range(args.warmup):
                    step()
                torch.cuda.synchronize()
                forms[name] = timed(step, args.steps)
                shape[name] = (engine, launch, ct)
    best = min(forms, key=forms.get)
    engine, cfg.launch, ct = shape[best]
    cfg.chains_per_block = ct if engine == "simt" else 0
    state["fn"] = "edg_hmc_hier_tc_run" if engine == "tc" else "edg_hmc_hier_run"
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            step()
    torch.cuda.current_stream().wait_stream(s)
    graph.replay()
    torch.cuda.synchronize()
    nacc.zero_()
    with ClockSampler(0) as clk:
        ms = timed(graph.replay, args.steps)
    work = float((hd.Ns.astype(np.int64) * hd.Ds).sum())
    x_passes = 1 if engine == "tc" else C // ct   # X streams per gradient evaluation
    flops = 4.0 * work * C * L
    peak, src = tensor_peak(measure_tf32_peak(torch.device("cuda")))
    ach = flops / (ms / 1e3) / 1e12
    line = {"metric": "HMC leapfrog chain-steps/s (%d ragged hierarchical logistic regressions)" % hd.I,
            "value": n * L / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"hier_ragged_I{hd.I}_C64_L10", "instances": hd.I, "chains": C,
                       "leapfrog_steps": L, "sum_N_D": int(work),
                       "x_bytes": int(work * 4), "launch": f"{best}, replayed from a CUDA graph",
                       "l2_flush": "inputs larger than L2 (X is %.2f GB)" % (work * 4 / 1e9)},
            "launch_forms_ms_per_step": forms,
            "gpu_launches": args.steps,
            "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                         "frac": ach / peak,
                         "traffic": read_traffic_file(
                             "hmc_hier_tc_kernel_ragged_I2048.txt" if engine == "tc"
                             else "hmc_hier_kernel_ragged_I2048.txt") if hd.I == 2048 else None,
                         "kernel": ("hmc_hier_tc_kernel (tcgen05 3xTF32, 64 chains x 128 rows)"
                                    if engine == "tc" else
                                    "hmc_hier_kernel<%d> (SIMT FP32)" % ct),
                         "peak_source": src, "algorithmic_flops_per_launch": flops,
                         "x_stream_GBs": x_passes * L * work * 4 / (ms / 1e3) / 1e9},
            "engine": engine,
            "cpu_baseline": None if args.no_cpu_baseline else cpu_hier_baseline(
                Xs, ys, C, L, budget_s=args.cpu_budget),
            "accept_rate": float(nacc.sum().item()) / (n * args.steps),
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_klqp(args):
    """KLqp (analytic KL, S = 5) on the 10,000 x 50 logistic regression; one
    fused launch per ELBO-gradient step + Adam apply, replayed from a CUDA graph."""
    import numpy as np
    import torch
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Normal
    X, y, _ = make_data()
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    inf = ed.KLqp([w, b], data={yv: y})
    inf.initialize(n_samples=5, n_iter=100000, n_print=0)
    for _ in range(max(args.warmup, 3)):
        inf._step(apply=True)
    K = args.steps
    ms = flush_timed(lambda: inf._step(apply=True), K, torch.device("cuda"))
    # the same steps back to back from a CUDA graph (X stays L2-resident)
    inf.steps(50)
    torch.cuda.synchronize()
    a, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(4):
        inf.steps(50)
    b2.record()
    b2.synchronize()
    ms_graph = a.elapsed_time(b2) / 200
    st = inf._read_state()
    line = {"metric": "KLqp ELBO-grad evals/s (Bayesian logistic regression, S=5)",
            "value": 1e3 / ms, "unit": "evals/s", "n_gpus": 1, "steps": K,
            "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "klqp_logreg_N10000_D50_S5", "launch": "one fused launch per step",
                       "l2_flush": "256 MB write before each timed step, outside the events"},
            "value_graph_l2_resident": 1e3 / ms_graph,
            "gpu_launches": K, "final_loss": float(st.loss), "t": int(st.t)}
    print(json.dumps(line), flush=True)
    return 0


def bnn_data(N=100000, D=32, H1=256, H2=256, seed=0):
    """X ~ N(0,1) [N, D]; y = a random 32-256-256-1 tanh network (weights
    N(0,1)/sqrt(fan_in)) + N(0, 0.1^2) noise."""
    import numpy as np
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, D), dtype=np.float32)
    W0 = (rng.standard_normal((D, H1)) / np.sqrt(D)).astype(np.float32)
    W1 = (rng.standard_normal((H1, H2)) / np.sqrt(H1)).astype(np.float32)
    W2 = (rng.standard_normal((H2, 1)) / np.sqrt(H2)).astype(np.float32)
    y = (np.tanh(np.tanh(X @ W0) @ W1) @ W2)[:, 0]
    return X, (y + 0.1 * rng.standard_normal(N)).astype(np.float32)


def run_bnn(args):
    """Bayesian NN 32-256-256-1 under KLqp (analytic KL), S = 64 weight samples,
    minibatch M = 4,096 rows gathered on the device from N = 100,000 with
    scale N / M, through ed.KLqp; steps replayed from a CUDA graph."""
    import numpy as np
    import torch
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    N, D, H1, H2, M, S = 100000, 32, 256, 256, 4096, 64
    cb = None if args.no_cpu_baseline else cpu_net_baseline(
        "bnn", 3, "the Bayesian NN KLqp step (S=64 network copies over M=4096 rows, analytic "
        "KL, Adam)")
    X, y = bnn_data(N, D, H1, H2)
    W0 = Normal(loc=ed.zeros([D, H1]), scale=ed.ones([D, H1]))
    W1 = Normal(loc=ed.zeros([H1, H2]), scale=ed.ones([H1, H2]))
    W2 = Normal(loc=ed.zeros([H2, 1]), scale=ed.ones([H2, 1]))
    b0, b1, b2 = (Normal(loc=ed.zeros(n), scale=ed.ones(n)) for n in (H1, H2, 1))
    h = ed.tanh(ed.matmul(X, W0) + b0)
    h = ed.tanh(ed.matmul(h, W1) + b1)
    yv = Normal(loc=ed.reshape(ed.matmul(h, W2) + b2, [-1]), scale=0.1)
    rng = np.random.default_rng(1)
    qs = {}
    for z in (W0, b0, W1, b1, W2, b2):
        qs[z] = Normal(loc=ed.Variable(rng.standard_normal(z.shape).astype(np.float32) * 0.1),
                       scale=ed.softplus(ed.Variable(np.full(z.shape, -3.0, np.float32))))
    inf = ed.KLqp(qs, data={yv: y})
    inf.initialize(n_samples=S, n_minibatch=M, n_iter=5000, n_print=0,
                   optimizer=ed.train.AdamOptimizer(1e-3))
    chunk = 10
    for _ in range(max(1, args.warmup // chunk + 1)):
        inf.steps(chunk)
    torch.cuda.synchronize()
    K = max(args.steps // chunk, 1) * chunk
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        a.record()
        for _ in range(K // chunk):
            inf.steps(chunk)
        b.record()
        b.synchronize()
    ms = a.elapsed_time(b) / K
    st = inf._read_state()
    P = inf._spec.P
    fwd = 2.0 * (D * H1 + H1 * H2 + H2) * M * S
    flops = 3.0 * fwd
    peak, src = tensor_peak(measure_tf32_peak(torch.device("cuda")))
    ach = flops / (ms / 1e3) / 1e12
    act_bytes = 4.0 * S * M * (H1 + H2)
    line = {"metric": "KLqp ELBO-grad evals/s (Bayesian NN 32-256-256-1, S=64, M=4096)",
            "value": 1e3 / ms, "unit": "evals/s", "n_gpus": 1, "steps": K,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "bnn_klqp_N100000_D32_H256_H256_S64_M4096", "params": P,
                       "launch": f"CUDA graph of {chunk} steps (gather + 13 launches each)",
                       "l2_flush": "inputs larger than L2 (activations %.0f MB per step)"
                                   % (act_bytes / 1e6)},
            "gpu_launches": K * 14,
            "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                         "frac": ach / peak,
                         "traffic": read_traffic_file("gemm_tc_kernel_bnn_S64_M4096.txt",
                                                      "dram_bytes_per_step"),
                         "kernel": "whole step (tcgen05 3xTF32 GEMMs + fused head/adjoint + finalize)",
                         "peak_source": src, "algorithmic_flops_per_step": flops},
            "final_loss": float(st.loss), "t": int(st.t), "clocks": clk.summary(),
            "cpu_baseline": cb}
    print(json.dumps(line), flush=True)
    return 0


def sbn_data(N=60000, V=784, H0=200, H1=200, seed=0):
    """Binary rows [N, V] (uint8) from a random sigmoid belief network
    H1 -> H0 -> V with W ~ N(0, 1) / sqrt(fan_in), zero biases, z1 ~ Bern(1/2)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((H1, H0)) / np.sqrt(H1)
    W0 = rng.standard_normal((H0, V)) / np.sqrt(H0)
    z1 = (rng.random((N, H1)) < 0.5).astype(np.float32)
    z0 = (rng.random((N, H0)) < 1.0 / (1.0 + np.exp(-(z1 @ W1)))).astype(np.float32)
    return (rng.random((N, V)) < 1.0 / (1.0 + np.exp(-(z0 @ W0)))).astype(np.uint8)


def _sbn_inference(data, B, S, baseline, seed=0):
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli
    ed.set_seed(seed)
    V, H0, H1 = data.shape[1], 200, 200
    x_ph = ed.placeholder(shape=[B, V])
    z1 = Bernoulli(logits=ed.zeros([B, H1]))
    z0 = Bernoulli(logits=ed.layers.dense(ed.cast(z1), H0))
    x = Bernoulli(logits=ed.layers.dense(ed.cast(z0), V))
    qz0 = Bernoulli(logits=ed.layers.dense(ed.cast(x_ph), H0))
    qz1 = Bernoulli(logits=ed.layers.dense(ed.cast(qz0), H1))
    inf = ed.ScoreKLqp({z0: qz0, z1: qz1}, data={x: data})
    inf.initialize(n_samples=S, n_minibatch=B, baseline=baseline, baseline_hidden=100,
                   n_print=0, optimizer=ed.train.AdamOptimizer(1e-3))
    return inf


def run_sbn(args):
    """Sigmoid belief network 784-200-200 under ScoreKLqp with the learned MLP
    baseline (784 -> 100 -> 1, trained online by its own kernels): S = 16
    samples, B = 1,024 rows gathered on the device per step from 60,000
    synthetic binary rows; steps replayed from a CUDA graph.  Also reports
    the q-gradient variance under each baseline at the trained parameters and
    the ELBO reached by the running-mean and MLP baselines with equal steps."""
    import numpy as np
    import torch
    V, H0, H1, B, S, BH = 784, 200, 200, 1024, 16, 100
    cb = None if args.no_cpu_baseline else cpu_net_baseline(
        "sbn", 5, "the plain ScoreKLqp step (S=16 copies of q and p over B=1024 rows, Adam)")
    data = sbn_data(V=V, H0=H0, H1=H1)
    inf = _sbn_inference(data, B, S, "mlp")
    chunk = 10
    for _ in range(max(1, args.warmup // chunk + 1)):
        inf.steps(chunk)
    torch.cuda.synchronize()
    K = args.steps
    # one step per CUDA graph replay, L2 flushed before each (the step's own
    # buffers, 117 MB, would otherwise stay in the 129 MB L2)
    one = graph_of(lambda: inf._step(apply=True))
    with ClockSampler(0) as clk:
        ms = flush_timed(one.replay, K, torch.device("cuda"))
    R = S * B
    flops = 4.0 * R * ((H0 + 1) * H1 + (H1 + 1) * H0 + (H0 + 1) * V) + \
        4.0 * B * (V + 1) * (H0 + BH)
    peak, src = tensor_peak(measure_tf32_peak(torch.device("cuda")))
    ach = flops / (ms / 1e3) / 1e12
    nq = (V + 1) * H0 + (H0 + 1) * H1

    def q_grad_variance(run, modes, draws=24):
        """Summed variance of the q-gradient over `draws` Philox draws at the
        run's current parameters and one frozen minibatch, per estimator."""
        run._sbn.gather = False
        out = {}
        for mode, rb, name in modes:
            run._cfg.baseline, run._cfg.rao_blackwell = mode, rb
            gs = []
            for k in range(draws):
                run.seed = 7000 + k
                gs.append(run.score_gradients()[1][:nq].double())
            out[name] = float(torch.stack(gs).var(dim=0).sum())
        run._cfg.baseline, run._cfg.rao_blackwell = 2, 0
        run._sbn.gather = True
        return out

    def train(run, n):
        """n steps; returns the ELBO per row (mean of the last 10 chunk-end losses)."""
        losses = []
        for i in range(n // chunk):
            run.steps(chunk)
            if i >= n // chunk - 10:
                losses.append(run._read_state().loss)
        return -float(np.mean(losses)) / B

    def ci95(xs):
        xs = np.asarray(xs, np.float64)
        t = {2: 12.71, 3: 4.30, 4: 3.18, 5: 2.78, 6: 2.57, 7: 2.45, 8: 2.36}.get(len(xs), 2.0)
        return [float(xs.mean() - t * xs.std(ddof=1) / np.sqrt(len(xs))),
                float(xs.mean() + t * xs.std(ddof=1) / np.sqrt(len(xs)))]
    # all four estimators at the trained parameters of the timed run
    gvar = q_grad_variance(inf, ((0, 0, "none"), (0, 1, "rao_blackwell"), (1, 0, "mean"),
                                 (2, 0, "mlp")))
    # learned baseline against the running mean over independent seeds: each seed
    # trains an MLP-baseline run and a running-mean run for the same steps, then
    # measures both estimators' q-gradient variance at the MLP run's parameters
    n_cmp = args.sbn_compare_steps
    seeds = []
    for sd in range(args.sbn_seeds):
        run_mlp = _sbn_inference(data, B, S, "mlp", seed=100 + sd)
        e_mlp = train(run_mlp, n_cmp)
        v = q_grad_variance(run_mlp, ((1, 0, "mean"), (2, 0, "mlp")))
        run_mean = _sbn_inference(data, B, S, "mean", seed=100 + sd)
        e_mean = train(run_mean, n_cmp)
        seeds.append({"seed": 100 + sd, "q_grad_var_mean": v["mean"], "q_grad_var_mlp": v["mlp"],
                      "variance_ratio_mlp_over_mean": v["mlp"] / v["mean"],
                      "elbo_per_row_mean": e_mean, "elbo_per_row_mlp": e_mlp})
        del run_mlp, run_mean
    ratios = [r["variance_ratio_mlp_over_mean"] for r in seeds]
    gains = [r["elbo_per_row_mlp"] - r["elbo_per_row_mean"] for r in seeds]
    baseline_gain = {
        "seeds": seeds, "steps_per_run": n_cmp,
        "variance_ratio_mlp_over_mean_mean": float(np.mean(ratios)),
        "variance_ratio_mlp_over_mean_ci95": ci95(ratios) if len(ratios) > 1 else None,
        "elbo_gain_per_row_mean": float(np.mean(gains)),
        "elbo_gain_per_row_ci95": ci95(gains) if len(gains) > 1 else None}
    # spec target for the learned part: wall time for the learned-baseline
    # run to come within 0.1 nat/row of the ELBO that the plain estimator (the
    # reference's ScoreKLqp, no baseline) reaches in n_cmp steps
    plain = _sbn_inference(data, B, S, "none", seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_plain = train(plain, n_cmp)
    plain_wall = time.perf_counter() - t0
    del plain
    learned = _sbn_inference(data, B, S, "mlp", seed=1)
    learned.steps(chunk)
    torch.cuda.synchronize()
    recent, steps, reached = [], chunk, None
    t0 = time.perf_counter()
    while steps < n_cmp:
        learned.steps(chunk)
        steps += chunk
        recent.append(learned._read_state().loss)
        if len(recent) >= 10 and -float(np.mean(recent[-10:])) / B >= e_plain - 0.1:
            reached = time.perf_counter() - t0
            break
    target = {"plain_method": f"ScoreKLqp without a baseline (the reference estimator), "
                              f"{n_cmp} steps", "plain_wall_s": plain_wall,
              "plain_elbo_per_row": e_plain, "learned_steps_to_within_0.1_nat": steps
              if reached is not None else None, "learned_wall_s": reached,
              "wall_time_ratio": plain_wall / reached if reached else None}
    st = inf._read_state()
    from edward_gb300 import _lib
    launches = _lib.load().edg_sbn_launches_per_step(inf._cfg, B, 1)
    line = {"metric": "ScoreKLqp ELBO-grad evals/s (sigmoid belief network 784-200-200, S=16, "
                      "B=1024, learned MLP baseline)",
            "value": 1e3 / ms, "unit": "evals/s", "n_gpus": 1, "steps": K,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "sbn_score_V784_H200_H200_S16_B1024_mlp100",
                       "params": inf._P, "baseline_params": int(inf._bparams.numel()),
                       "launch": "one CUDA graph replay per step",
                       "l2_flush": "256 MB write before each timed step, outside the events"},
            "gpu_launches": K * (1 + launches),
            "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                         "frac": ach / peak,
                         "traffic": read_traffic_file("sbn_score_step_B1024_S16.txt",
                                                      "dram_bytes_per_step"),
                         "kernel": "whole step (tcgen05 3xTF32 GEMMs, row kernels, baseline MLP)",
                         "peak_source": src, "algorithmic_flops_per_step": flops},
            "q_grad_variance": gvar, "learned_baseline_gain": baseline_gain,
            "target": target, "cpu_baseline": cb,
            "final_loss": float(st.loss), "t": int(st.t), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_sgld(args):
    """SGLD (edward/inferences/sgld.py) on the 10,000 x 50 logistic regression with
    4,096 chains.  Tensor-core engine: one launch per call of run_iterations,
    each iteration one 3xTF32 gradient evaluation with the update fused in;
    SIMT engine: a batched log-joint gradient + update kernel per iteration."""
    import numpy as np
    import torch
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, Normal
    X, y, _ = make_data()
    C = 4096
    K = 10   # iterations per launch for the multi-iteration figure
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    T = args.steps * (K + 1) + 2 * args.warmup + 4
    qw = Empirical(ed.Variable(np.zeros((T, C, N_FEAT), np.float32)), n_chains=C)
    qb = Empirical(ed.Variable(np.zeros((T, C), np.float32)), n_chains=C)
    inf = ed.SGLD({w: qw, b: qb}, data={yv: y}, n_chains=C)
    inf.initialize(step_size=1e-4, n_print=0, engine=args.engine)
    inf.run_iterations(args.warmup)
    torch.cuda.synchronize()
    dev = torch.device("cuda")
    with ClockSampler(0) as clk:
        ms = flush_timed(lambda: inf.run_iterations(1), args.steps, dev)
        inf.run_iterations(args.warmup * K)
        ms_k = flush_timed(lambda: inf.run_iterations(K), args.steps, dev) / K
    P = N_FEAT + 1
    flops = 4.0 * N_ROWS * P * C
    tc = inf.engine == "tc"
    if tc:
        peak, src = tensor_peak(None if args.no_extras else measure_tf32_peak(dev))
        kern = "hmc_glm_tc_kernel<SG> (tcgen05 3xTF32, the SGLD update fused in)"
        launches = args.steps
    else:
        peak, src = None, None
        kern = "glm_partial_kernel + glm_reduce_kernel + sgmcmc update (SIMT)"
        launches = 3 * args.steps
    ach = flops / (ms / 1e3) / 1e12
    line = {"metric": "SGLD chain-iterations/s (Bayesian logistic regression, batched chains)",
            "value": C / (ms / 1e3), "unit": "chain-iterations/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "engine": inf.engine,
            "cpu_baseline": None if args.no_cpu_baseline else cpu_mc_baseline(
                "sgld", args.cpu_budget),
            "config": {"workload": "sgld_logreg_N10000_D50_C4096", "chains": C,
                       "l2_flush": "256 MB write before each timed launch, outside the events"},
            "multi_iteration": {"iterations_per_launch": K, "ms_per_iteration": ms_k,
                                "value": C / (ms_k / 1e3)},
            "gpu_launches": launches,
            "roofline": {"bound": "tensor" if tc else "fp32", "achieved": ach,
                         "unit": "TFLOP/s",
                         "traffic": read_traffic_file(
                             "hmc_glm_tc_kernel_sgmcmc_mh_logreg_C4096.txt") if tc else None,
                         "peak": peak,
                         "frac": ach / peak if peak else None, "peak_source": src,
                         "kernel": kern, "algorithmic_flops_per_step": flops},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_mh(args):
    """MetropolisHastings (edward/inferences/metropolis_hastings.py) with Normal
    random-walk proposals (scale 0.01) on the 10,000 x 50 logistic regression
    with 4,096 chains.  Tensor-core engine: one launch per call of
    run_iterations, each iteration the proposal, one 3xTF32 log-joint
    evaluation (its gradient included) and the FP64 test; SIMT engine: propose,
    batched log joint and accept kernels per iteration."""
    import numpy as np
    import torch
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, Normal
    X, y, _ = make_data()
    C = 4096
    K = 10
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    T = args.steps * (K + 1) + 2 * args.warmup + 4
    qw = Empirical(ed.Variable(np.zeros((T, C, N_FEAT), np.float32)), n_chains=C)
    qb = Empirical(ed.Variable(np.zeros((T, C), np.float32)), n_chains=C)
    props = {w: Normal(loc=w, scale=0.01 * ed.ones(N_FEAT)), b: Normal(loc=b, scale=0.01)}
    inf = ed.MetropolisHastings({w: qw, b: qb}, props, data={yv: y}, n_chains=C)
    inf.initialize(n_print=0, engine=args.engine)
    inf.run_iterations(args.warmup)
    torch.cuda.synchronize()
    dev = torch.device("cuda")
    with ClockSampler(0) as clk:
        ms = flush_timed(lambda: inf.run_iterations(1), args.steps, dev)
        inf.run_iterations(args.warmup * K)
        ms_k = flush_timed(lambda: inf.run_iterations(K), args.steps, dev) / K
    P = N_FEAT + 1
    tc = inf.engine == "tc"
    flops = (4.0 if tc else 2.0) * N_ROWS * P * C  # executed: the tensor-core form adds the adjoint
    alg = 2.0 * N_ROWS * P * C                    # algorithmic: the log joint alone
    if tc:
        peak, src = tensor_peak(None if args.no_extras else measure_tf32_peak(dev))
        kern = "hmc_glm_tc_kernel<2> (tcgen05 3xTF32, proposal and FP64 test fused in)"
        launches = args.steps
    else:
        peak, src = None, None
        kern = "mh propose + glm_partial_kernel + glm_reduce_kernel + mh accept (SIMT)"
        launches = 4 * args.steps
    ach = alg / (ms / 1e3) / 1e12
    line = {"metric": "Metropolis-Hastings chain-iterations/s (Bayesian logistic regression, "
                      "batched chains)",
            "value": C / (ms / 1e3), "unit": "chain-iterations/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "engine": inf.engine,
            "cpu_baseline": None if args.no_cpu_baseline else cpu_mc_baseline(
                "mh", args.cpu_budget),
            "config": {"workload": "mh_logreg_N10000_D50_C4096_walk0.01", "chains": C,
                       "l2_flush": "256 MB write before each timed launch, outside the events"},
            "multi_iteration": {"iterations_per_launch": K, "ms_per_iteration": ms_k,
                                "value": C / (ms_k / 1e3)},
            "accept_rate": float(inf.n_accept.sum().item()) / (C * max(inf.t, 1)),
            "gpu_launches": launches,
            "roofline": {"bound": "tensor" if tc else "fp32", "achieved": ach,
                         "unit": "TFLOP/s", "traffic": None, "peak": peak,
                         "frac": ach / peak if peak else None, "peak_source": src,
                         "kernel": kern, "algorithmic_flops_per_step": alg,
                         "executed_flops_per_step": flops},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ct", type=int, default=0, help="SIMT chains per block (0 = autotune)")
    ap.add_argument("--engine", default="auto", choices=["auto", "tc", "simt"])
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline HMC measurement only (no KLqp record, posterior error, "
                         "wall-time target or TF32 peak)")
    ap.add_argument("--klqp-steps", type=int, default=200)
    ap.add_argument("--long-chain-iters", type=int, default=10000)
    ap.add_argument("--hier-instances", type=int, default=2048)
    ap.add_argument("--sbn-compare-steps", type=int, default=1000)
    ap.add_argument("--sbn-seeds", type=int, default=5)
    ap.add_argument("--workload", default="hmc_logreg", choices=["hmc_logreg", "hier", "klqp", "bnn", "sbn", "sgld", "mh"],
                    help="hmc_logreg is the headline; the others are secondary measurements")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "hier":
        return run_hier(args)
    if args.workload == "klqp":
        return run_klqp(args)
    if args.workload == "bnn":
        return run_bnn(args)
    if args.workload == "sbn":
        return run_sbn(args)
    if args.workload == "sgld":
        return run_sgld(args)
    if args.workload == "mh":
        return run_mh(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
