"""Parity at the benchmark workloads themselves, with the error of every
result measured against the FP64 oracle and against the oracle's FP32 mode.

* HMC at exactly the 4,096-chain configuration: N = 10,000, D = 50 (+ bias),
  C = 4,096 chains, 10 leapfrog steps of 0.005; one iteration fed the
  oracle's momenta and uniforms, then iterations with in-kernel Philox draws;
  both engines.
* KLqp at the S = 5 configuration (N = 10,000, D = 50): loss and gradients
  of the three estimators for given draws and for in-kernel Philox draws,
  and the final ELBO of a 1,000-step run against the oracle's run.

The FP32 mode of the oracle computes the contraction X z, the per-row terms
and the adjoint in FP32 (as the reference's TF CPU path does) with FP64 sums
over rows; positions and momenta step in FP32 and the Metropolis ratio is
FP64, as in the kernels.

Tolerances (1e-5 relative throughout):
* vectors (positions, gradients, log joints): max |gpu - oracle| <= 1e-5 *
  max |oracle| over the compared array;
* scalars (KLqp loss): |gpu - oracle| <= 1e-5 * |oracle|;
* the log acceptance ratio is a difference of two log joints of ~10^3-10^4
  nats whose per-row terms are FP32 (in the kernels and in the reference),
  so its error is measured in nats and bounded by 1e-5 of the log-joint
  magnitude; accept decisions must agree wherever |log u - ratio| exceeds
  the measured ratio error.

Set EDG_PARITY_REPORT=<path> to write the measured errors as JSON.
"""
import ctypes
import json
import os

import numpy as np
import pytest
import torch

from oracle.glm import GLM
from oracle.hmc import glm_lj_grad, hmc_step
from oracle.klqp import REPARAM, REPARAM_KL, SCORE, klqp_glm_loss_and_grads, run_klqp_glm
from oracle.philox import KIND_EPS, KIND_MOMENTUM, KIND_UNIFORM, normals, uniforms64

pytestmark = pytest.mark.gpu
RTOL = 1e-5
N_ROWS, N_FEAT, N_CHAINS, N_LEAP, STEP = 10_000, 50, 4096, 10, 0.005
REPORT = {}


@pytest.fixture(scope="module", autouse=True)
def _report():
    yield
    path = os.environ.get("EDG_PARITY_REPORT")
    if path and REPORT:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


def _rel(a, b):
    """max |a - b| / max |b| over the array."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _data(seed=0):
    """The benchmark's synthetic logistic regression: X ~ N(0,1) fp32,
    w ~ N(0,1)^50, b ~ N(0,1), y ~ Bernoulli(sigmoid(Xw + b)); chains from
    N(0, 1)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N_ROWS, N_FEAT)).astype(np.float32)
    w = rng.standard_normal(N_FEAT)
    b = rng.standard_normal()
    p = 1.0 / (1.0 + np.exp(-(X.astype(np.float64) @ w + b)))
    y = (rng.random(N_ROWS) < p).astype(np.float32)
    z0 = rng.standard_normal((N_CHAINS, N_FEAT + 1)).astype(np.float32)
    return X, y, z0


@pytest.fixture(scope="module")
def workload(cuda):
    from edward_gb300.compile import GLMSpec
    from edward_gb300.ops import GLMDevice
    X, y, z0 = _data()
    P = N_FEAT + 1
    m = GLM(X, y, bias=True)
    spec = GLMSpec(X=X, y=y, bias=True, lik=0, lik_scale=1.0,
                   prior_loc=np.zeros(P, np.float32), prior_scale=np.ones(P, np.float32))
    return m, GLMDevice(spec, cuda), z0


def _tiles(dev, cuda):
    from edward_gb300 import _lib
    lib = _lib.load()
    nb = lib.edg_hmc_glm_tc_tiles_bytes(dev.ref())
    tiles = torch.empty(nb, dtype=torch.uint8, device=cuda)
    _lib.call("edg_hmc_glm_tc_prepare", dev.ref(), _lib.ptr(tiles), nb, _lib.stream_ptr())
    return tiles


def _lj_grad(m, dtype):
    """(log joint [B] FP64, gradient [B, P]) with the contraction, the
    per-row terms and the adjoint in `dtype` (one pass over X each way)."""
    def f(Z):
        Z = np.asarray(Z, np.float64)
        e = m.eta(Z, dtype)
        lp, r = m._terms(e)
        X = m.X.astype(dtype)
        g = np.concatenate([r.T @ X, r.sum(axis=0)[:, None]], axis=1)
        lj = m.log_prior(Z) + lp.sum(axis=0, dtype=np.float64)
        return lj, np.asarray(g, np.float64) + m.grad_log_prior(Z)
    return f


@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_hmc_exact_benchmark_config_parity(cuda, workload, engine):
    """The kernels run all 4,096 chains; the oracles follow every 7th chain
    (586 chains spread over every cluster and TMEM lane quarter; the chains
    are independent, so following a subset is exact)."""
    m, dev, z0 = workload
    C, P = N_CHAINS, N_FEAT + 1
    sub = np.unique(np.r_[np.arange(0, C, 7), C - 1])
    tiles = _tiles(dev, cuda) if engine == "tc" else None
    f64 = _lj_grad(m, np.float64)
    f32 = _lj_grad(m, np.float32)
    rec = {"config": f"N{N_ROWS} D{N_FEAT}+bias C{C} L{N_LEAP} eps{STEP}",
           "oracle_chains": int(sub.size), "iterations": []}
    seed = 123
    zc = z0[sub].astype(np.float64)
    lj64, g64 = f64(zc)
    lj32, g32 = f32(zc)
    z = torch.as_tensor(z0, device=cuda).clone()
    g = torch.zeros(C, P, device=cuda)
    lj = torch.zeros(C, dtype=torch.float64, device=cuda)
    cache = 0
    for it in range(3):
        given = it == 0
        r_all = normals(seed, KIND_MOMENTUM, it, C, P)
        u_all = uniforms64(seed, KIND_UNIFORM, it, C)
        if given:
            r_all = r_all.astype(np.float32)
        r0, u = r_all[sub], u_all[sub]
        ratio = torch.zeros(1, C, dtype=torch.float64, device=cuda)
        r_dev = torch.as_tensor(r_all[None], dtype=torch.float32, device=cuda).contiguous() \
            if given else None
        u_dev = torch.as_tensor(u_all[None], device=cuda).contiguous() if given else None
        nacc = _run_at(engine, dev, tiles, z, g, lj, cache, it, seed, r_dev, u_dev, ratio)
        cache = 1
        e64 = hmc_step(f64, zc, g64, lj64, r0, u, STEP, N_LEAP)
        e32 = hmc_step(f32, zc, g32, lj32, np.asarray(r0, np.float32), u, STEP, N_LEAP,
                       dtype=np.float32)
        kr = ratio.cpu().numpy()[0][sub]
        lj_scale = float(max(np.abs(lj64).max(), np.abs(e64["lj"]).max()))
        err_ratio64 = float(np.abs(kr - e64["ratio"]).max())
        err_ratio32 = float(np.abs(kr - e32["ratio"]).max())
        k_acc = nacc.cpu().numpy().astype(bool)[sub]
        differ = k_acc != e64["accept"]
        margin = np.abs(np.log(u) - e64["ratio"])
        assert np.all(margin[differ] <= max(err_ratio64, 1e-12)), (margin[differ], err_ratio64)
        same = ~differ
        zk, gk, ljk = z.cpu().numpy()[sub], g.cpu().numpy()[sub], lj.cpu().numpy()[sub]
        row = {"iteration": it, "draws": "oracle momenta/uniforms" if given else "in-kernel Philox",
               "accept_rate": float(k_acc.mean()), "decisions_differing": int(differ.sum()),
               "ratio_abs_err_nats_fp64": err_ratio64, "ratio_abs_err_nats_fp32": err_ratio32,
               "log_joint_magnitude": lj_scale,
               "ratio_err_rel_to_log_joint_fp64": err_ratio64 / lj_scale,
               "position_rel_err_fp64": _rel(zk[same], e64["z"][same]),
               "position_rel_err_fp32": _rel(zk[same], e32["z"][same]),
               "gradient_rel_err_fp64": _rel(gk[same], e64["g"][same]),
               "gradient_rel_err_fp32": _rel(gk[same], e32["g"][same]),
               "log_joint_rel_err_fp64": _rel(ljk[same], e64["lj"][same]),
               "log_joint_rel_err_fp32": _rel(ljk[same], e32["lj"][same]),
               "fp32_oracle_position_rel_err_vs_fp64": _rel(e32["z"], e64["z"])}
        rec["iterations"].append(row)
        for k in ("position_rel_err_fp64", "position_rel_err_fp32", "gradient_rel_err_fp64",
                  "gradient_rel_err_fp32", "log_joint_rel_err_fp64", "log_joint_rel_err_fp32",
                  "ratio_err_rel_to_log_joint_fp64"):
            assert row[k] <= RTOL, (k, row[k])
        # resynchronise both oracles on the kernel's kept states
        zc = zk.astype(np.float64)
        lj64, g64 = f64(zc)
        lj32, g32 = f32(zc)
    REPORT[f"hmc_{engine}"] = rec


def _run_at(engine, dev, tiles, z, g, lj, cache, it, seed, r, u, ratio):
    """One iteration whose Philox counters use iteration index `it` (the
    state record's t starts at it)."""
    from edward_gb300 import _lib
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed = STEP, N_LEAP, seed
    C = z.shape[0]
    st = _lib.new_state(z.device, t=it)
    nacc = torch.zeros(C, dtype=torch.int32, device=z.device)
    if engine == "tc":
        _lib.call("edg_hmc_glm_tc_run", dev.ref(), ctypes.byref(cfg), C, 1, _lib.ptr(tiles),
                  _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), cache, _lib.ptr(nacc), _lib.ptr(st),
                  None, 0, None, _lib.ptr(r), _lib.ptr(u), _lib.ptr(ratio), _lib.stream_ptr())
    else:
        cfg.chains_per_block = 32
        _lib.call("edg_hmc_glm_run", dev.ref(), ctypes.byref(cfg), C, 1, _lib.ptr(z),
                  _lib.ptr(g), _lib.ptr(lj), cache, _lib.ptr(nacc), _lib.ptr(st), None, 0, None,
                  _lib.ptr(r), _lib.ptr(u), _lib.ptr(ratio), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert _lib.read_state(st).error == 0, "a kernel gave up a bounded wait"
    return nacc


def test_glm_logjoint_grad_exact_benchmark_shape(cuda, workload):
    """The batched log joint and adjoint for all 4,096 chain states."""
    from edward_gb300.ops import glm_logjoint_grad
    m, dev, z0 = workload
    lp, g = glm_logjoint_grad(dev, torch.as_tensor(z0, device=cuda))
    lp, g = lp.cpu().numpy(), g.cpu().numpy()
    rec = {"log_joint_rel_err_fp64": _rel(lp, m.log_joint(z0)),
           "log_joint_rel_err_fp32": _rel(lp, m.log_joint(z0, dtype=np.float32)),
           "gradient_rel_err_fp64": _rel(g, m.grad_log_joint(z0)),
           "gradient_rel_err_fp32": _rel(g, m.grad_log_joint(z0, dtype=np.float32))}
    REPORT["glm_logjoint_grad_C4096"] = rec
    for k, v in rec.items():
        assert v <= RTOL, (k, v)


def _klqp_inference(m, n_samples=5, n_iter=1000):
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Normal
    X = m.X.astype(np.float32)
    w = Normal(loc=ed.zeros(N_FEAT), scale=ed.ones(N_FEAT))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    inf = ed.KLqp([w, b], data={yv: m.y.astype(np.float32)})
    inf.initialize(n_samples=n_samples, n_iter=n_iter, n_print=0)
    return inf


@pytest.mark.parametrize("method", [REPARAM_KL, REPARAM, SCORE])
def test_klqp_benchmark_config_parity(cuda, workload, method):
    m = workload[0]
    inf = _klqp_inference(m)
    inf._cfg.method = method
    P = N_FEAT + 1
    rng = np.random.default_rng(method)
    mu = (rng.standard_normal(P) * 0.3).astype(np.float32)
    rho = (rng.standard_normal(P) * 0.3 - 1).astype(np.float32)
    inf._mu.copy_(torch.as_tensor(mu))
    inf._rho.copy_(torch.as_tensor(rho))
    rec = {}
    for draws in ("given", "philox"):
        if draws == "given":
            eps = rng.standard_normal((5, P)).astype(np.float32)
            loss, gmu, grho = inf.loss_and_gradients(eps)
        else:
            eps = normals(inf.seed, KIND_EPS, 0, 5, P)
            loss, gmu, grho = inf.loss_and_gradients(None)
        gmu, grho = gmu.cpu().numpy(), grho.cpu().numpy()
        l64, gm64, gr64, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, method)
        l32, gm32, gr32, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, method, dtype=np.float32)
        r = {"loss_rel_err_fp64": abs(loss - l64) / abs(l64),
             "loss_rel_err_fp32": abs(loss - l32) / abs(l32),
             "grad_mu_rel_err_fp64": _rel(gmu, gm64), "grad_mu_rel_err_fp32": _rel(gmu, gm32),
             "grad_rho_rel_err_fp64": _rel(grho, gr64), "grad_rho_rel_err_fp32": _rel(grho, gr32)}
        rec[draws] = r
        for k, v in r.items():
            assert v <= RTOL, (draws, k, v)
    REPORT[f"klqp_S5_method{method}"] = rec


def test_klqp_1000_step_run_final_elbo(cuda, workload):
    """1,000 fused steps (analytic KL, S = 5, default Adam with the staircase
    learning rate 0.1 * 0.9^(t/100)) end at the oracle's final ELBO: the mean
    of the last 100 losses per datum within 1e-4 nats, and the final q
    parameters within 1e-3 relative."""
    m = workload[0]
    inf = _klqp_inference(m)
    P = N_FEAT + 1
    mu0 = inf._mu.cpu().numpy().astype(np.float64)
    rho0 = inf._rho.cpu().numpy().astype(np.float64)
    losses = []
    for _ in range(1000):
        inf._step(apply=True)
        losses.append(float(inf._read_state().loss))
    losses = np.array(losses)
    mu_k, rho_k = inf._mu.cpu().numpy(), inf._rho.cpu().numpy()
    e_mu, e_rho, e_losses = run_klqp_glm(m, mu0, rho0, 1000, 5, seed=inf.seed)
    elbo_k = -losses[-100:].mean() / N_ROWS
    elbo_o = -e_losses[-100:].mean() / N_ROWS
    rec = {"final_elbo_per_datum_gpu": elbo_k, "final_elbo_per_datum_oracle": elbo_o,
           "elbo_per_datum_abs_err": abs(elbo_k - elbo_o),
           "final_mu_rel_err": _rel(mu_k, e_mu), "final_rho_rel_err": _rel(rho_k, e_rho),
           "first_loss_rel_err": abs(losses[0] - e_losses[0]) / abs(e_losses[0])}
    REPORT["klqp_S5_1000_steps"] = rec
    assert rec["elbo_per_datum_abs_err"] < 1e-4, rec
    assert rec["final_mu_rel_err"] < 1e-3 and rec["final_rho_rel_err"] < 1e-3, rec
    assert inf.t == 1000
