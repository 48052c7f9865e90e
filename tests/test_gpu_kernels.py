"""GPU parity of the CUDA kernels against the oracle, through the C ABI.

Tolerance: 1e-5 relative to the FP64 oracle (scaled by the largest
magnitude of the compared vector); bit-exact for Philox integer streams."""
import ctypes
import os

import numpy as np
import pytest
import torch

from oracle.glm import GLM, NORMAL, synthetic_logreg
from oracle.hmc import glm_lj_grad, hmc_step
from oracle.klqp import REPARAM, REPARAM_KL, SCORE, TFAdam, default_learning_rate, \
    klqp_glm_loss_and_grads
from oracle.philox import raw_u32, normals, uniforms64

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")
RTOL = 1e-5


def close(a, b, rtol=RTOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * scale)


def glm_device(m, cuda):
    from edward_gb300.compile import GLMSpec
    from edward_gb300.ops import GLMDevice
    spec = GLMSpec(X=m.X.astype(np.float32), y=m.y.astype(np.float32), bias=m.bias, lik=m.lik,
                   lik_scale=m.lik_scale, prior_loc=m.prior_loc.astype(np.float32),
                   prior_scale=m.prior_scale.astype(np.float32))
    return GLMDevice(spec, cuda)


def f32(m):
    """Oracle model on the FP32-rounded data the GPU sees."""
    return GLM(m.X.astype(np.float32), m.y.astype(np.float32), bias=m.bias, lik=m.lik,
               lik_scale=m.lik_scale, prior_loc=m.prior_loc.astype(np.float32),
               prior_scale=m.prior_scale.astype(np.float32), data_scale=m.data_scale)


# ----------------------------------------------------------------- Philox

def test_philox_streams_bit_exact(cuda):
    from edward_gb300 import ops
    g = np.load(GOLD)
    seed = 0x0123456789ABCDEF
    u = ops.philox_u32(seed, 1, 7, 5, 10).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(u, g["philox_u32"])
    n = ops.philox_normal(seed, 1, 7, 5, 10).cpu().numpy()
    np.testing.assert_allclose(n, g["philox_normal"], rtol=2e-6, atol=2e-6)
    u64 = ops.philox_uniform64(seed, 2, 7, 5).cpu().numpy()
    np.testing.assert_array_equal(u64, g["philox_uniform64"])
    big = ops.philox_u32(12345, 3, 99, 300, 129).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(big, raw_u32(12345, 3, 99, 300, 129))


# ----------------------------------------------------------------- GLM log joint

CASES = [
    # (N, D, bias, lik, B)
    (37, 5, True, 0, 3),        # ragged tiny
    (1000, 50, True, 0, 5),     # logistic regression, S = 5
    (10000, 50, True, 0, 70),   # several vector tiles and row chunks
    (50, 1, False, 1, 4),       # Normal-Normal
    (513, 130, True, 1, 17),    # wide, Normal likelihood
    (4099, 7, False, 0, 33),
]


@pytest.mark.parametrize("N,D,bias,lik,B", CASES)
def test_glm_logjoint_grad_parity(cuda, N, D, bias, lik, B):
    from edward_gb300.ops import glm_logjoint_grad
    X, y, _, _ = synthetic_logreg(N, D, seed=N + D)
    if lik == 1:
        y = (X @ np.linspace(-1, 1, D) + 0.3).astype(np.float32)
    m = f32(GLM(X, y, bias=bias, lik=lik, lik_scale=0.8, prior_loc=0.1, prior_scale=1.7))
    Z = np.random.default_rng(B).standard_normal((B, m.P)).astype(np.float32) * 0.3
    dev = glm_device(m, cuda)
    for prior in (True, False):
        lp, g = glm_logjoint_grad(dev, torch.as_tensor(Z, device=cuda), include_prior=prior)
        if prior:
            exp_lp, exp_g = m.log_joint(Z), m.grad_log_joint(Z)
        else:
            exp_lp, exp_g = m.log_lik(Z, scaled=False), m.grad_log_lik(Z, scaled=False)
        close(lp.cpu().numpy(), exp_lp)
        close(g.cpu().numpy(), exp_g)


def test_glm_golden_fixture(cuda):
    from edward_gb300.ops import glm_logjoint_grad
    g = np.load(GOLD)
    m = f32(GLM(g["lr_X"], g["lr_y"], bias=True, prior_loc=0.25, prior_scale=1.5))
    dev = glm_device(m, cuda)
    lp, gr = glm_logjoint_grad(dev, torch.as_tensor(g["lr_Z"], dtype=torch.float32, device=cuda))
    close(lp.cpu().numpy(), g["lr_lp"], rtol=1e-5)
    close(gr.cpu().numpy(), g["lr_grad"], rtol=1e-5)


def test_glm_autograd_function(cuda):
    """The autograd Function's backward is the hand-written adjoint; checked
    against FP64 central finite differences of the oracle log joint."""
    from edward_gb300.ops import glm_log_joint
    X, y, _, _ = synthetic_logreg(300, 6, seed=9)
    m = f32(GLM(X, y, bias=True))
    dev = glm_device(m, cuda)
    Z = torch.randn(4, 7, device=cuda, requires_grad=True)
    lp = glm_log_joint(dev, Z)
    lp.sum().backward()
    Zn = Z.detach().cpu().numpy().astype(np.float64)
    fd = np.zeros_like(Zn)
    h = 1e-6
    for b in range(4):
        for p in range(7):
            a, c = Zn.copy(), Zn.copy()
            a[b, p] += h
            c[b, p] -= h
            fd[b, p] = (m.log_joint(a[b:b + 1])[0] - m.log_joint(c[b:b + 1])[0]) / (2 * h)
    close(Z.grad.cpu().numpy(), fd, rtol=1e-5)


# ----------------------------------------------------------------- KLqp step

def _klqp(m, cuda, method, n_samples, optimizer=None):
    import edward_gb300 as ed
    from edward_gb300.models import Normal, Bernoulli
    D = m.D
    X = m.X.astype(np.float32)
    w = Normal(loc=ed.zeros(D) + m.prior_loc[:D], scale=ed.ones(D) * m.prior_scale[:D])
    latents = [w]
    eta = ed.dot(X, w)
    if m.bias:
        b = Normal(loc=float(m.prior_loc[D]), scale=float(m.prior_scale[D]))
        latents.append(b)
        eta = eta + b
    if m.lik == NORMAL:
        y = Normal(loc=eta, scale=float(m.lik_scale))
    else:
        y = Bernoulli(logits=eta)
    cls = {REPARAM_KL: ed.ReparameterizationKLKLqp, REPARAM: ed.ReparameterizationKLqp,
           SCORE: ed.ScoreKLqp}[method]
    inf = cls(latents, data={y: m.y.astype(np.float32)})
    inf.initialize(n_samples=n_samples, n_iter=10, n_print=0, optimizer=optimizer,
                   scale={y: float(m.data_scale)})
    return inf


@pytest.mark.parametrize("method", [REPARAM_KL, REPARAM, SCORE])
# (15000, 10, 3): 118 row blocks, more than one batch of block partials in the
# step's tail; (3000, 8, 12): 16-vector tiles; (2000, 20, 40): 40 samples, the
# per-sample sums loop
@pytest.mark.parametrize("N,D,S", [(37, 5, 4), (10000, 50, 5), (2000, 20, 40), (15000, 10, 3),
                                   (3000, 8, 12)])
def test_klqp_loss_and_gradients_parity(cuda, method, N, D, S):
    X, y, _, _ = synthetic_logreg(N, D, seed=N)
    m = f32(GLM(X, y, bias=True, data_scale=1.5, prior_scale=1.2))
    inf = _klqp(m, cuda, method, S)
    rng = np.random.default_rng(S)
    P = m.P
    mu = (rng.standard_normal(P) * 0.3).astype(np.float32)
    rho = (rng.standard_normal(P) * 0.3 - 1).astype(np.float32)
    inf._mu.copy_(torch.as_tensor(mu))
    inf._rho.copy_(torch.as_tensor(rho))
    eps = rng.standard_normal((S, P)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    e_loss, e_gmu, e_grho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, method)
    assert abs(loss - e_loss) <= RTOL * abs(e_loss)
    tol = RTOL
    close(gmu.cpu().numpy(), e_gmu, tol)
    close(grho.cpu().numpy(), e_grho, tol)
    # in-kernel Philox eps: compare against the oracle fed the same stream
    loss2, gmu2, _ = inf.loss_and_gradients(None)
    eps_k = normals(inf.seed, 0, 0, S, P)
    e_loss2, e_gmu2, _, _ = klqp_glm_loss_and_grads(m, mu, rho, eps_k, method)
    assert abs(loss2 - e_loss2) <= RTOL * abs(e_loss2)
    close(gmu2.cpu().numpy(), e_gmu2, tol)


@pytest.mark.parametrize("method", [REPARAM_KL, REPARAM, SCORE])
def test_klqp_normal_likelihood_with_scalings_parity(cuda, method):
    """Bayesian linear regression (Normal likelihood, scale 0.7) with a data
    scale of 2 on y, and for the analytic-KL estimator a KL scaling of 0.5 on w
    (``kl_scaling``, klqp.py:105-113); loss and gradients against the FP64
    oracle at the same draws, 1e-5."""
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    N, D, S = 3000, 12, 5
    rng = np.random.default_rng(40 + method)
    X = rng.standard_normal((N, D)).astype(np.float32)
    y = (X @ rng.standard_normal(D) + 0.3 + 0.7 * rng.standard_normal(N)).astype(np.float32)
    m = f32(GLM(X, y, bias=True, lik=NORMAL, lik_scale=0.7, data_scale=2.0, prior_scale=1.3))
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D) * 1.3)
    b = Normal(loc=0.0, scale=1.3)
    yv = Normal(loc=ed.dot(X, w) + b, scale=0.7)
    cls = {REPARAM_KL: ed.ReparameterizationKLKLqp, REPARAM: ed.ReparameterizationKLqp,
           SCORE: ed.ScoreKLqp}[method]
    inf = cls([w, b], data={yv: y})
    kls = {w: 0.5} if method == REPARAM_KL else None
    inf.initialize(n_samples=S, n_iter=10, n_print=0, scale={yv: 2.0}, kl_scaling=kls)
    P = m.P
    mu = (rng.standard_normal(P) * 0.3).astype(np.float32)
    rho = (rng.standard_normal(P) * 0.3 - 1).astype(np.float32)
    inf._mu.copy_(torch.as_tensor(mu))
    inf._rho.copy_(torch.as_tensor(rho))
    eps = rng.standard_normal((S, P)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    kl_scaling = np.concatenate([np.full(D, 0.5), [1.0]]) if method == REPARAM_KL else 1.0
    e_loss, e_gmu, e_grho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, method,
                                                       kl_scaling=kl_scaling)
    assert abs(loss - e_loss) <= RTOL * abs(e_loss)
    close(gmu.cpu().numpy(), e_gmu, RTOL)
    close(grho.cpu().numpy(), e_grho, RTOL)


def test_klqp_adam_trajectory_golden(cuda):
    """Three fused steps (analytic KL + TF Adam, default staircase lr) match
    the FP64 oracle trajectory in the golden fixture."""
    g = np.load(GOLD)
    m = f32(GLM(g["lr_X"], g["lr_y"], bias=True, prior_loc=0.25, prior_scale=1.5))
    inf = _klqp(m, cuda, REPARAM_KL, 4)
    inf._mu.copy_(torch.as_tensor(g["kq_mu"], dtype=torch.float32))
    inf._rho.copy_(torch.as_tensor(g["kq_rho"], dtype=torch.float32))
    eps = torch.as_tensor(g["kq_eps"], dtype=torch.float32, device=cuda).contiguous()
    for t in range(3):
        inf._step(apply=True, eps=eps)
        th = torch.cat([inf._mu, inf._rho]).cpu().numpy()
        close(th, g["kq_adam_traj"][t], rtol=2e-5)
    assert inf.t == 3


@pytest.mark.parametrize("opt_name", ["gradientdescent", "momentum", "adagrad", "rmsprop", "adam"])
def test_klqp_optimizers_apply(cuda, opt_name):
    """Each fused optimizer applies its TF update rule (one step from zero slots)."""
    X, y, _, _ = synthetic_logreg(500, 3, seed=1)
    m = f32(GLM(X, y, bias=True))
    inf = _klqp(m, cuda, REPARAM_KL, 2, optimizer=opt_name)
    mu0, rho0 = inf._mu.cpu().numpy().copy(), inf._rho.cpu().numpy().copy()
    eps = torch.randn(2, 4, device=cuda)
    _, gmu, grho = inf.loss_and_gradients(eps)
    g = torch.cat([gmu, grho]).cpu().numpy().astype(np.float64)
    inf._step(apply=True, eps=eps)
    th = torch.cat([inf._mu, inf._rho]).cpu().numpy()
    p0 = np.concatenate([mu0, rho0]).astype(np.float64)
    lr = 0.01
    if opt_name == "gradientdescent":
        exp = p0 - lr * g
    elif opt_name == "momentum":
        exp = p0 - lr * g
    elif opt_name == "adagrad":
        exp = p0 - lr * g / np.sqrt(0.1 + g * g)
    elif opt_name == "rmsprop":
        ms = 0.9 * 1.0 + 0.1 * g * g
        exp = p0 - lr * g / np.sqrt(ms + 1e-10)
    else:
        exp = TFAdam(8).apply(p0, g, lr)
    close(th, exp, rtol=1e-5)


# ----------------------------------------------------------------- HMC

def _hmc_setup(N, D, C, cuda, lik=0, bias=True):
    X, y, _, _ = synthetic_logreg(N, D, seed=C + N)
    if lik == 1:
        y = (X @ np.linspace(-1, 1, D) * 0.5).astype(np.float32)
    m = f32(GLM(X, y, bias=bias, lik=lik, lik_scale=0.5, prior_scale=1.3))
    return m, glm_device(m, cuda)


def _run_hmc_kernel(dev, C, z0, step, L, n_iter, r=None, u=None, ct=0, samples=None, seed=5):
    from edward_gb300 import _lib
    cuda = z0.device
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed, cfg.chains_per_block = step, L, seed, ct
    P = dev.P
    z = z0.clone()
    g = torch.zeros(C, P, device=cuda)
    lj = torch.zeros(C, dtype=torch.float64, device=cuda)
    nacc = torch.zeros(C, dtype=torch.int32, device=cuda)
    st = _lib.new_state(cuda)
    ratio = torch.zeros(n_iter, C, dtype=torch.float64, device=cuda)
    _lib.call("edg_hmc_glm_run", dev.ref(), ctypes.byref(cfg), C, n_iter, _lib.ptr(z),
              _lib.ptr(g), _lib.ptr(lj), 0, _lib.ptr(nacc), _lib.ptr(st), _lib.ptr(samples),
              samples.shape[0] if samples is not None else 0, None, _lib.ptr(r), _lib.ptr(u),
              _lib.ptr(ratio), _lib.stream_ptr())
    torch.cuda.synchronize()
    return z, g, lj, nacc, ratio, _lib.read_state(st)


@pytest.mark.parametrize("ct", [8, 16, 32])
@pytest.mark.parametrize("N,D,C,L,lik", [(37, 5, 3, 3, 0), (10000, 50, 70, 10, 0),
                                          (700, 130, 33, 4, 1), (50, 1, 9, 2, 1)])
def test_hmc_iteration_parity(cuda, ct, N, D, C, L, lik):
    """One iteration with override draws: leapfrog end point, FP64 ratio and
    accept decision match the oracle."""
    m, dev = _hmc_setup(N, D, C, cuda, lik=lik, bias=D > 1)
    P = m.P
    rng = np.random.default_rng(C)
    z0 = (rng.standard_normal((C, P)) * 0.2).astype(np.float32)
    r0 = rng.standard_normal((C, P)).astype(np.float32)
    u = rng.random(C)
    step = 0.01 if N > 1000 else 0.05
    if lik == 1:
        step = 0.002 if D > 1 else 0.05
    if ct == 8 and D > 64:
        pytest.skip("8 chains per block uses 256-row tiles: too much shared memory for P > 64")
    z, g, lj, nacc, ratio, st = _run_hmc_kernel(
        dev, C, torch.as_tensor(z0, device=cuda), step, L, 1,
        r=torch.as_tensor(r0[None], device=cuda).contiguous(),
        u=torch.as_tensor(u[None], device=cuda).contiguous(), ct=ct)
    f = glm_lj_grad(m)
    lj0, g0 = f(z0.astype(np.float64))
    res = hmc_step(f, z0, g0, lj0, r0, u, step, L)
    # the ratio is a difference of log joints of magnitude |lj|: 1e-5 relative to |lj|
    lj_scale = max(np.abs(lj0).max(), np.abs(res["lj"]).max(), np.abs(res["ratio"]).max())
    np.testing.assert_allclose(ratio.cpu().numpy()[0], res["ratio"], rtol=0,
                               atol=1e-5 * lj_scale + 1e-6)
    acc = nacc.cpu().numpy().astype(bool)
    margin = np.abs(np.log(u) - res["ratio"])
    assert np.all((acc == res["accept"]) | (margin < 1e-3))
    zk = z.cpu().numpy()
    for c in range(C):
        if acc[c] == res["accept"][c]:
            close(zk[c], res["z"][c], rtol=RTOL)
    assert st.t == 1


def test_hmc_golden_fixture(cuda):
    g = np.load(GOLD)
    m = f32(GLM(g["lr_X"], g["lr_y"], bias=True, prior_loc=0.25, prior_scale=1.5))
    dev = glm_device(m, cuda)
    z, _, _, nacc, ratio, _ = _run_hmc_kernel(
        dev, 3, torch.as_tensor(g["hmc_z0"], dtype=torch.float32, device=cuda), 0.05, 3, 1,
        r=torch.as_tensor(g["hmc_r0"][None], dtype=torch.float32, device=cuda).contiguous(),
        u=torch.as_tensor(g["hmc_u"][None], device=cuda).contiguous())
    # the ratio differences two log joints: 1e-5 of their magnitude
    lj_scale = np.abs(m.log_joint(g["hmc_z0"].astype(np.float64))).max()
    np.testing.assert_allclose(ratio.cpu().numpy()[0], g["hmc_ratio"], rtol=0,
                               atol=RTOL * lj_scale)
    np.testing.assert_array_equal(nacc.cpu().numpy(), g["hmc_accept"])
    close(z.cpu().numpy(), g["hmc_z"], rtol=1e-5)


def test_hmc_multi_iteration_in_kernel_rng(cuda):
    """Several iterations in one launch with in-kernel Philox draws match the
    oracle stepping the same stream (decisions may differ only where the
    ratio is within rounding of log u)."""
    C, N, D, L, T = 40, 2000, 10, 5, 6
    m, dev = _hmc_setup(N, D, C, cuda)
    P = m.P
    z0 = (np.random.default_rng(0).standard_normal((C, P)) * 0.1).astype(np.float32)
    samples = torch.zeros(T, C, P, device=cuda)
    z, _, _, nacc, ratio, st = _run_hmc_kernel(dev, C, torch.as_tensor(z0, device=cuda), 0.02,
                                               L, T, samples=samples, seed=77)
    f = glm_lj_grad(m)
    zc = z0.astype(np.float64)
    lj, gg = f(zc)
    kr = ratio.cpu().numpy()
    ks = samples.cpu().numpy()
    for t in range(T):
        r0 = normals(77, 1, t, C, P)
        u = uniforms64(77, 2, t, C)
        res = hmc_step(f, zc, gg, lj, r0, u, 0.02, L)
        np.testing.assert_allclose(kr[t], res["ratio"], rtol=0, atol=1e-5 * np.abs(lj).max())
        k_acc = np.log(u) < kr[t]
        differ = k_acc != res["accept"]
        assert np.all(np.abs(np.log(u) - res["ratio"])[differ] < 1e-3)
        same = ~differ
        close(ks[t][same], res["z"][same], rtol=RTOL)
        zc = ks[t].astype(np.float64)   # resynchronise on the kernel's kept states
        lj, gg = f(zc)
    assert st.t == T


def test_hmc_zero_steps_always_accepts(cuda):
    m, dev = _hmc_setup(100, 3, 5, cuda)
    z0 = torch.zeros(5, m.P, device=cuda)
    z, _, _, nacc, ratio, _ = _run_hmc_kernel(dev, 5, z0, 0.1, 0, 4)
    assert torch.all(nacc == 4)
    assert torch.all(ratio == 0)
