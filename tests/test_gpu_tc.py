"""GPU parity of the tensor-core (tcgen05 3xTF32) HMC engine against the
oracle and against the SIMT engine, through the C ABI."""
import ctypes

import numpy as np
import pytest
import torch

from oracle.glm import GLM, synthetic_logreg
from oracle.hmc import glm_lj_grad, hmc_step
from oracle.philox import normals, uniforms64

pytestmark = pytest.mark.gpu


def close(a, b, rtol):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * max(np.abs(b).max(), 1e-30))


def setup(N, D, C, cuda, lik=0, bias=True, seed=0):
    from edward_gb300 import _lib
    from edward_gb300.compile import GLMSpec
    from edward_gb300.ops import GLMDevice
    X, y, _, _ = synthetic_logreg(N, D, seed=seed + N)
    if lik == 1:
        y = (X @ np.linspace(-1, 1, D) * 0.5).astype(np.float32)
    m = GLM(X, y, bias=bias, lik=lik, lik_scale=0.5, prior_loc=0.1, prior_scale=1.3)
    P = m.P
    spec = GLMSpec(X=X, y=y.astype(np.float32), bias=bias, lik=lik, lik_scale=0.5,
                   prior_loc=np.full(P, 0.1, np.float32), prior_scale=np.full(P, 1.3, np.float32))
    dev = GLMDevice(spec, cuda)
    lib = _lib.load()
    nb = lib.edg_hmc_glm_tc_tiles_bytes(dev.ref())
    assert nb > 0
    tiles = torch.empty(nb, dtype=torch.uint8, device=cuda)
    _lib.call("edg_hmc_glm_tc_prepare", dev.ref(), _lib.ptr(tiles), nb, _lib.stream_ptr())
    return m, dev, tiles


def run_tc(dev, tiles, C, z0, step, L, n_iter, r=None, u=None, cluster=0, seed=5,
           samples=None, cache=None):
    from edward_gb300 import _lib
    cuda = z0.device
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed, cfg.cluster_size = step, L, seed, cluster
    P = dev.P
    z = z0.clone()
    g = torch.zeros(C, P, device=cuda) if cache is None else cache[0].clone()
    lj = torch.zeros(C, dtype=torch.float64, device=cuda) if cache is None else cache[1].clone()
    nacc = torch.zeros(C, dtype=torch.int32, device=cuda)
    st = _lib.new_state(cuda)
    ratio = torch.zeros(max(n_iter, 1), C, dtype=torch.float64, device=cuda)
    _lib.call("edg_hmc_glm_tc_run", dev.ref(), ctypes.byref(cfg), C, n_iter, _lib.ptr(tiles),
              _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), 0 if cache is None else 1, _lib.ptr(nacc),
              _lib.ptr(st), _lib.ptr(samples), samples.shape[0] if samples is not None else 0,
              None, _lib.ptr(r), _lib.ptr(u), _lib.ptr(ratio), _lib.stream_ptr())
    torch.cuda.synchronize()
    state = _lib.read_state(st)
    assert state.error == 0, "tensor-core kernel reported a wait timeout"
    return z, g, lj, nacc, ratio, state


@pytest.mark.parametrize("N,D,C,L,cluster,lik", [
    (640, 50, 128, 2, 4, 0),      # one cluster, 10 row tiles
    (2000, 50, 200, 3, 4, 0),     # partial second cluster, ragged last tile
    (1000, 13, 130, 2, 0, 1),     # P = 14 -> PP = 16 (one CTA per cluster), Normal likelihood
    (4096, 31, 256, 2, 0, 0),     # PP = 32, cluster of 2
    (6000, 60, 130, 2, 0, 0),     # PP = 64, partial second cluster
    (10000, 50, 256, 4, 4, 0),    # benchmark shape, 2 clusters
])
def test_tc_iteration_parity(cuda, N, D, C, L, cluster, lik):
    m, dev, tiles = setup(N, D, C, cuda, lik=lik)
    P = m.P
    rng = np.random.default_rng(C + N)
    z0 = (rng.standard_normal((C, P)) * 0.2).astype(np.float32)
    r0 = rng.standard_normal((C, P)).astype(np.float32)
    u = rng.random(C)
    step = 0.01 if lik == 0 else 0.003
    r_dev = torch.as_tensor(r0[None], device=cuda).contiguous()
    u_dev = torch.as_tensor(u[None], device=cuda).contiguous()
    z, g, lj, nacc, ratio, st = run_tc(dev, tiles, C, torch.as_tensor(z0, device=cuda), step, L,
                                       1, r=r_dev, u=u_dev, cluster=cluster)
    f = glm_lj_grad(m)
    lj0, g0 = f(z0.astype(np.float64))
    res = hmc_step(f, z0, g0, lj0, r0, u, step, L)
    scale = max(np.abs(lj0).max(), np.abs(res["lj"]).max())
    np.testing.assert_allclose(ratio.cpu().numpy()[0], res["ratio"], rtol=0, atol=1e-5 * scale)
    acc = nacc.cpu().numpy().astype(bool)
    differ = acc != res["accept"]
    assert np.all(np.abs(np.log(u) - res["ratio"])[differ] < 1e-3)
    zk, gk, ljk = z.cpu().numpy(), g.cpu().numpy(), lj.cpu().numpy()
    same = ~differ
    close(zk[same], res["z"][same], 1e-5)
    close(gk[same], res["g"][same], 1e-5)
    np.testing.assert_allclose(ljk[same], res["lj"][same], rtol=1e-5)
    assert st.t == 1


def test_tc_matches_simt_engine_multi_iteration(cuda):
    """Eight iterations with in-kernel Philox draws: the tensor-core and SIMT
    engines produce the same chains (both draw identical momenta/uniforms)."""
    from edward_gb300 import _lib
    N, D, C, L, T = 3000, 40, 192, 5, 8
    m, dev, tiles = setup(N, D, C, cuda)
    P = m.P
    z0 = torch.as_tensor((np.random.default_rng(1).standard_normal((C, P)) * 0.1)
                         .astype(np.float32), device=cuda)
    s_tc = torch.zeros(T, C, P, device=cuda)
    z_tc, _, _, n_tc, r_tc, _ = run_tc(dev, tiles, C, z0, 0.01, L, T, samples=s_tc, seed=9)
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed, cfg.chains_per_block = 0.01, L, 9, 32
    z = z0.clone()
    g = torch.zeros(C, P, device=cuda)
    lj = torch.zeros(C, dtype=torch.float64, device=cuda)
    nacc = torch.zeros(C, dtype=torch.int32, device=cuda)
    st = _lib.new_state(cuda)
    s_simt = torch.zeros(T, C, P, device=cuda)
    r_simt = torch.zeros(T, C, dtype=torch.float64, device=cuda)
    _lib.call("edg_hmc_glm_run", dev.ref(), ctypes.byref(cfg), C, T, _lib.ptr(z), _lib.ptr(g),
              _lib.ptr(lj), 0, _lib.ptr(nacc), _lib.ptr(st), _lib.ptr(s_simt), T, None, None,
              None, _lib.ptr(r_simt), _lib.stream_ptr())
    torch.cuda.synchronize()
    a_tc = s_tc.cpu().numpy()
    a_si = s_simt.cpu().numpy()
    # chains whose accept decisions agreed at every step must agree in value
    same = (n_tc == nacc).cpu().numpy()
    assert same.mean() > 0.95
    close(a_tc[:, same], a_si[:, same], 1e-5)
    # the ratios: 1e-5 of the log-joint magnitude they difference
    f = glm_lj_grad(m)
    lj_scale = np.abs(f(a_si[-1].astype(np.float64))[0]).max()
    np.testing.assert_allclose(r_tc.cpu().numpy()[:, same], r_simt.cpu().numpy()[:, same], rtol=0,
                               atol=1e-5 * lj_scale)


def test_tc_cache_continuation(cuda):
    """Running 2 + 3 iterations with the carried gradient / log-joint cache
    equals running 5 iterations in one launch."""
    N, D, C, L = 1500, 20, 128, 3
    m, dev, tiles = setup(N, D, C, cuda)
    P = m.P
    z0 = torch.as_tensor((np.random.default_rng(2).standard_normal((C, P)) * 0.1)
                         .astype(np.float32), device=cuda)
    z5, g5, lj5, n5, _, _ = run_tc(dev, tiles, C, z0, 0.02, L, 5, seed=3)
    from edward_gb300 import _lib
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed = 0.02, L, 3
    z = z0.clone()
    g = torch.zeros(C, P, device=cuda)
    lj = torch.zeros(C, dtype=torch.float64, device=cuda)
    nacc = torch.zeros(C, dtype=torch.int32, device=cuda)
    st = _lib.new_state(cuda)
    for k, cache in ((2, 0), (3, 1)):
        _lib.call("edg_hmc_glm_tc_run", dev.ref(), ctypes.byref(cfg), C, k, _lib.ptr(tiles),
                  _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), cache, _lib.ptr(nacc), _lib.ptr(st),
                  None, 0, None, None, None, None, _lib.stream_ptr())
    torch.cuda.synchronize()
    assert _lib.read_state(st).t == 5
    np.testing.assert_array_equal(z.cpu().numpy(), z5.cpu().numpy())
    np.testing.assert_array_equal(nacc.cpu().numpy(), n5.cpu().numpy())


def test_tc_public_api_engine(cuda):
    """ed.HMC(engine='tc') through the public API: chains move, samples land
    in Empirical.params, t advances."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, Normal
    X, y, _, _ = synthetic_logreg(2000, 10, seed=4)
    w = Normal(loc=ed.zeros(10), scale=ed.ones(10))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    T, C = 50, 256
    qw = Empirical(ed.Variable(np.zeros((T, C, 10), np.float32)), n_chains=C)
    qb = Empirical(ed.Variable(np.zeros((T, C), np.float32)), n_chains=C)
    inf = ed.HMC({w: qw, b: qb}, data={yv: y}, n_chains=C)
    inf.run(step_size=0.02, n_steps=5, engine="tc", n_print=0)
    inf.check_errors()
    assert inf.engine == "tc" and inf.t == T
    acc = inf.n_accept.float().mean().item() / T
    assert 0.3 < acc <= 1.0
    assert torch.isfinite(qw.params).all() and qw.params[-1].abs().sum() > 0


def test_tiny_dataset_falls_back_to_the_simt_engine(cuda):
    """40 rows and P = 51: one row tile cannot be split over the 4-CTA cluster
    that P = 51 needs, so the tensor-core engine reports EDG_E_UNSUPPORTED
    (engine='tc' raises) and the automatic choice takes the SIMT engine."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, Normal
    X, y, _, _ = synthetic_logreg(40, 50, seed=9)

    def model(engine):
        w = Normal(loc=ed.zeros(50), scale=ed.ones(50))
        b = Normal(loc=0.0, scale=1.0)
        yv = Bernoulli(logits=ed.dot(X, w) + b)
        T, C = 20, 16
        qw = Empirical(ed.Variable(np.zeros((T, C, 50), np.float32)), n_chains=C)
        qb = Empirical(ed.Variable(np.zeros((T, C), np.float32)), n_chains=C)
        inf = ed.HMC({w: qw, b: qb}, data={yv: y}, n_chains=C)
        inf.run(step_size=0.05, n_steps=3, engine=engine, n_print=0)
        return inf, qw
    with pytest.raises(Exception):
        model("tc")
    inf, qw = model("auto")
    assert inf.engine == "simt" and inf.t == 20
    assert torch.isfinite(qw.params).all() and qw.params[-1].abs().sum() > 0
