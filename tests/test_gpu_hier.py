"""GPU parity of the ragged hierarchical HMC kernel against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import hier
from oracle.hmc import hmc_step
from oracle.philox import normals, uniforms64

pytestmark = pytest.mark.gpu


def _instances(seed=3):
    Xs, ys = hier.synthetic_instances(5, seed=seed, n_range=(50, 700), d_range=(8, 40))
    X2, y2 = hier.synthetic_instances(1, seed=seed + 1, n_range=(300, 300), d_range=(128, 128))
    return Xs + X2, ys + y2


def _run(hd, C, z0, n_iter, step, L, r=None, u=None, seed=7, samples=None, launch=0, ct=32,
         engine="simt"):
    from edward_gb300 import _lib
    cuda = z0.device
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed, cfg.launch = step, L, seed, launch
    cfg.chains_per_block = ct
    n = hd.I * C
    z = z0.clone()
    g = torch.zeros_like(z)
    lj = torch.zeros(n, dtype=torch.float64, device=cuda)
    nacc = torch.zeros(n, dtype=torch.int32, device=cuda)
    st = _lib.new_state(cuda)
    ratio = torch.zeros(max(n_iter, 1), n, dtype=torch.float64, device=cuda)
    if engine == "tc":
        tiles, toff = hd.tc_tiles()
        fn, lead = "edg_hmc_hier_tc_run", (_lib.ptr(hd.order), _lib.ptr(tiles), _lib.ptr(toff))
    else:
        fn, lead = "edg_hmc_hier_run", (_lib.ptr(hd.order),)
    _lib.call(fn, hd.ref(), ctypes.byref(cfg), C, n_iter, *lead,
              _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), 0, _lib.ptr(nacc), _lib.ptr(st),
              _lib.ptr(samples), samples.shape[0] if samples is not None else 0, None,
              _lib.ptr(r), _lib.ptr(u), _lib.ptr(ratio), _lib.stream_ptr())
    torch.cuda.synchronize()
    return z, g, lj, nacc, ratio, _lib.read_state(st)


@pytest.mark.parametrize("engine,ct,C", [("simt", 32, 40), ("simt", 16, 40), ("tc", 0, 40),
                                         ("tc", 0, 100)])
def test_hier_iteration_parity(cuda, engine, ct, C):
    """One iteration of every instance against the oracle: the SIMT engine in
    both tile shapes (32 chains x 64 rows, 16 chains x 128 rows) and the
    tensor-core engine (64 chains x 128 rows; 100 chains = a full and a
    partial chain tile per instance).  Instances span D = 8..40 and D = 128
    over 3 row tiles (the last one partial)."""
    from edward_gb300.ops import HierDevice
    Xs, ys = _instances()
    kw = dict(mu_loc=0.1, mu_scale=1.2, tau_scale=0.8)
    hd = HierDevice(Xs, ys, **kw)
    L, step = 3, 0.01
    SP = hd.SP
    rng = np.random.default_rng(0)
    z0 = np.zeros((hd.I * C, SP), np.float32)
    r0 = np.zeros((1, hd.I * C, SP), np.float32)
    cols = lambda D: list(range(D)) + [SP - 2, SP - 1]   # noqa: E731  (w, mu, u)
    for i, X in enumerate(Xs):
        D = X.shape[1]
        z0[i * C:(i + 1) * C, cols(D)] = rng.standard_normal((C, D + 2)) * 0.2
        r0[0][i * C:(i + 1) * C, cols(D)] = rng.standard_normal((C, D + 2))
    u = rng.random((1, hd.I * C))
    z, g, lj, nacc, ratio, st = _run(hd, C, torch.as_tensor(z0, device=cuda), 1, step, L,
                                     r=torch.as_tensor(r0, device=cuda),
                                     u=torch.as_tensor(u, device=cuda), ct=ct, engine=engine)
    assert st.t == 1
    zk, rk, ak = z.cpu().numpy(), ratio.cpu().numpy()[0], nacc.cpu().numpy().astype(bool)
    for i, (X, y) in enumerate(zip(Xs, ys)):
        D = X.shape[1]
        sl = slice(i * C, (i + 1) * C)
        f = hier.lj_grad_fn(X, y, **kw)
        zi = z0[sl][:, cols(D)].astype(np.float64)
        lj0, g0 = f(zi)
        res = hmc_step(f, zi, g0, lj0, r0[0][sl][:, cols(D)], u[0, sl], step, L)
        scale = max(np.abs(lj0).max(), np.abs(res["lj"]).max())
        np.testing.assert_allclose(rk[sl], res["ratio"], rtol=0, atol=1e-5 * scale)
        differ = ak[sl] != res["accept"]
        assert np.all(np.abs(np.log(u[0, sl]) - res["ratio"])[differ] < 1e-3)
        same = ~differ
        exp = res["z"][same]
        np.testing.assert_allclose(zk[sl][:, cols(D)][same], exp, rtol=1e-5,
                                   atol=1e-5 * np.abs(exp).max())


@pytest.mark.parametrize("engine", ["simt", "tc"])
def test_hier_in_kernel_rng_two_iterations(cuda, engine):
    from edward_gb300.ops import HierDevice
    Xs, ys = _instances(seed=9)
    hd = HierDevice(Xs, ys)
    C, L, step, T, seed = 33, 2, 0.02, 2, 11
    SP = hd.SP
    z0 = np.zeros((hd.I * C, SP), np.float32)
    rng = np.random.default_rng(1)
    cols = lambda D: list(range(D)) + [SP - 2, SP - 1]   # noqa: E731
    for i, X in enumerate(Xs):
        z0[i * C:(i + 1) * C, cols(X.shape[1])] = rng.standard_normal((C, X.shape[1] + 2)) * 0.1
    samples = torch.zeros(T, hd.I * C, SP, device=cuda)
    z, _, _, nacc, ratio, st = _run(hd, C, torch.as_tensor(z0, device=cuda), T, step, L,
                                    seed=seed, samples=samples, engine=engine)
    assert st.t == T
    sk = samples.cpu().numpy()
    rk = ratio.cpu().numpy()
    for i, (X, y) in enumerate(zip(Xs, ys)):
        D = X.shape[1]
        f = hier.lj_grad_fn(X, y)
        zi = z0[i * C:(i + 1) * C][:, cols(D)].astype(np.float64)
        lj, gr = f(zi)
        for t in range(T):
            r0 = normals(seed, 1, t, C, D + 2, row0=i * C)
            uu = uniforms64(seed, 2, t, C, row0=i * C)
            res = hmc_step(f, zi, gr, lj, r0, uu, step, L)
            scale = max(np.abs(lj).max(), 1.0)
            np.testing.assert_allclose(rk[t, i * C:(i + 1) * C], res["ratio"], rtol=0,
                                       atol=1e-5 * scale)
            zi = sk[t, i * C:(i + 1) * C][:, cols(D)].astype(np.float64)  # resync on kept states
            lj, gr = f(zi)


def test_hier_public_api_ragged_batch(cuda):
    """Edward-style model code: mu ~ N(0,1), tau ~ HalfNormal(1) with support
    'nonnegative', w ~ N(mu, tau), y ~ Bernoulli(X w); X and y bound to lists
    of arrays form a ragged batch of independent instances."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, HalfNormal, Normal
    Xs, ys = hier.synthetic_instances(6, seed=21, n_range=(100, 1500), d_range=(5, 30))
    Dmax = max(x.shape[1] for x in Xs)
    X = ed.placeholder(np.float32, [None, None])
    mu = Normal(loc=0.0, scale=1.0)
    tau = HalfNormal(scale=1.0)
    tau.support = "nonnegative"
    w = Normal(loc=mu * ed.ones(Dmax), scale=tau * ed.ones(Dmax))
    y = Bernoulli(logits=ed.dot(X, w))
    T, C = 300, 16
    qw = Empirical(ed.Variable(np.zeros((T, 6, C, Dmax), np.float32)), n_chains=None)
    qmu = Empirical(ed.Variable(np.zeros((T, 6, C), np.float32)))
    qtau = Empirical(ed.Variable(np.zeros((T, 6, C), np.float32)))
    inf = ed.HMC({w: qw, mu: qmu, tau: qtau}, data={X: Xs, y: ys}, n_chains=C)
    inf.run(step_size=0.02, n_steps=8, n_print=0)
    assert inf.engine == "hier" and inf.t == T
    acc = inf.n_accept.float().mean().item() / T
    assert 0.2 < acc <= 1.0
    taus = qtau.params[T // 2:]
    assert torch.all(taus > 0)
    # posterior mean of w per instance correlates with the truth-generating direction
    wm = qw.params[T // 2:].mean(dim=(0, 2)).cpu().numpy()
    for i, (Xi, yi) in enumerate(zip(Xs, ys)):
        D = Xi.shape[1]
        assert np.all(np.isfinite(wm[i, :D])) and np.all(wm[i, D:] == 0)


@pytest.mark.parametrize("engine", ["simt", "tc"])
def test_hier_launch_forms_agree(cuda, engine):
    """The persistent work-queue grid and the one-CTA-per-item grid run the
    same arithmetic per (instance, chain tile): identical chains, ratios and
    acceptance counts; t advances and the work counter is left at 0."""
    from edward_gb300.ops import HierDevice
    Xs, ys = _instances(seed=11)
    hd = HierDevice(Xs, ys)
    C, T = 48, 3
    z0 = torch.as_tensor(np.random.default_rng(2).standard_normal((hd.I * C, hd.SP))
                         .astype(np.float32) * 0.1, device=cuda)
    outs = []
    for launch in (0, 1):
        samples = torch.zeros(T, hd.I * C, hd.SP, device=cuda)
        z, g, lj, nacc, ratio, st = _run(hd, C, z0, T, 0.01, 4, seed=5, samples=samples,
                                         launch=launch, engine=engine)
        assert st.t == T and st.done == 0 and st.reserved == 0
        outs.append((samples.cpu().numpy(), lj.cpu().numpy(), nacc.cpu().numpy(),
                     ratio.cpu().numpy()))
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)


def test_hier_graph_replay_matches_direct_launch(cuda):
    """ed.HMC on the ragged batch replays k-iteration launches from a CUDA
    graph once the gradient cache is valid: five one-iteration calls (the
    first launched directly, the rest replayed) give the same samples as one
    five-iteration launch."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Empirical, HalfNormal, Normal
    Xs, ys = hier.synthetic_instances(4, seed=31, n_range=(100, 900), d_range=(5, 20))
    Dmax = max(x.shape[1] for x in Xs)
    runs = []
    for mode in ("graph", "direct"):
        ed.set_seed(9)
        X = ed.placeholder(np.float32, [None, None])
        mu = Normal(loc=0.0, scale=1.0)
        tau = HalfNormal(scale=1.0)
        tau.support = "nonnegative"
        w = Normal(loc=mu * ed.ones(Dmax), scale=tau * ed.ones(Dmax))
        y = Bernoulli(logits=ed.dot(X, w))
        T, C = 5, 8
        qw = Empirical(ed.Variable(np.zeros((T, 4, C, Dmax), np.float32)), n_chains=None)
        qmu = Empirical(ed.Variable(np.zeros((T, 4, C), np.float32)))
        qtau = Empirical(ed.Variable(np.zeros((T, 4, C), np.float32)))
        inf = ed.HMC({w: qw, mu: qmu, tau: qtau}, data={X: Xs, y: ys}, n_chains=C)
        inf.initialize(step_size=0.02, n_steps=4, n_print=0)
        if mode == "graph":
            for _ in range(T):
                inf.run_iterations(1)
            assert 1 in inf._graphs
        else:
            inf.run_iterations(T)
        torch.cuda.synchronize()
        assert inf.t == T
        runs.append((qw.params.cpu().numpy(), qmu.params.cpu().numpy(),
                     inf.n_accept.cpu().numpy()))
    for a, b in zip(runs[0], runs[1]):
        np.testing.assert_array_equal(a, b)


def test_hier_engines_agree(cuda):
    """The tensor-core and SIMT engines draw the same Philox momenta and
    uniforms: over 4 iterations of 100 chains per instance the log acceptance
    ratios agree to 1e-5 of the log joint, and the kept states agree wherever
    both engines took the same decisions (all of them, away from ties)."""
    from edward_gb300.ops import HierDevice
    Xs, ys = _instances(seed=13)
    hd = HierDevice(Xs, ys)
    C, T = 100, 4
    z0 = torch.as_tensor(np.random.default_rng(4).standard_normal((hd.I * C, hd.SP))
                         .astype(np.float32) * 0.1, device=cuda)
    outs = {}
    for engine in ("simt", "tc"):
        samples = torch.zeros(T, hd.I * C, hd.SP, device=cuda)
        z, g, lj, nacc, ratio, st = _run(hd, C, z0, T, 0.01, 4, seed=3, samples=samples,
                                         engine=engine)
        assert st.t == T and st.error == 0
        outs[engine] = (samples.cpu().numpy(), lj.cpu().numpy(), ratio.cpu().numpy(),
                        nacc.cpu().numpy())
    s_a, lj_a, r_a, n_a = outs["simt"]
    s_b, lj_b, r_b, n_b = outs["tc"]
    scale = max(np.abs(lj_a).max(), 1.0)
    np.testing.assert_allclose(r_b, r_a, rtol=0, atol=1e-5 * scale)
    if np.array_equal(n_a, n_b):
        np.testing.assert_allclose(s_b, s_a, rtol=1e-5, atol=1e-5 * np.abs(s_a).max())
        np.testing.assert_allclose(lj_b, lj_a, rtol=0, atol=1e-5 * scale)


@pytest.mark.parametrize("C", [1, 65])
def test_hier_tensor_core_edge_shapes(cuda, C):
    """The tensor-core engine on edge shapes against the oracle: D = 1, 3
    (one 8-wide K step), 64 / 65 (the K-step and XF chunk boundaries), 127 and
    128 (the feature limit); N = 1, 128 and 129 rows (exact and one-over tiles),
    300; a single chain and 65 chains (a second chain tile of one chain)."""
    from edward_gb300.ops import HierDevice
    rng = np.random.default_rng(17)
    shapes = [(1, 5), (128, 1), (129, 3), (300, 64), (200, 65), (129, 127), (257, 128)]
    Xs, ys = [], []
    for N, D in shapes:
        X = rng.standard_normal((N, D)).astype(np.float32)
        w = rng.standard_normal(D) * 0.5
        p = 1.0 / (1.0 + np.exp(-(X.astype(np.float64) @ w)))
        Xs.append(X)
        ys.append((rng.random(N) < p).astype(np.float32))
    kw = dict(mu_loc=-0.2, mu_scale=0.9, tau_scale=1.3)
    hd = HierDevice(Xs, ys, **kw)
    L, step = 3, 0.02
    SP = hd.SP
    z0 = np.zeros((hd.I * C, SP), np.float32)
    r0 = np.zeros((1, hd.I * C, SP), np.float32)
    cols = lambda D: list(range(D)) + [SP - 2, SP - 1]   # noqa: E731
    for i, X in enumerate(Xs):
        D = X.shape[1]
        z0[i * C:(i + 1) * C, cols(D)] = rng.standard_normal((C, D + 2)) * 0.2
        r0[0][i * C:(i + 1) * C, cols(D)] = rng.standard_normal((C, D + 2))
    u = rng.random((1, hd.I * C))
    z, g, lj, nacc, ratio, st = _run(hd, C, torch.as_tensor(z0, device=cuda), 1, step, L,
                                     r=torch.as_tensor(r0, device=cuda),
                                     u=torch.as_tensor(u, device=cuda), engine="tc")
    assert st.t == 1 and st.error == 0
    zk, gk, rk = z.cpu().numpy(), g.cpu().numpy(), ratio.cpu().numpy()[0]
    ak = nacc.cpu().numpy().astype(bool)
    for i, (X, y) in enumerate(zip(Xs, ys)):
        D = X.shape[1]
        sl = slice(i * C, (i + 1) * C)
        f = hier.lj_grad_fn(X, y, **kw)
        zi = z0[sl][:, cols(D)].astype(np.float64)
        lj0, g0 = f(zi)
        res = hmc_step(f, zi, g0, lj0, r0[0][sl][:, cols(D)], u[0, sl], step, L)
        scale = max(np.abs(lj0).max(), np.abs(res["lj"]).max(), 1.0)
        np.testing.assert_allclose(rk[sl], res["ratio"], rtol=0, atol=1e-5 * scale)
        same = ak[sl] == res["accept"]
        exp = res["z"][same]
        np.testing.assert_allclose(zk[sl][:, cols(D)][same], exp, rtol=1e-5,
                                   atol=1e-5 * max(np.abs(exp).max(), 1.0))
        # the cached gradient belongs to the kept state
        _, gkept = f(zk[sl][:, cols(D)].astype(np.float64))
        np.testing.assert_allclose(gk[sl][:, cols(D)], gkept, rtol=1e-5,
                                   atol=1e-5 * max(np.abs(gkept).max(), 1.0))
