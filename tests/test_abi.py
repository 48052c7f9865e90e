"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/edward_gb300.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "edward_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|size_t|const char\*)\s+(edg_\w+)\s*\(",
                                 src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from edward_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    assert "edg_hmc_glm_run" in names and "edg_klqp_glm_step" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from edward_gb300 import _lib
    assert set(declared()) <= set(_lib.exported_symbols())


def test_abi_version_and_null_checks(lib):
    lib.edg_abi_version.restype = ctypes.c_int
    assert lib.edg_abi_version() == 1
    lib.edg_last_error_string.restype = ctypes.c_char_p
    lib.edg_glm_logjoint_grad.restype = ctypes.c_int
    rc = lib.edg_glm_logjoint_grad(None, None, 1, 1, ctypes.c_float(1.0), None, None, None,
                                   ctypes.c_size_t(0), None)
    assert rc == -1  # EDG_E_NULL, raised before any CUDA call
    assert b"NULL" in lib.edg_last_error_string()


def test_library_targets_sm103a():
    """The build uses exactly one -gencode, for sm_103a."""
    from edward_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_workspace_sizes_beyond_2gib(lib):
    """Workspace sizes are computed in size_t: a batch whose gradient partials
    pass 4 GiB reports at least the bytes of those partials (an int round-up
    would wrap to a small value and accept an undersized buffer).  No GPU is
    needed: the size query only reads the descriptor (fake non-NULL pointers)."""
    from edward_gb300 import _lib
    g = _lib.EdgGLM()
    g.X = g.y = g.prior_loc = g.prior_scale = 0x1000
    g.N, g.D, g.bias, g.lik, g.lik_scale = 10_000, 255, 1, 0, 1.0
    f = lib.edg_glm_logjoint_grad_workspace_bytes
    f.restype = ctypes.c_size_t
    f.argtypes = [ctypes.POINTER(_lib.EdgGLM), ctypes.c_int32]
    B, PP = 4_300_000, 256
    need = f(ctypes.byref(g), B)
    partials = B * PP * 4 + B * 8            # one row chunk of FP32 gradients + FP64 sums
    assert partials > 2 ** 32
    assert need >= partials, (need, partials)
    assert need % 8 == 0
    small = f(ctypes.byref(g), 64)
    assert 0 < small < need


def test_hier_tc_tile_offsets(lib):
    """The host-side layout of the re-laid ragged batch: instance i starts at
    the sum over earlier instances of ceil(N/128) * 128 * (round_up(D, 8) + 1)
    floats; D outside [1, 128] or a negative N is rejected with -1."""
    import numpy as np
    f = lib.edg_hmc_hier_tc_tile_offsets
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    N = np.array([1, 128, 129, 0, 20000], np.int32)
    D = np.array([1, 8, 9, 64, 128], np.int32)
    off = np.zeros(5, np.int64)
    total = f(N.ctypes.data, D.ctypes.data, 5, off.ctypes.data)
    sizes = [((n + 127) // 128) * 128 * (((d + 7) // 8) * 8 + 1) for n, d in zip(N, D)]
    assert total == sum(sizes)
    assert list(off) == list(np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert all(o % 4 == 0 for o in off)          # 16-byte aligned float offsets
    assert f(N.ctypes.data, D.ctypes.data, 5, None) == total
    for bad_d in (0, 129):
        Db = D.copy()
        Db[2] = bad_d
        assert f(N.ctypes.data, Db.ctypes.data, 5, off.ctypes.data) == -1
    Nb = N.copy()
    Nb[0] = -1
    assert f(Nb.ctypes.data, D.ctypes.data, 5, off.ctypes.data) == -1


def test_tensor_core_entry_points_validate_before_any_cuda_call():
    """The SG-MCMC, Metropolis-Hastings and hierarchical tensor-core entry
    points reject bad arguments on the host, with the documented codes, before
    they touch the GPU (fake non-NULL device pointers; nothing is launched)."""
    import ctypes as ct
    from edward_gb300 import _lib
    lib = _lib.load()
    fake = ct.c_void_p(0x1000)
    g = _lib.EdgGLM()
    g.X = g.y = g.prior_loc = g.prior_scale = 0x1000
    g.N, g.D, g.bias, g.lik, g.lik_scale = 100, 3, 1, 0, 1.0
    sg = _lib.EdgSGMCMC()
    sg.method, sg.step_size, sg.friction, sg.data_scale, sg.seed = 7, 0.1, 0.0, 1.0, 1
    rc = lib.edg_sgmcmc_glm_tc_run(ct.byref(g), ct.byref(sg), 4, 1, fake, fake, fake, fake, 0,
                                   fake, fake, None, 0, None, None)
    assert rc == _lib.EDG_E_VALUE
    sg.method = _lib.SGMCMC_SGHMC
    rc = lib.edg_sgmcmc_glm_tc_run(ct.byref(g), ct.byref(sg), 4, 1, fake, fake, None, fake, 0,
                                   fake, fake, None, 0, None, None)
    assert rc == _lib.EDG_E_NULL  # SGHMC needs the velocity
    sg.method, sg.step_size = _lib.SGMCMC_SGLD, 0.0
    rc = lib.edg_sgmcmc_glm_tc_run(ct.byref(g), ct.byref(sg), 4, 1, fake, fake, None, fake, 0,
                                   fake, fake, None, 0, None, None)
    assert rc == _lib.EDG_E_VALUE
    mhc = _lib.EdgMH()
    mhc.proposal_loc, mhc.proposal_scale, mhc.seed = None, None, 1
    rc = lib.edg_mh_glm_tc_run(ct.byref(g), ct.byref(mhc), 4, 1, fake, fake, fake, fake, 0, fake,
                               fake, None, 0, None, None, None, None)
    assert rc == _lib.EDG_E_NULL
    g.D = 70  # P = 71 > 64
    mhc.proposal_scale = 0x1000
    rc = lib.edg_mh_glm_tc_run(ct.byref(g), ct.byref(mhc), 4, 1, fake, fake, fake, fake, 0, fake,
                               fake, None, 0, None, None, None, None)
    assert rc == _lib.EDG_E_UNSUPPORTED
    hm = _lib.EdgHier()
    hm.X = hm.y = hm.x_offset = hm.y_offset = hm.N = hm.D = 0x1000
    hm.I, hm.max_D, hm.mu_loc, hm.mu_scale, hm.tau_scale = 2, 16, 0.0, 1.0, 1.0
    cfg = _lib.EdgHMC()
    cfg.step_size, cfg.n_steps, cfg.seed = 0.01, 3, 1
    args = lambda tiles, toff: (ct.byref(hm), ct.byref(cfg), 4, 1, None, tiles, toff,  # noqa: E731
                                fake, fake, fake, 0, None, fake, None, 0, None, None, None,
                                None, None)
    assert lib.edg_hmc_hier_tc_run(*args(None, fake)) == _lib.EDG_E_NULL
    assert lib.edg_hmc_hier_tc_run(*args(ct.c_void_p(0x1004), fake)) == _lib.EDG_E_VALUE
    hm.max_D = 129
    assert lib.edg_hmc_hier_tc_run(*args(fake, fake)) == _lib.EDG_E_UNSUPPORTED
    for code in (_lib.EDG_E_NULL, _lib.EDG_E_VALUE, _lib.EDG_E_UNSUPPORTED):
        assert code < 0
