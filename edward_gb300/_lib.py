"""ctypes binding of the C ABI declared in ``include/edward_gb300.h``.

The CUDA library is loaded from ``edward_gb300/_lib/libedward_gb300.so``
(built in-tree by ``edward_gb300/build.py``).  There is no CPU or PyTorch
fallback: if the library cannot be loaded, every compute call raises.
"""
import ctypes
import os
import threading

import torch

from . import build as _build

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_uint32 = ctypes.c_uint32
c_uint64 = ctypes.c_uint64
c_float = ctypes.c_float
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_size_t = ctypes.c_size_t

EDG_OK = 0
EDG_E_NULL, EDG_E_SHAPE, EDG_E_VALUE, EDG_E_CUDA = -1, -2, -3, -4
EDG_E_NONFINITE, EDG_E_TIMEOUT, EDG_E_UNSUPPORTED, EDG_E_WORKSPACE = -5, -6, -7, -8

LIK_BERNOULLI, LIK_NORMAL = 0, 1
KLQP_REPARAM_KL, KLQP_REPARAM, KLQP_SCORE = 0, 1, 2
BASELINE_NONE, BASELINE_MEAN, BASELINE_MLP = 0, 1, 2
GEMM_TC, GEMM_SIMT = 0, 1
SGMCMC_SGLD, SGMCMC_SGHMC = 0, 1
EXPFAM_BETA, EXPFAM_GAMMA, EXPFAM_DIRICHLET = 0, 1, 2
PREDICT_MEAN, PREDICT_ETA, PREDICT_SAMPLE = 0, 1, 2
OPT_ADAM, OPT_SGD, OPT_MOMENTUM, OPT_ADAGRAD, OPT_RMSPROP, OPT_ADADELTA = range(6)


class EdgGLM(ctypes.Structure):
    _fields_ = [("X", c_void_p), ("y", c_void_p), ("N", c_int32), ("D", c_int32),
                ("bias", c_int32), ("lik", c_int32), ("lik_scale", c_float),
                ("prior_loc", c_void_p), ("prior_scale", c_void_p)]


class EdgState(ctypes.Structure):
    _fields_ = [("t", c_int64), ("global_step", c_int64), ("beta1_power", c_float),
                ("beta2_power", c_float), ("done", c_uint32), ("nonfinite", c_uint32),
                ("error", c_uint32), ("reserved", c_uint32), ("loss", c_double),
                ("aux", c_double * 3)]


class EdgOpt(ctypes.Structure):
    _fields_ = [("optimizer", c_int32), ("lr0", c_float), ("decay_steps", c_int64),
                ("decay_rate", c_float), ("staircase", c_int32), ("beta1", c_float),
                ("beta2", c_float), ("epsilon", c_float), ("momentum", c_float), ("rho", c_float)]


class EdgKLqp(ctypes.Structure):
    _fields_ = [("method", c_int32), ("n_samples", c_int32), ("data_scale", c_float),
                ("kl_scaling", c_void_p), ("latent_scale", c_void_p), ("seed", c_uint64),
                ("point", c_void_p)]


class EdgHier(ctypes.Structure):
    _fields_ = [("X", c_void_p), ("y", c_void_p), ("x_offset", c_void_p), ("y_offset", c_void_p),
                ("N", c_void_p), ("D", c_void_p), ("I", c_int32), ("max_D", c_int32),
                ("mu_loc", c_float), ("mu_scale", c_float), ("tau_scale", c_float)]


class EdgBNN(ctypes.Structure):
    _fields_ = [("D", c_int32), ("H1", c_int32), ("H2", c_int32), ("n_samples", c_int32),
                ("noise", c_float), ("prior_scale", c_float), ("data_scale", c_float),
                ("method", c_int32), ("gemm_engine", c_int32), ("seed", c_uint64)]


class EdgSBN(ctypes.Structure):
    _fields_ = [("V", c_int32), ("H0", c_int32), ("H1", c_int32), ("n_samples", c_int32),
                ("baseline", c_int32), ("baseline_hidden", c_int32), ("baseline_decay", c_float),
                ("gemm_engine", c_int32), ("seed", c_uint64), ("rao_blackwell", c_int32),
                ("reserved", c_int32)]


class EdgSGMCMC(ctypes.Structure):
    _fields_ = [("method", c_int32), ("step_size", c_float), ("friction", c_float),
                ("data_scale", c_float), ("seed", c_uint64)]


class EdgMH(ctypes.Structure):
    _fields_ = [("proposal_loc", c_void_p), ("proposal_scale", c_void_p), ("seed", c_uint64)]


class EdgExpFam(ctypes.Structure):
    _fields_ = [("family", c_int32), ("K", c_int32), ("prior", c_void_p), ("stats", c_void_p),
                ("transform", c_int32)]


class EdgHMC(ctypes.Structure):
    _fields_ = [("step_size", c_float), ("n_steps", c_int32), ("seed", c_uint64),
                ("chains_per_block", c_int32), ("cluster_size", c_int32), ("launch", c_int32)]


# name -> (restype, argtypes)
_SIGS = {
    "edg_abi_version": (c_int32, []),
    "edg_last_error_string": (ctypes.c_char_p, []),
    "edg_device_info": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "edg_philox_u32": (c_int32, [c_uint64, c_uint32, c_uint32, c_int32, c_int32, c_void_p, c_void_p]),
    "edg_philox_normal": (c_int32, [c_uint64, c_uint32, c_uint32, c_int32, c_int32, c_void_p, c_void_p]),
    "edg_philox_uniform64": (c_int32, [c_uint64, c_uint32, c_uint32, c_int32, c_void_p, c_void_p]),
    "edg_glm_logjoint_grad_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgGLM), c_int32]),
    "edg_glm_logjoint_grad": (c_int32, [ctypes.POINTER(EdgGLM), c_void_p, c_int32, c_int32, c_float,
                                        c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "edg_glm_logjoint_grad_noalloc": (c_int32, [ctypes.POINTER(EdgGLM), c_void_p, c_int32, c_int32,
                                                c_float, c_void_p, c_void_p, c_void_p]),
    "edg_klqp_glm_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgKLqp)]),
    "edg_klqp_glm_step": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgKLqp),
                                    ctypes.POINTER(EdgOpt), c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_int32, c_void_p, c_size_t, c_void_p]),
    "edg_hmc_glm_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgHMC), c_int32, c_int32,
                                  c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p,
                                  c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "edg_hmc_hier_run": (c_int32, [ctypes.POINTER(EdgHier), ctypes.POINTER(EdgHMC), c_int32,
                                   c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_int32,
                                   c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p]),
    "edg_hmc_hier_tc_tile_offsets": (c_int64, [c_void_p, c_void_p, c_int32, c_void_p]),
    "edg_hmc_hier_tc_prepare": (c_int32, [ctypes.POINTER(EdgHier), c_void_p, c_void_p, c_void_p]),
    "edg_hmc_hier_tc_run": (c_int32, [ctypes.POINTER(EdgHier), ctypes.POINTER(EdgHMC), c_int32,
                                      c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_int64,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "edg_gemm_workspace_bytes": (c_size_t, [c_int32, c_int32, c_int32, c_int32, c_int32, c_int32]),
    "edg_gemm": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_int32,
                           c_int64, c_void_p, c_int32, c_int64, c_void_p, c_int32, c_int64, c_int32,
                           c_int32, c_void_p, c_size_t, c_void_p]),
    "edg_gemm_status": (c_int32, [c_void_p, c_void_p]),
    "edg_check_bounded_wait": (c_int32, [c_void_p, c_void_p]),
    "edg_bnn_num_params": (c_int32, [c_int32, c_int32, c_int32]),
    "edg_bnn_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgBNN), c_int32]),
    "edg_bnn_klqp_step": (c_int32, [ctypes.POINTER(EdgBNN), ctypes.POINTER(EdgOpt), c_void_p,
                                    c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_int32, c_void_p, c_size_t, c_void_p]),
    "edg_bnn_loglik_grad": (c_int32, [ctypes.POINTER(EdgBNN), c_void_p, c_void_p, c_int32,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "edg_minibatch_gather": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_uint64,
                                       c_void_p, c_void_p, c_void_p, c_void_p]),
    "edg_sbn_num_params": (c_int32, [c_int32, c_int32, c_int32]),
    "edg_sbn_baseline_num_params": (c_int32, [c_int32, c_int32]),
    "edg_sbn_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgSBN), c_int32]),
    "edg_sbn_launches_per_step": (c_int32, [ctypes.POINTER(EdgSBN), c_int32, c_int32]),
    "edg_sbn_score_step": (c_int32, [ctypes.POINTER(EdgSBN), ctypes.POINTER(EdgOpt),
                                     ctypes.POINTER(EdgOpt), c_void_p, c_int32, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_size_t,
                                     c_void_p]),
    "edg_minibatch_gather_u8": (c_int32, [c_void_p, c_int64, c_int32, c_int32, c_uint64, c_void_p,
                                          c_void_p, c_void_p]),
    "edg_sgmcmc_glm_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgGLM), c_int32]),
    "edg_sgmcmc_glm_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgSGMCMC), c_int32,
                                     c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_int64, c_void_p, c_void_p, c_size_t, c_void_p]),
    "edg_mh_glm_workspace_bytes": (c_size_t, [ctypes.POINTER(EdgGLM), c_int32]),
    "edg_mh_glm_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgMH), c_int32, c_int32,
                                 c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                                 c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                 c_void_p]),
    "edg_expfam_hmc_run": (c_int32, [ctypes.POINTER(EdgExpFam), ctypes.POINTER(EdgHMC), c_int32,
                                     c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_void_p,
                                     c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "edg_expfam_klqp_step": (c_int32, [ctypes.POINTER(EdgExpFam), c_int32, c_uint64,
                                       ctypes.POINTER(EdgOpt), c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p, c_int32, c_void_p]),
    "edg_glm_predict": (c_int32, [ctypes.POINTER(EdgGLM), c_void_p, c_int32, c_int32, c_uint64,
                                  c_uint32, c_void_p, c_void_p]),
    "edg_hmc_glm_tc_tiles_bytes": (c_size_t, [ctypes.POINTER(EdgGLM)]),
    "edg_hmc_glm_tc_prepare": (c_int32, [ctypes.POINTER(EdgGLM), c_void_p, c_size_t, c_void_p]),
    "edg_hmc_glm_tc_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgHMC), c_int32,
                                     c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_int32,
                                     c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p]),
    "edg_mh_glm_tc_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgMH), c_int32,
                                    c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_int32,
                                    c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    "edg_sgmcmc_glm_tc_run": (c_int32, [ctypes.POINTER(EdgGLM), ctypes.POINTER(EdgSGMCMC),
                                        c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_int32, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                        c_void_p]),
}

_lock = threading.Lock()
_lib = None


class EdgError(RuntimeError):
    pass


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Loads (building first if needed and possible) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise EdgError(f"edward_gb300 CUDA library not found at {path}; run edward_gb300/build.py")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols():
    return list(_SIGS)


_EXC = {
    EDG_E_NULL: ValueError,
    EDG_E_SHAPE: ValueError,
    EDG_E_VALUE: ValueError,
    EDG_E_CUDA: RuntimeError,
    EDG_E_NONFINITE: FloatingPointError,
    EDG_E_TIMEOUT: TimeoutError,
    EDG_E_UNSUPPORTED: NotImplementedError,
    EDG_E_WORKSPACE: RuntimeError,
}


def check(rc):
    if rc == EDG_OK:
        return
    msg = load().edg_last_error_string().decode(errors="replace")
    raise _EXC.get(rc, EdgError)(msg)


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("edward_gb300 kernels need CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("edward_gb300 kernels need contiguous tensors")
    return c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return c_void_p(s.cuda_stream)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("edward_gb300 runs its inference kernels on a CUDA GPU (sm_103a); "
                           "no CUDA device is visible")
    load()


def new_state(device, beta1=0.9, beta2=0.999, t=0):
    """Device edg_state_t initialised like TF's Adam accumulators, at
    iteration t."""
    st = EdgState()
    st.beta1_power = beta1
    st.beta2_power = beta2
    st.t = t
    host = torch.frombuffer(bytearray(bytes(st)), dtype=torch.uint8)
    return host.to(device)


def read_state(state_tensor):
    raw = bytes(state_tensor.cpu().numpy().tobytes())
    return EdgState.from_buffer_copy(raw)
