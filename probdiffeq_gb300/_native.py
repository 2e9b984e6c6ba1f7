"""ctypes binding of the C ABI in ``include/pdq.h``.

This module is the only place that talks to ``libpdq_gb300.so``.  It fails
loudly when the library is missing: there is no CPU fallback.
"""

import ctypes
import math
import os

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libpdq_gb300.so")

ABI_VERSION = 2

# enums (include/pdq.h)
SSM = {"isotropic": 0, "blockdiag": 1, "dense": 2}
CONSTRAINT = {"ts0": 0, "ts1": 1}
STRATEGY = {"filter": 0, "fixedpoint": 1}
SOLVER = {"none": 0, "mle": 1, "dynamic": 2}
ERROR = {"residual_std": 0, "state_std": 1}
CONTROL = {"integral": 0, "proportional_integral": 1}
PRECISION = {"float32": 0, "float64": 1}
FIELD = {"lotka_volterra": 0, "van_der_pol": 1, "fitzhugh_nagumo": 2, "burgers": 3}
FIELD_USER_BASE = 1000  # PDQ_FIELD_USER_BASE: ids of fields registered at run time
INSTANCE_STATUS = {0: "ok", 1: "max_steps", 2: "dt_underflow", 3: "nonfinite"}


class PdqConfig(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_uint32),
        ("ssm", ctypes.c_int32),
        ("constraint", ctypes.c_int32),
        ("strategy", ctypes.c_int32),
        ("solver", ctypes.c_int32),
        ("error", ctypes.c_int32),
        ("control", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("field", ctypes.c_int32),
        ("num_derivatives", ctypes.c_int32),
        ("ode_dim", ctypes.c_int32),
        ("clip_dt", ctypes.c_int32),
        ("correct_asymptotic_underconfidence", ctypes.c_int32),
        ("kernel_variant", ctypes.c_int32),
        ("safety", ctypes.c_double),
        ("factor_min", ctypes.c_double),
        ("factor_max", ctypes.c_double),
        ("exponent_integral", ctypes.c_double),
        ("exponent_proportional", ctypes.c_double),
        ("atol", ctypes.c_double),
        ("rtol", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("damp", ctypes.c_double),
        ("max_attempts", ctypes.c_int64),
        ("instances_per_block", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
    ]


class PdqAdaptiveArgs(ctypes.Structure):
    _fields_ = [
        ("num_instances", ctypes.c_int64),
        ("num_save_at", ctypes.c_int32),
        ("terminal_only", ctypes.c_int32),
        ("save_at", ctypes.c_void_p),
        ("params", ctypes.c_void_p),
        ("y0", ctypes.c_void_p),
        ("dt0", ctypes.c_void_p),
        ("u_mean", ctypes.c_void_p),
        ("u_chol", ctypes.c_void_p),
        ("output_scale", ctypes.c_void_p),
        ("t", ctypes.c_void_p),
        ("num_steps", ctypes.c_void_p),
        ("num_attempts", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
        ("cond_A", ctypes.c_void_p),
        ("cond_noise_mean", ctypes.c_void_p),
        ("cond_noise_chol", ctypes.c_void_p),
        ("cond_to_latent", ctypes.c_void_p),
        ("cond_to_observed", ctypes.c_void_p),
        ("filter_mean", ctypes.c_void_p),
        ("filter_chol", ctypes.c_void_p),
        ("u_mean_d_params", ctypes.c_void_p),
        ("u_mean_d_y0", ctypes.c_void_p),
    ]


class PdqSampleArgs(ctypes.Structure):
    _fields_ = [
        ("ssm", ctypes.c_int32),
        ("num_derivatives", ctypes.c_int32),
        ("ode_dim", ctypes.c_int32),
        ("num_points", ctypes.c_int32),
        ("num_instances", ctypes.c_int64),
        ("num_samples", ctypes.c_int32),
        ("marginal_mean", ctypes.c_void_p),
        ("marginal_chol", ctypes.c_void_p),
        ("cond_A", ctypes.c_void_p),
        ("cond_noise_mean", ctypes.c_void_p),
        ("cond_noise_chol", ctypes.c_void_p),
        ("cond_to_latent", ctypes.c_void_p),
        ("cond_to_observed", ctypes.c_void_p),
        ("normals", ctypes.c_void_p),
        ("samples", ctypes.c_void_p),
    ]


class PdqOffgridArgs(ctypes.Structure):
    _fields_ = [
        ("ssm", ctypes.c_int32),
        ("strategy", ctypes.c_int32),
        ("num_derivatives", ctypes.c_int32),
        ("ode_dim", ctypes.c_int32),
        ("num_instances", ctypes.c_int64),
        ("num_points", ctypes.c_int32),
        ("num_queries", ctypes.c_int32),
        ("t", ctypes.c_void_p),
        ("u_mean", ctypes.c_void_p),
        ("u_chol", ctypes.c_void_p),
        ("filter_mean", ctypes.c_void_p),
        ("filter_chol", ctypes.c_void_p),
        ("output_scale", ctypes.c_void_p),
        ("t_query", ctypes.c_void_p),
        ("mean_out", ctypes.c_void_p),
        ("chol_out", ctypes.c_void_p),
    ]


class PdqLmlArgs(ctypes.Structure):
    _fields_ = [
        ("num_instances", ctypes.c_int64),
        ("num_steps", ctypes.c_int32),
        ("save_every", ctypes.c_int32),
        ("average_pdfs", ctypes.c_int32),
        ("with_gradient", ctypes.c_int32),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("params", ctypes.c_void_p),
        ("y0", ctypes.c_void_p),
        ("data", ctypes.c_void_p),
        ("std", ctypes.c_void_p),
        ("lml", ctypes.c_void_p),
        ("grad", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
    ]



class PdqLmlAdjointArgs(ctypes.Structure):
    _fields_ = [
        ("lml", PdqLmlArgs),
        ("checkpoint_every", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("cotangent", ctypes.c_void_p),
        ("grad_y0", ctypes.c_void_p),
    ]

class PdqTerminalAdjointArgs(ctypes.Structure):
    _fields_ = [
        ("num_instances", ctypes.c_int64),
        ("capacity", ctypes.c_int32),
        ("checkpoint_every", ctypes.c_int32),
        ("params", ctypes.c_void_p),
        ("y0", ctypes.c_void_p),
        ("num_steps", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
        ("cotangent", ctypes.c_void_p),
        ("grad_params", ctypes.c_void_p),
        ("grad_y0", ctypes.c_void_p),
    ]


# Every symbol include/pdq.h declares, with its ctypes signature.
SIGNATURES = {
    "pdq_abi_version": (ctypes.c_uint32, []),
    "pdq_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pdq_config_default": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
    ),
    "pdq_workspace_size": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "pdq_solve_adaptive": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqAdaptiveArgs), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "pdq_lml_workspace_size": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "pdq_lml_fixed_grid": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqLmlArgs), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "pdq_lml_adjoint_workspace_size": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
         ctypes.POINTER(ctypes.c_size_t)],
    ),
    "pdq_lml_fwd": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqLmlAdjointArgs), ctypes.c_void_p, ctypes.c_size_t,
         ctypes.c_void_p],
    ),
    "pdq_lml_bwd": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqLmlAdjointArgs), ctypes.c_void_p, ctypes.c_size_t,
         ctypes.c_void_p],
    ),
    "pdq_lml_fixed_grid_static": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqLmlArgs), ctypes.c_void_p],
    ),
    "pdq_terminal_record_size": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "pdq_terminal_fwd": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqAdaptiveArgs), ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_size_t, ctypes.c_void_p],
    ),
    "pdq_terminal_bwd": (
        ctypes.c_int,
        [ctypes.POINTER(PdqConfig), ctypes.POINTER(PdqTerminalAdjointArgs), ctypes.c_void_p, ctypes.c_size_t,
         ctypes.c_void_p],
    ),
    "pdq_sample_markov": (ctypes.c_int, [ctypes.POINTER(PdqSampleArgs), ctypes.c_void_p]),
    "pdq_offgrid_marginals": (ctypes.c_int, [ctypes.POINTER(PdqOffgridArgs), ctypes.c_void_p]),
    "pdq_register_field": (
        ctypes.c_int,
        [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
         ctypes.c_char_p, ctypes.c_size_t],
    ),
    "pdq_register_stencil": (
        ctypes.c_int,
        [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.c_char_p,
         ctypes.c_size_t],
    ),
    "pdq_probe_fp32_fma": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
    ),
    "pdq_probe_sm_count": (ctypes.c_int, []),
}

_LIB = None


class NativeError(RuntimeError):
    """A non-zero pdq_status returned by the native library."""

    def __init__(self, status, where):
        self.status = status
        super().__init__(f"{where}: {status_string(status)} (pdq_status {status})")


def load():
    """Load ``libpdq_gb300.so`` (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"native library {LIB_PATH} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)"
        )
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.pdq_abi_version() != ABI_VERSION:
        raise RuntimeError("libpdq_gb300.so ABI version mismatch")
    _LIB = lib
    return lib


def status_string(status):
    return load().pdq_status_string(int(status)).decode()


def check(status, where):
    if status != 0:
        raise NativeError(status, where)


def register_field(name, source, dim, num_params):
    """Compile a user vector field (CUDA C++ source of ``struct Field``) with
    NVRTC (``pdq_register_field``); returns its field id and makes ``name``
    usable wherever a field name is accepted.  Raises NativeError with the
    compiler log on failure."""
    lib = load()
    fid = ctypes.c_int32(-1)
    log = ctypes.create_string_buffer(1 << 16)
    st = lib.pdq_register_field(name.encode(), source.encode(), int(dim), int(num_params), ctypes.byref(fid), log,
                                ctypes.sizeof(log))
    if st != 0:
        raise NativeError(st, "pdq_register_field:\n" + log.value.decode(errors="replace"))
    FIELD[name] = fid.value
    return fid.value


def register_stencil(name, source, num_params):
    """Compile a stencil field for the block-diagonal kernel (CUDA C++ source
    of ``struct Stencil``, any d on a periodic grid) with NVRTC
    (``pdq_register_stencil``); returns its field id and makes ``name`` usable
    as the field of a block-diagonal configuration (TS0).  Raises NativeError
    with the compiler log on failure."""
    lib = load()
    fid = ctypes.c_int32(-1)
    log = ctypes.create_string_buffer(1 << 16)
    st = lib.pdq_register_stencil(name.encode(), source.encode(), int(num_params), ctypes.byref(fid), log,
                                  ctypes.sizeof(log))
    if st != 0:
        raise NativeError(st, "pdq_register_stencil:\n" + log.value.decode(errors="replace"))
    FIELD[name] = fid.value
    return fid.value


def config_default(ssm, field, num_derivatives, ode_dim):
    cfg = PdqConfig()
    check(load().pdq_config_default(ctypes.byref(cfg), SSM[ssm], FIELD[field], num_derivatives, ode_dim), "pdq_config_default")
    return cfg


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream_handle(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def solve_adaptive(cfg, save_at, params, y0, dt0, terminal_only, outputs, stream=None, workspace=None):
    """Call pdq_solve_adaptive on device tensors (all float64, contiguous).

    ``outputs`` is a dict of preallocated device tensors (see ``alloc_outputs``).
    """
    B = y0.shape[0]
    args = PdqAdaptiveArgs()
    args.num_instances = B
    args.num_save_at = save_at.shape[1]
    args.terminal_only = 1 if terminal_only else 0
    args.save_at = _ptr(save_at)
    args.params = _ptr(params)
    args.y0 = _ptr(y0)
    args.dt0 = _ptr(dt0)
    for k in ("u_mean", "u_chol", "output_scale", "t", "num_steps", "num_attempts", "status"):
        setattr(args, k, _ptr(outputs[k]))
    for k in OPTIONAL_OUTPUTS + SENSITIVITY_OUTPUTS:
        setattr(args, k, _ptr(outputs.get(k)))
    lib = load()
    ws_bytes = workspace_size(cfg, B, save_at.shape[1])
    ws = workspace if workspace is not None else None
    if ws_bytes > 0 and (ws is None or ws.numel() * ws.element_size() < ws_bytes):
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=y0.device)
    check(
        lib.pdq_solve_adaptive(ctypes.byref(cfg), ctypes.byref(args), _ptr(ws), ctypes.c_size_t(ws_bytes), _stream_handle(stream)),
        "pdq_solve_adaptive",
    )
    if ws is not None:
        outputs["_workspace"] = ws
    return outputs


OPTIONAL_OUTPUTS = ("cond_A", "cond_noise_mean", "cond_noise_chol", "cond_to_latent", "cond_to_observed", "filter_mean", "filter_chol")
SENSITIVITY_OUTPUTS = ("u_mean_d_params", "u_mean_d_y0")


INSTANCE_RECORD_FULL = 4
TERMINAL_CAPACITY = 2048  # first guess of accepted steps per instance for terminal_fwd


def terminal_record_size(cfg, B, capacity, checkpoint_every):
    nbytes = ctypes.c_size_t(0)
    check(load().pdq_terminal_record_size(ctypes.byref(cfg), int(B), int(capacity), int(checkpoint_every),
                                          ctypes.byref(nbytes)), "pdq_terminal_record_size")
    return int(nbytes.value)


def terminal_fwd(cfg, save_at, params, y0, dt0, *, capacity=None, checkpoint_every=None, stream=None):
    """Terminal values (``pdq_terminal_fwd``) with the record the adjoint
    pass reads.  Device tensors as ``solve_adaptive`` (save_at (B, 2)).
    ``capacity`` None: a first guess, and when an instance took more accepted
    steps (PDQ_INSTANCE_RECORD_FULL; one host synchronisation) a rerun with
    exactly the largest count; ``checkpoint_every`` None: round(sqrt(capacity)).
    Returns the outputs of ``alloc_outputs`` plus the record ("_record",
    "_capacity", "_checkpoint_every")."""
    B = y0.shape[0]
    outputs = alloc_outputs(cfg, B, 2, True, y0.device)
    cap = int(capacity) if capacity is not None else TERMINAL_CAPACITY
    lib = load()
    while True:
        ckpt = min(cap, int(checkpoint_every) if checkpoint_every else max(1, round(math.sqrt(cap))))
        nbytes = terminal_record_size(cfg, B, cap, ckpt)
        rec = torch.empty(nbytes, dtype=torch.uint8, device=y0.device)
        args = PdqAdaptiveArgs()
        args.num_instances = B
        args.num_save_at = 2
        args.terminal_only = 1
        args.save_at, args.params, args.y0, args.dt0 = _ptr(save_at), _ptr(params), _ptr(y0), _ptr(dt0)
        for k in ("u_mean", "u_chol", "output_scale", "t", "num_steps", "num_attempts", "status"):
            setattr(args, k, _ptr(outputs[k]))
        check(lib.pdq_terminal_fwd(ctypes.byref(cfg), ctypes.byref(args), cap, ckpt, _ptr(rec), ctypes.c_size_t(nbytes),
                                   _stream_handle(stream)), "pdq_terminal_fwd")
        if capacity is None and bool((outputs["status"] == INSTANCE_RECORD_FULL).any()):
            cap = int(outputs["num_steps"].max())
            continue
        break
    outputs.update(_record=rec, _capacity=cap, _checkpoint_every=ckpt)
    return outputs


def terminal_bwd(cfg, fwd, params, y0, cotangent, *, params_grad=True, y0_grad=True, stream=None):
    """The adjoint pass (``pdq_terminal_bwd``) for a cotangent (B, n, d) of
    the terminal mean of ``terminal_fwd``'s outputs ``fwd`` (same cfg,
    params and y0); returns (grad_params (B, P) or None, grad_y0 (B, d) or None)."""
    B = y0.shape[0]
    f64 = dict(dtype=torch.float64, device=y0.device)
    cot = cotangent.detach().to(dtype=torch.float64).contiguous()
    gp = torch.empty((B, params.shape[1]), **f64) if params_grad else None
    gy = torch.empty((B, y0.shape[1]), **f64) if y0_grad else None
    t = PdqTerminalAdjointArgs()
    t.num_instances = B
    t.capacity, t.checkpoint_every = fwd["_capacity"], fwd["_checkpoint_every"]
    t.params, t.y0 = _ptr(params), _ptr(y0)
    t.num_steps, t.status = _ptr(fwd["num_steps"]), _ptr(fwd["status"])
    t.cotangent, t.grad_params, t.grad_y0 = _ptr(cot), _ptr(gp), _ptr(gy)
    rec = fwd["_record"]
    check(load().pdq_terminal_bwd(ctypes.byref(cfg), ctypes.byref(t), _ptr(rec), ctypes.c_size_t(rec.numel()),
                                  _stream_handle(stream)), "pdq_terminal_bwd")
    return gp, gy


def workspace_size(cfg, B, S):
    ws = ctypes.c_size_t(0)
    check(load().pdq_workspace_size(ctypes.byref(cfg), B, S, ctypes.byref(ws)), "pdq_workspace_size")
    return int(ws.value)


def alloc_outputs(cfg, B, S, terminal_only, device, posterior=False, num_params=None):
    """Output tensors; ``posterior`` adds the smoother's conditionals and filtering
    marginals; ``num_params`` (isotropic) adds the mean records' sensitivities
    ``u_mean_d_params`` (B, S_out, n, d, P) and ``u_mean_d_y0`` (B, S_out, n, d, d)."""
    n = cfg.num_derivatives + 1
    d = cfg.ode_dim
    S_out = 1 if terminal_only else S
    f64 = dict(dtype=torch.float64, device=device)
    i32 = dict(dtype=torch.int32, device=device)
    extra = {}
    if cfg.ssm == SSM["dense"]:
        N = n * d
        mean_shape, chol_shape = (B, S_out, N), (B, S_out, N, N)
        if posterior:
            extra = {
                "cond_A": torch.empty((B, S - 1, N, N), **f64),
                "cond_noise_mean": torch.empty((B, S - 1, N), **f64),
                "cond_noise_chol": torch.empty((B, S - 1, N, N), **f64),
                "cond_to_latent": torch.empty((B, S - 1, N), **f64),
                "cond_to_observed": torch.empty((B, S - 1, N), **f64),
                "filter_mean": torch.empty((B, S, N), **f64),
                "filter_chol": torch.empty((B, S, N, N), **f64),
            }
    elif cfg.ssm == SSM["blockdiag"]:
        mean_shape, chol_shape = (B, S_out, d, n), (B, S_out, d, n, n)
        if posterior:
            extra = {
                "cond_A": torch.empty((B, S - 1, d, n, n), **f64),
                "cond_noise_mean": torch.empty((B, S - 1, d, n), **f64),
                "cond_noise_chol": torch.empty((B, S - 1, d, n, n), **f64),
                "cond_to_latent": torch.empty((B, S - 1, d, n), **f64),
                "cond_to_observed": torch.empty((B, S - 1, d, n), **f64),
                "filter_mean": torch.empty((B, S, d, n), **f64),
                "filter_chol": torch.empty((B, S, d, n, n), **f64),
            }
    else:
        mean_shape, chol_shape = (B, S_out, n, d), (B, S_out, n, n)
        if posterior:
            extra = {
                "cond_A": torch.empty((B, S - 1, n, n), **f64),
                "cond_noise_mean": torch.empty((B, S - 1, n, d), **f64),
                "cond_noise_chol": torch.empty((B, S - 1, n, n), **f64),
                "cond_to_latent": torch.empty((B, S - 1, n), **f64),
                "cond_to_observed": torch.empty((B, S - 1, n), **f64),
                "filter_mean": torch.empty((B, S, n, d), **f64),
                "filter_chol": torch.empty((B, S, n, n), **f64),
            }
    if num_params is not None:
        if cfg.ssm != SSM["isotropic"]:
            raise NotImplementedError("sensitivities: isotropic factorisation")
        extra["u_mean_d_params"] = torch.empty((B, S_out, n, d, int(num_params)), **f64)
        extra["u_mean_d_y0"] = torch.empty((B, S_out, n, d, d), **f64)
    return {
        **extra,
        "u_mean": torch.empty(mean_shape, **f64),
        "u_chol": torch.empty(chol_shape, **f64),
        "output_scale": torch.empty((B, S_out, d) if cfg.ssm == SSM["blockdiag"] else (B, S_out), **f64),
        "t": torch.empty((B, S_out), **f64),
        "num_steps": torch.empty((B, S_out), **i32),
        "num_attempts": torch.empty((B,), **i32),
        "status": torch.empty((B,), **i32),
    }


_LML_WORKSPACES = {}


def lml_fixed_grid(cfg, params, y0, data, std, *, t0, dt, num_steps, save_every, average_pdfs=False, gradient=True,
                   stream=None, workspace=None, outputs=None):
    """Call pdq_lml_fixed_grid on device tensors (float64, contiguous); returns (lml, grad, status)."""
    lib = load()
    B = y0.shape[0]
    P = params.shape[1]
    dev = y0.device
    if outputs is None:
        outputs = {
            "lml": torch.empty(B, dtype=torch.float64, device=dev),
            "grad": torch.empty((B, P), dtype=torch.float64, device=dev) if gradient else None,
            "status": torch.empty(B, dtype=torch.int32, device=dev),
        }
    nbytes = ctypes.c_size_t(0)
    check(lib.pdq_lml_workspace_size(ctypes.byref(cfg), B, num_steps, save_every, ctypes.byref(nbytes)), "pdq_lml_workspace_size")
    ws = workspace
    if ws is None:
        # one persistent workspace per device, stream and size: its leading covariance plan is
        # reused by later calls with the same grid (a freed block could be partly rewritten by
        # other tensors); calls on one stream are ordered, so they may share it
        key = (str(dev), _stream_handle(stream).value, int(nbytes.value))
        ws = _LML_WORKSPACES.get(key)
        if ws is None:
            ws = torch.zeros(max(1, nbytes.value), dtype=torch.uint8, device=dev)
            _LML_WORKSPACES[key] = ws
    elif ws.numel() * ws.element_size() < nbytes.value:
        raise ValueError("the LML workspace is smaller than pdq_lml_workspace_size")
    a = PdqLmlArgs()
    a.num_instances, a.num_steps, a.save_every = B, num_steps, save_every
    a.average_pdfs, a.with_gradient = int(bool(average_pdfs)), int(bool(gradient))
    a.t0, a.dt = float(t0), float(dt)
    a.params, a.y0, a.data, a.std = _ptr(params), _ptr(y0), _ptr(data), _ptr(std)
    a.lml, a.grad, a.status = _ptr(outputs["lml"]), _ptr(outputs.get("grad")), _ptr(outputs["status"])
    check(lib.pdq_lml_fixed_grid(ctypes.byref(cfg), ctypes.byref(a), _ptr(ws), ctypes.c_size_t(nbytes.value), _stream_handle(stream)),
          "pdq_lml_fixed_grid")
    outputs["_workspace"] = ws
    return outputs



def lml_adjoint_workspace_bytes(cfg, B, num_steps, save_every, checkpoint_every=0):
    """pdq_lml_adjoint_workspace_size: bytes of the plan plus the residuals of B samples."""
    lib = load()
    nbytes = ctypes.c_size_t(0)
    check(lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), B, num_steps, save_every, checkpoint_every,
                                             ctypes.byref(nbytes)), "pdq_lml_adjoint_workspace_size")
    return int(nbytes.value)


# Free adjoint workspaces per (device, stream, size).  A workspace holds the
# shared covariance plan (built on the device the first time, in
# milliseconds) followed by one call's residuals; a workspace whose backward
# call has been enqueued (lml_bwd(..., release=True)) may serve the next
# forward call on the same stream, which then reuses its plan.
_LML_ADJ_POOL = {}


def lml_fwd(cfg, params, y0, data, std, *, t0, dt, num_steps, save_every, average_pdfs=False, checkpoint_every=0,
            stream=None, workspace=None, outputs=None):
    """Call pdq_lml_fwd on device tensors (float64, contiguous).

    Returns a dict with ``lml`` (B,), ``status`` (B,) and the state that
    :func:`lml_bwd` needs (the argument struct and the workspace holding the
    plan and the residuals; keep it untouched until the backward call).
    Without ``workspace`` one is taken from the pool of released workspaces
    of this device, stream and size, or allocated.
    """
    lib = load()
    B = y0.shape[0]
    dev = y0.device
    if outputs is None:
        outputs = {
            "lml": torch.empty(B, dtype=torch.float64, device=dev),
            "status": torch.empty(B, dtype=torch.int32, device=dev),
        }
    nbytes = lml_adjoint_workspace_bytes(cfg, B, num_steps, save_every, checkpoint_every)
    ws = workspace
    pool_key = None
    if ws is None:
        pool_key = (str(dev), _stream_handle(stream).value, int(nbytes))
        free = _LML_ADJ_POOL.get(pool_key)
        ws = free.pop() if free else torch.zeros(max(1, nbytes), dtype=torch.uint8, device=dev)
    elif ws.numel() * ws.element_size() < nbytes:
        raise ValueError("the LML workspace is smaller than pdq_lml_adjoint_workspace_size")
    a = PdqLmlAdjointArgs()
    a.lml.num_instances, a.lml.num_steps, a.lml.save_every = B, num_steps, save_every
    a.lml.average_pdfs, a.lml.with_gradient = int(bool(average_pdfs)), 0
    a.lml.t0, a.lml.dt = float(t0), float(dt)
    a.lml.params, a.lml.y0, a.lml.data, a.lml.std = _ptr(params), _ptr(y0), _ptr(data), _ptr(std)
    a.lml.lml, a.lml.status = _ptr(outputs["lml"]), _ptr(outputs["status"])
    a.checkpoint_every = int(checkpoint_every)
    check(lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), _ptr(ws), ctypes.c_size_t(nbytes), _stream_handle(stream)),
          "pdq_lml_fwd")
    outputs["_workspace"] = ws
    # the inputs stay referenced: the backward call reads them again
    outputs["_saved"] = (cfg, a, nbytes, params, y0, data, std, stream)
    outputs["_pool_key"] = pool_key
    return outputs


def lml_release(fwd):
    """Return the workspace of :func:`lml_fwd`'s call ``fwd`` to the pool (its
    residuals are then no longer available to :func:`lml_bwd`).  Launches
    already enqueued on the call's stream still see them: a later forward
    call on that stream runs after them."""
    key = fwd.get("_pool_key")
    ws = fwd.pop("_workspace", None)
    fwd["_released"] = True
    if key is not None and ws is not None:
        _LML_ADJ_POOL.setdefault(key, []).append(ws)


def lml_bwd(fwd, cotangent=None, *, params_grad=True, y0_grad=False, outputs=None, release=False):
    """Call pdq_lml_bwd for the residuals of :func:`lml_fwd`'s call ``fwd``.

    cotangent: (B,) float64 device tensor (d loss / d lml) or None for ones.
    Returns ``{"grad": (B, P) or None, "grad_y0": (B, d) or None}``.
    ``release=True`` returns the workspace to the pool after enqueueing the
    launch (no further backward call on ``fwd``).
    """
    if fwd.get("_released"):
        raise RuntimeError("the residuals of this LML forward call were released after its backward call; "
                           "run the forward call again to differentiate it again")
    lib = load()
    cfg, a0, nbytes, params, y0, data, std, stream = fwd["_saved"]
    B, P, D = y0.shape[0], params.shape[1], y0.shape[1]
    if outputs is None:
        outputs = {
            "grad": torch.empty((B, P), dtype=torch.float64, device=y0.device) if params_grad else None,
            "grad_y0": torch.empty((B, D), dtype=torch.float64, device=y0.device) if y0_grad else None,
        }
    a = PdqLmlAdjointArgs.from_buffer_copy(a0)
    if cotangent is not None:
        cotangent = cotangent.detach().to(dtype=torch.float64).contiguous()
    a.cotangent = _ptr(cotangent)
    a.lml.grad = _ptr(outputs.get("grad"))
    a.grad_y0 = _ptr(outputs.get("grad_y0"))
    check(lib.pdq_lml_bwd(ctypes.byref(cfg), ctypes.byref(a), _ptr(fwd["_workspace"]), ctypes.c_size_t(nbytes),
                          _stream_handle(stream)), "pdq_lml_bwd")
    outputs["_cotangent"] = cotangent
    if release:
        lml_release(fwd)
    return outputs

def sample_markov(ssm, num_derivatives, ode_dim, marginal_mean, marginal_chol, posterior, normals, stream=None):
    """Call pdq_sample_markov on device float64 tensors; returns the samples tensor.

    marginal_*: the last point's marginal (B, ...); posterior: the fixed-point
    outputs ``cond_*`` (B, S - 1, ...); normals (B, K, S, n) isotropic or
    (B, K, S, N) dense.
    """
    B, K, S = normals.shape[0], normals.shape[1], normals.shape[2]
    n = num_derivatives + 1
    shape = (B, K, S, n, ode_dim) if ssm == "isotropic" else (B, K, S, n * ode_dim)
    samples = torch.empty(shape, dtype=torch.float64, device=normals.device)
    a = PdqSampleArgs()
    a.ssm, a.num_derivatives, a.ode_dim, a.num_points = SSM[ssm], num_derivatives, ode_dim, S
    a.num_instances, a.num_samples = B, K
    # keep the contiguous copies alive until the launch is enqueued
    marginal_mean, marginal_chol = marginal_mean.contiguous(), marginal_chol.contiguous()
    a.marginal_mean, a.marginal_chol = _ptr(marginal_mean), _ptr(marginal_chol)
    for k in ("cond_A", "cond_noise_mean", "cond_noise_chol", "cond_to_latent", "cond_to_observed"):
        setattr(a, k, _ptr(posterior[k]) if posterior is not None else None)
    a.normals, a.samples = _ptr(normals), _ptr(samples)
    check(load().pdq_sample_markov(ctypes.byref(a), _stream_handle(stream)), "pdq_sample_markov")
    return samples


OFFGRID_STRATEGY = {"filter": 0, "fixedinterval": 2}


def offgrid_marginals(ssm, strategy, num_derivatives, ode_dim, t, u_mean, u_chol, output_scale, t_query,
                      filter_mean=None, filter_chol=None, stream=None):
    """Call pdq_offgrid_marginals on device float64 tensors; returns (mean, chol) at the queries.

    t, output_scale: (B, S); u_*, filter_*: the grid marginals (B, S, ...);
    t_query: (B, Q).  ``strategy``: "filter" or "fixedinterval" (which needs
    the filtering marginals).
    """
    if strategy not in OFFGRID_STRATEGY:
        raise NotImplementedError(f"off-grid marginals are not defined for the {strategy} strategy")
    f64 = lambda x: None if x is None else x.to(torch.float64).contiguous()
    t, u_mean, u_chol, output_scale, t_query = map(f64, (t, u_mean, u_chol, output_scale, t_query))
    filter_mean, filter_chol = f64(filter_mean), f64(filter_chol)
    B, S = t.shape
    Q = t_query.shape[1]
    n = num_derivatives + 1
    if ssm == "isotropic":
        mshape, cshape = (B, Q, n, ode_dim), (B, Q, n, n)
    else:
        N = n * ode_dim
        mshape, cshape = (B, Q, N), (B, Q, N, N)
    mean = torch.empty(mshape, dtype=torch.float64, device=t.device)
    chol = torch.empty(cshape, dtype=torch.float64, device=t.device)
    a = PdqOffgridArgs()
    a.ssm, a.strategy, a.num_derivatives, a.ode_dim = SSM[ssm], OFFGRID_STRATEGY[strategy], num_derivatives, ode_dim
    a.num_instances, a.num_points, a.num_queries = B, S, Q
    a.t, a.u_mean, a.u_chol, a.output_scale, a.t_query = map(_ptr, (t, u_mean, u_chol, output_scale, t_query))
    a.filter_mean = _ptr(filter_mean) if filter_mean is not None else None
    a.filter_chol = _ptr(filter_chol) if filter_chol is not None else None
    a.mean_out, a.chol_out = _ptr(mean), _ptr(chol)
    check(load().pdq_offgrid_marginals(ctypes.byref(a), _stream_handle(stream)), "pdq_offgrid_marginals")
    return mean, chol
