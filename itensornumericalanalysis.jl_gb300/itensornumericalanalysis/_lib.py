"""ctypes binding of libtnfa (include/tnfa.h).

The library is loaded from ``_lib/libtnfa.so`` inside this package.  There is
no fallback: if the library is missing or no CUDA device is visible, every
compute call raises :class:`TnfaError`.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libtnfa.so"

# tnfa_status
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_TOPOLOGY = 4
ERR_SHAPE = 5
ERR_DTYPE = 6
ERR_NOT_CONVERGED = 7
ERR_TIMEOUT = 8
ERR_DOMAIN = 9
ERR_UNSUPPORTED = 10
STATUS_NAMES = {
    0: "TNFA_OK",
    1: "TNFA_ERR_INVALID_ARGUMENT",
    2: "TNFA_ERR_CUDA",
    3: "TNFA_ERR_OUT_OF_MEMORY",
    4: "TNFA_ERR_TOPOLOGY",
    5: "TNFA_ERR_SHAPE",
    6: "TNFA_ERR_DTYPE",
    7: "TNFA_ERR_NOT_CONVERGED",
    8: "TNFA_ERR_TIMEOUT",
    9: "TNFA_ERR_DOMAIN",
    10: "TNFA_ERR_UNSUPPORTED",
}
# tnfa_dtype
F64, F32, C128 = 0, 1, 2
# tnfa_memory
MEM_HOST, MEM_DEVICE = 0, 1
# tnfa_precision
PREC_F64, PREC_F32, PREC_MIXED, PREC_MIXED_FAST = 0, 1, 2, 3
# tnfa_leg_kind
LEG_REAL, LEG_IMAG, LEG_OPERATOR = 0, 1, 2
# tnfa_out
OUT_F64, OUT_F32, OUT_F32_SCALED, OUT_C128 = 0, 1, 2, 3


class TnfaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Topology(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32),
        ("parent", C.POINTER(C.c_int32)),
        ("link_dim", C.POINTER(C.c_int32)),
        ("n_legs", C.POINTER(C.c_int32)),
        ("leg_dim", C.POINTER(C.c_int32)),
        ("leg_var", C.POINTER(C.c_int32)),
        ("leg_digit", C.POINTER(C.c_int32)),
        ("leg_kind", C.POINTER(C.c_int32)),
    ]


class TruncParams(C.Structure):
    _fields_ = [
        ("cutoff", C.c_double),
        ("maxdim", C.c_int32),
        ("mindim", C.c_int32),
        ("normalize", C.c_int32),
        ("precision", C.c_int32),
    ]


class DmrgParams(C.Structure):
    _fields_ = [
        ("nsweeps", C.c_int32),
        ("maxdim", C.c_int32),
        ("cutoff", C.c_double),
        ("tol", C.c_double),
        ("krylov_dim", C.c_int32),
        ("restarts", C.c_int32),
    ]


class LinsolveParams(C.Structure):
    _fields_ = [
        ("nsweeps", C.c_int32),
        ("maxdim", C.c_int32),
        ("cutoff", C.c_double),
        ("tol", C.c_double),
        ("krylov_dim", C.c_int32),
        ("precision", C.c_int32),
        ("a0", C.c_double),
        ("a1", C.c_double),
        ("refinements", C.c_int32),
        ("refine_cutoff", C.c_double),
    ]


BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2

_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I32 = C.c_int32
_I64 = C.c_int64
_PI32 = C.POINTER(C.c_int32)
_PD = C.POINTER(C.c_double)

# name -> (restype, argtypes); the complete ABI of include/tnfa.h
SIGNATURES = {
    "tnfa_version": (C.c_char_p, []),
    "tnfa_ctx_create": (C.c_int, [C.c_int, _P, _PP]),
    "tnfa_ctx_destroy": (C.c_int, [_P]),
    "tnfa_ctx_synchronize": (C.c_int, [_P]),
    "tnfa_ctx_set_wait_budget": (C.c_int, [_P, C.c_uint32, C.c_int]),
    "tnfa_ctx_inject_faults": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "tnfa_last_error_string": (C.c_char_p, [_P]),
    "tnfa_ctx_set_timing": (C.c_int, [_P, C.c_int]),
    "tnfa_ctx_set_autotune": (C.c_int, [_P, C.c_int, C.c_double, C.c_int]),
    "tnfa_ctx_tuning_report": (C.c_int, [_P, C.c_char_p, _I64, C.POINTER(_I64)]),
    "tnfa_ctx_kernel_stats": (
        C.c_int,
        [_P, _I32, C.c_char_p, C.POINTER(_I64), _PD, _PD, _PD, _PI32, C.c_int],
    ),
    "tnfa_net_create": (C.c_int, [_P, C.POINTER(Topology), C.c_int, _P, C.c_int, _PP]),
    "tnfa_net_destroy": (C.c_int, [_P]),
    "tnfa_net_info": (C.c_int, [_P, _PI32, _PI32, C.POINTER(_I64), _PI32]),
    "tnfa_net_download": (C.c_int, [_P, _P, _P, C.c_int]),
    "tnfa_net_copy": (C.c_int, [_P, _P, _PP]),
    "tnfa_net_scale": (C.c_int, [_P, _P, _I32, C.c_double, C.c_double]),
    "tnfa_net_topology": (
        C.c_int,
        [_P, _PI32, _PI32, _PI32, _PI32, _PI32, _PI32, _PI32, _PI32],
    ),
    "tnfa_net_concat": (C.c_int, [_P, _P, _P, _PP]),
    "tnfa_net_gather": (C.c_int, [_P, _P, C.POINTER(Topology), _PI32, C.POINTER(C.c_int64), _PP]),
    "tnfa_net_convert": (C.c_int, [_P, _P, C.c_int, _PP]),
    "tnfa_evaluate": (
        C.c_int,
        [_P, _P, _P, _I64, _I32, _PI32, C.c_int, _P, C.c_int, C.c_int, C.c_int],
    ),
    "tnfa_evaluate_noalloc": (
        C.c_int,
        [_P, _P, _P, _I64, _I32, _PI32, _P, C.c_int, C.c_int],
    ),
    "tnfa_eval_plan_create": (
        C.c_int,
        [_P, _P, _P, _I64, _I32, _PI32, _P, C.c_int, C.c_int, _PP],
    ),
    "tnfa_eval_plan_launch": (C.c_int, [_P, _P]),
    "tnfa_eval_plan_check": (C.c_int, [_P, _P]),
    "tnfa_eval_plan_destroy": (C.c_int, [_P]),
    "tnfa_integrate": (C.c_int, [_P, _P, C.c_int, _PD]),
    "tnfa_integrate_operator": (C.c_int, [_P, _P, _P, C.c_int, _PD]),
    "tnfa_partial_integrate": (C.c_int, [_P, _P, _I32, _PI32, C.c_int, C.c_int, _PI32, _PP, _PI32]),
    "tnfa_add": (C.c_int, [_P, _P, _P, _PP]),
    "tnfa_multiply": (C.c_int, [_P, _P, _P, _PP]),
    "tnfa_operator_proj": (C.c_int, [_P, _P, _PP]),
    "tnfa_cross": (C.c_int, [_P, _P, C.c_int, _I32, _I32, C.c_double, _I32, _PI32, _PI32, _PI32, _PD]),
    "tnfa_op_stencil_terms": (
        C.c_int,
        [C.POINTER(Topology), _I32, _PD, _I32, _I32, _I32, _I32, _PD, _PI32, _PI32, _PD, _PI32, _PI32],
    ),
    "tnfa_op_from_terms": (
        C.c_int,
        [_P, C.POINTER(Topology), _I32, _PD, _PI32, _PI32, _PD, C.c_double, _PP],
    ),
    "tnfa_op_build_stencil": (
        C.c_int,
        [_P, C.POINTER(Topology), _I32, _PD, _I32, _I32, _I32, _I32, C.c_double, _PP],
    ),
    "tnfa_apply": (C.c_int, [_P, _P, _P, C.POINTER(TruncParams), _PP]),
    "tnfa_apply_batched": (C.c_int, [_P, _I32, _PP, _PP, C.POINTER(TruncParams), _PP]),
    "tnfa_apply_exact": (C.c_int, [_P, _P, _P, _PP]),
    "tnfa_apply_vjp": (C.c_int, [_P, _P, _P, _P, C.c_int, _P, C.c_int]),
    "tnfa_truncate": (C.c_int, [_P, _P, C.POINTER(TruncParams), _PP]),
    "tnfa_truncate_batched": (C.c_int, [_P, _I32, _PP, C.POINTER(TruncParams), _PP]),
    "tnfa_inner": (C.c_int, [_P, _P, _P, _PD]),
    "tnfa_linsolve": (C.c_int, [_P, _P, _P, _P, C.POINTER(LinsolveParams), _PP, _PD]),
    "tnfa_dmrg": (C.c_int, [_P, _P, _P, C.POINTER(DmrgParams), _PP, _PD]),
    "tnfa_evaluate_vjp": (
        C.c_int,
        [_P, _P, _P, _I64, _I32, _PI32, C.c_int, _P, C.c_int, _P, C.c_int],
    ),
}

_lib = None
_lib_lock = threading.Lock()


def load() -> C.CDLL:
    """Load libtnfa.so (once) and declare every signature."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise TnfaError(
                    ERR_UNSUPPORTED,
                    f"{LIB_PATH} is missing: build it with "
                    "itensornumericalanalysis._build.build() (needs nvcc)",
                )
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


class Context:
    """A libtnfa context bound to one device and one stream."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.tnfa_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h))
        if st != OK:
            raise TnfaError(st, f"tnfa_ctx_create(device={device}) failed (no CUDA device?)")
        self.handle = h
        self.device = device

    def check(self, status: int) -> None:
        if status != OK:
            msg = self.lib.tnfa_last_error_string(self.handle)
            raise TnfaError(status, msg.decode() if msg else "")

    def call(self, name: str, *args) -> None:
        self.check(getattr(self.lib, name)(self.handle, *args))

    def set_timing(self, enable: bool) -> None:
        self.check(self.lib.tnfa_ctx_set_timing(self.handle, int(enable)))

    def set_autotune(self, enable: bool | None = None, min_work: float | None = None,
                     forget: bool = False) -> None:
        """Autotuning of launch variants (tnfa_ctx_set_autotune); None keeps a setting."""
        self.check(self.lib.tnfa_ctx_set_autotune(
            self.handle, -1 if enable is None else int(enable),
            -1.0 if min_work is None else float(min_work), int(forget)))

    def tuning_report(self) -> dict:
        """shape key -> (kept variant, [ms of each variant when timed])."""
        need = _I64()
        self.check(self.lib.tnfa_ctx_tuning_report(self.handle, None, 0, C.byref(need)))
        buf = C.create_string_buffer(int(need.value))
        self.check(self.lib.tnfa_ctx_tuning_report(self.handle, buf, need.value, C.byref(need)))
        out = {}
        for line in buf.value.decode().splitlines():
            parts = line.split()
            out[parts[0]] = (int(parts[1]), [float(x) for x in parts[2:]])
        return out

    def kernel_stats(self, reset: bool = False) -> dict:
        """family -> {launches, ms, flops, bytes} since the last reset."""
        m = 64
        names = C.create_string_buffer(32 * m)
        la = (_I64 * m)()
        ms, fl, by = (C.c_double * m)(), (C.c_double * m)(), (C.c_double * m)()
        n = C.c_int32()
        self.check(self.lib.tnfa_ctx_kernel_stats(self.handle, m, names, la, ms, fl, by,
                                                  C.byref(n), int(reset)))
        out = {}
        for i in range(min(n.value, m)):
            nm = names.raw[32 * i : 32 * i + 32].split(b"\0")[0].decode()
            out[nm] = {"launches": la[i], "ms": ms[i], "flops": fl[i], "bytes": by[i]}
        return out

    def set_wait_budget(self, polls: int = 0, drop_arrive: bool = False) -> None:
        """tnfa_ctx_set_wait_budget: try_wait polls before a tensor-core
        pipeline wait gives up (0 keeps the budget), and the test switch that
        withholds one arrive so that a wait runs out."""
        self.check(self.lib.tnfa_ctx_set_wait_budget(self.handle, int(polls), int(drop_arrive)))

    def inject_faults(self, fail_alloc_after: int = -1, jacobi_sweep_cap: int = 0) -> None:
        """tnfa_ctx_inject_faults: fail the device allocation after the next
        `fail_alloc_after` ones (-1: never); cap Jacobi sweeps (0: off)."""
        self.check(self.lib.tnfa_ctx_inject_faults(self.handle, int(fail_alloc_after),
                                                   int(jacobi_sweep_cap)))

    def synchronize(self) -> None:
        self.call("tnfa_ctx_synchronize")

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.tnfa_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None
_ctx_lock = threading.Lock()


def default_context() -> Context:
    """The process-wide context on device $TNFA_DEVICE (default 0)."""
    global _default_ctx
    with _ctx_lock:
        if _default_ctx is None:
            _default_ctx = Context(int(os.environ.get("TNFA_DEVICE", "0")))
    return _default_ctx


def set_default_context(ctx: Context | None) -> None:
    global _default_ctx
    with _ctx_lock:
        _default_ctx = ctx
