"""ctypes binding of libgfe.so (the CUDA engine) with Iron-style error handling.

Every entry point returns an int status; a non-zero status raises GfeError carrying the
library's message, the way Iron's Python bindings raise CMFEError on a non-zero error code
(bindings/python/opencmiss/iron/_utils.in.py:27-78).  There is no CPU fallback: if the library
is missing or no GPU is present, calls fail loudly.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import torch

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgfe.so"

GFE_OK = 0
GFE_ERR = {
    -1: "GFE_ERR_ARG",
    -2: "GFE_ERR_CUDA",
    -3: "GFE_ERR_STRUCTURE",
    -4: "GFE_ERR_NUMERIC",
    -5: "GFE_ERR_NOCONV",
    -6: "GFE_ERR_TIMEOUT",
    -7: "GFE_ERR_NOMEM",
}
GFE_FP64 = 0
GFE_MIXED = 1

DEVERR_SLOT, DEVERR_JACOBIAN, DEVERR_NONFINITE, DEVERR_TIMEOUT = 1, 2, 4, 8


class GfeError(RuntimeError):
    """A libgfe call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.message = message
        super().__init__(f"{GFE_ERR.get(status, status)}: {message}")


_lock = threading.Lock()
_lib = None

# (name, restype, argtypes) of every exported entry point; kept in step with include/gfe.h
vp, i32, i64, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_double
SIGNATURES = {
    "gfe_version": (C.c_int, []),
    "gfe_clear_stale_error": (C.c_int, []),
    "gfe_release_scratch": (C.c_int, []),
    "gfe_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "gfe_device_errors": (C.c_int, [C.POINTER(C.c_uint32), vp]),
    "gfe_set_thread_error_word": (C.c_int, [vp]),
    "gfe_profile_enable": (C.c_int, [C.c_int]),
    "gfe_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int]),
    "gfe_probe_fma_rate": (C.c_int, [i32, C.POINTER(C.c_double), vp]),
    "gfe_ctx_create": (C.c_int, [vp, C.POINTER(vp)]),
    "gfe_ctx_destroy": (C.c_int, [vp]),
    "gfe_ctx_device_errors": (C.c_int, [vp, C.POINTER(C.c_uint32)]),
    "gfe_ctx_cached_meshes": (C.c_int, [vp, C.POINTER(C.c_int32)]),
    "gfe_mesh_create": (C.c_int, [vp, i32, i32, vp, i32, C.POINTER(vp)]),
    "gfe_mesh_create_regular": (C.c_int, [vp, i32, i32, i32, C.POINTER(vp)]),
    "gfe_mesh_destroy": (C.c_int, [vp]),
    "gfe_mesh_csr": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "gfe_assemble_laplace": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, i32]),
    "gfe_solve_laplace": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, f64, i32, i32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_double)]),
    "gfe_csr_structure": (C.c_int, [i32, i32, vp, i32, vp, vp, i64, C.POINTER(C.c_int64), vp]),
    "gfe_laplace_assemble": (C.c_int, [i32, i32, vp, vp, vp, vp, vp, i32, vp, vp, i64, vp, vp, vp, i32, vp]),
    "gfe_laplace_assemble_generalised": (C.c_int, [i32, i32, vp, vp, vp, vp, i32, vp, vp, i32, vp, vp, i64, vp, vp,
                                                   vp]),
    "gfe_laplace_element_matrices": (C.c_int, [i32, i32, vp, vp, vp, vp, i32, vp]),
    "gfe_laplace_assemble_regular": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp]),
    "gfe_laplace_regular_workspace_bytes": (C.c_int64, [i32, i32, i32, i32]),
    "gfe_laplace_assemble_regular_ws": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp, vp]),
    "gfe_laplace_assemble_regular_layers": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp, i32, i32, i32,
                                                      vp]),
    "gfe_laplace_assemble_regular_host": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp, i32,
                                                    vp]),
    "gfe_laplace_assemble_tp": (C.c_int, [vp, vp, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp, vp, C.c_int64, vp, vp,
                                          vp, vp, i32, vp]),
    "gfe_laplace_tp_slot_map": (C.c_int, [i32, i32, vp, vp, vp, C.c_int64, vp, vp]),
    "gfe_laplace_regular_check": (C.c_int, [i32, i32, i32, vp, vp, C.POINTER(C.c_int64), vp]),
    "gfe_mr_regular_structure": (C.c_int, [i32, i32, i32, vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
    "gfe_csr_spmv": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "gfe_solver_structure": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, C.c_int64, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int64), vp]),
    "gfe_solver_matrix": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "gfe_solver_rhs": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "gfe_solver_update_dependent": (C.c_int, [i32, vp, vp, vp, vp]),
    "gfe_mr_residual": (C.c_int, [i32, vp, vp, i32, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp]),
    "gfe_mr_slot_map": (C.c_int, [i32, vp, vp, i32, vp, vp, vp, vp, vp]),
    "gfe_mr_jacobian": (C.c_int, [i32, vp, vp, i32, i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, i64, vp, i32, vp]),
    "gfe_mr_tangent": (C.c_int, [i32, vp, vp, i32, i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, i64, vp, i32, vp]),
    "gfe_mr_jacobian_fd": (C.c_int, [i32, vp, vp, i32, i32, vp, vp, vp, i32, vp, vp, f64, vp, vp, i64, vp, vp]),
    "gfe_mr_residual_vjp": (C.c_int, [i32, vp, vp, i32, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp, vp]),
    "gfe_cg_solve": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, f64, i32, i32, C.POINTER(C.c_int32),
                               C.POINTER(C.c_double), vp]),
    "gfe_cg_solve_noalloc": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, f64, i32, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_double), vp]),
    "gfe_cg_workspace_bytes": (C.c_int64, [i32]),
    "gfe_cg_begin": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, f64, vp, vp]),
    "gfe_cg_steps": (C.c_int, [i32, vp, vp, vp, vp, vp, i32, vp, vp]),
    "gfe_cg_status": (C.c_int, [i32, vp, vp, vp]),
    "gfe_minres_solve": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, vp, f64, i32, i32, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_double), vp]),
    "gfe_minres_solve_nodal": (C.c_int, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, f64, i32, i32,
                                         C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_int32), vp]),
    "gfe_gmres_solve": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp, vp, f64, i32, i32, i32, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_double), vp]),
    "gfe_saddle_preconditioner": (C.c_int, [i32, i32, vp, vp, vp, vp, vp, vp]),
}


def load(path: Path | None = None):
    """Load libgfe.so (built by iron_gb300.build) and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise GfeError(-2, f"{p} is not built; run iron_gb300.build.build() (nvcc, sm_103a)")
        L = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def last_error() -> str:
    L = load()
    buf = C.create_string_buffer(2048)
    L.gfe_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != GFE_OK:
        raise GfeError(status, last_error())


# CUDA runtime errors that other code on a thread left behind before a library call, by
# (entry point, error code): cleared so that the entry point's launch check reports only its own
STALE_ERRORS: dict = {}


def call(name: str, *args) -> None:
    L = load()
    fn = getattr(L, name)
    stale = L.gfe_clear_stale_error()
    if stale:
        STALE_ERRORS[(name, stale)] = STALE_ERRORS.get((name, stale), 0) + 1
    check(fn(*args))


def ptr(t: torch.Tensor | None):
    """Device pointer of a CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise GfeError(-1, "expected a CUDA tensor")
    if not t.is_contiguous():
        raise GfeError(-1, "expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def host_ptr(t: torch.Tensor | None):
    """Address of a contiguous host tensor (None -> NULL)."""
    if t is None:
        return None
    if t.is_cuda:
        raise GfeError(-1, "expected a host tensor")
    if not t.is_contiguous():
        raise GfeError(-1, "expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def stream_handle(stream: torch.cuda.Stream | None = None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise GfeError(-2, "no CUDA device: the GB300 engine has no CPU path")
    load()
    return torch.device("cuda", torch.cuda.current_device())


STAGE_LAPLACE_ELEMENTS, STAGE_SPMV, STAGE_MR_RESIDUAL, STAGE_MR_JACOBIAN = 0, 1, 2, 3


def profile_enable(on: bool = True) -> None:
    load().gfe_profile_enable(1 if on else 0)


def profile_read(stage: int, reset: bool = True):
    """(device ms, launches) recorded for a stage since the last reset."""
    ms = C.c_double(0.0)
    n = C.c_int64(0)
    check(load().gfe_profile_read(stage, C.byref(ms), C.byref(n), 1 if reset else 0))
    return float(ms.value), int(n.value)


def probe_fma_rate(precision: int, stream=None) -> float:
    g = C.c_double(0.0)
    check(load().gfe_probe_fma_rate(precision, C.byref(g), stream_handle(stream)))
    return float(g.value)


def device_errors(stream=None) -> int:
    L = load()
    bits = C.c_uint32(0)
    check(L.gfe_device_errors(C.byref(bits), stream_handle(stream)))
    return int(bits.value)


def set_thread_error_word(word: torch.Tensor | None) -> None:
    """Route this thread's kernel error reports to `word` (a zeroed CUDA int32/uint32 scalar), or
    back to the library's per-device word with None."""
    check(load().gfe_set_thread_error_word(ptr(word) if word is not None else None))


def raise_device_errors(what: str, stream=None) -> None:
    bits = device_errors(stream)
    if bits:
        names = [n for b, n in ((DEVERR_SLOT, "missing CSR slot"), (DEVERR_JACOBIAN, "non-positive Jacobian"),
                                (DEVERR_NONFINITE, "non-finite value"), (DEVERR_TIMEOUT, "device wait timeout"))
                 if bits & b]
        raise GfeError(-4 if not bits & DEVERR_SLOT else -3, f"{what}: device reported {', '.join(names)}")
