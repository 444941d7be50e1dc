"""ctypes binding of ``libneb_gb300.so`` (the C ABI declared in include/neb_gb300.h).

The library is built in-tree by :mod:`neb_gb300.build`.  There is no fallback:
if the library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_size_t, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libneb_gb300.so"

NEB_OK = 0
NEB_ERR_ARG = -1
NEB_ERR_CUDA = -2
NEB_ERR_WORKSPACE = -3
NEB_ERR_NOT_PD = -4
NEB_ERR_NONFINITE = -5
NEB_ERR_SOLVER = -6
NEB_ERR_UNSUPPORTED = -7
NEB_ERR_TIMEOUT = -8

PREC = {"fp32": 0, "fp64": 1, "bf16x3": 2, "tf32": 3, "bf16x9": 4}
FEAT = {"periodic": 0, "multihole": 1, "raw3d": 2}
MAX_HIDDEN = 8


GRAM = {"plain": 0, "compensated": 1}


class NebNet(ctypes.Structure):
    _fields_ = [("dim", c_int32), ("n_hidden", c_int32),
                ("widths", c_int32 * (MAX_HIDDEN + 2)), ("precision", c_int32),
                ("gram", c_int32)]

    @classmethod
    def make(cls, dim: int, widths, precision: str, gram: str = "plain") -> "NebNet":
        widths = list(widths)
        n_hidden = len(widths) - 2
        if not 1 <= n_hidden <= MAX_HIDDEN:
            raise ValueError(f"need 1..{MAX_HIDDEN} hidden layers, got widths={widths}")
        if gram not in GRAM:
            raise ValueError(f"gram must be one of {tuple(GRAM)}")
        arr = (c_int32 * (MAX_HIDDEN + 2))(*(widths + [0] * (MAX_HIDDEN + 2 - len(widths))))
        return cls(dim, n_hidden, arr, PREC[precision], GRAM[gram])


class ModeNet(ctypes.Structure):
    """neb_modes: shape of a mode-stacked SIREN network."""
    _fields_ = [("dim", c_int32), ("order", c_int32), ("n_layers", c_int32),
                ("widths", c_int32 * (MAX_HIDDEN + 2)), ("n_modes", c_int32),
                ("precision", c_int32), ("omega_first", c_double), ("omega_hidden", c_double)]


_P = c_void_p
_PP = POINTER(c_void_p)

# name -> (restype, argtypes)
_SIGNATURES = {
    "neb_last_error": (ctypes.c_char_p, []),
    "neb_kernel_launches": (ctypes.c_ulonglong, []),
    "neb_timing_begin": (c_int, []),
    "neb_timing_end": (c_int, [c_int, ctypes.c_char_p, c_int, POINTER(c_int), POINTER(c_double),
                               POINTER(c_double), POINTER(c_double), POINTER(c_int)]),
    "neb_tape_bytes": (c_size_t, [POINTER(NebNet), c_int64]),
    "neb_workspace_bytes": (c_size_t, [POINTER(NebNet), c_int64]),
    "neb_features": (c_int, [POINTER(NebNet), c_int, c_int, POINTER(c_double), c_int, c_void_p,
                             c_int64, c_void_p, c_void_p]),
    "neb_forward": (c_int, [POINTER(NebNet), POINTER(c_void_p), POINTER(c_void_p), c_void_p,
                            c_int64, c_void_p, c_void_p, c_size_t, c_void_p]),
    "neb_output": (c_int, [POINTER(NebNet), c_void_p, c_void_p, c_int, c_int, c_int64, c_void_p,
                           c_void_p, c_void_p]),
    "neb_hidden_gram": (c_int, [POINTER(NebNet), c_void_p, c_int64, c_void_p, c_void_p, c_void_p,
                                c_int, c_void_p, c_size_t, c_void_p]),
    "neb_hidden_gram_static": (c_int, [POINTER(NebNet), c_void_p, c_int64, c_void_p, c_void_p,
                                       c_void_p, c_void_p]),
    "neb_fields_gram": (c_int, [POINTER(NebNet), c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "neb_spectral_workspace_bytes": (c_size_t, [c_int]),
    "neb_spectral": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "neb_spectral_range_workspace_bytes": (c_size_t, [c_int]),
    "neb_spectral_range": (c_int, [c_int, c_void_p, c_void_p, c_void_p, ctypes.c_double, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_int),
                                   c_void_p, c_void_p, c_size_t, c_void_p]),
    "neb_spectral_mixed_workspace_bytes": (c_size_t, [c_int]),
    "neb_spectral_mixed": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                   c_void_p]),
    "neb_pencil_workspace_bytes": (c_size_t, [c_int, c_int]),
    "neb_pencil_project": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_size_t, c_void_p]),
    "neb_pencil_pullback": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "neb_backward_hidden": (c_int, [POINTER(NebNet), POINTER(c_void_p), c_void_p, c_void_p,
                                    c_void_p, c_int64, c_void_p, POINTER(c_void_p),
                                    POINTER(c_void_p), c_int, c_void_p, c_size_t, c_void_p]),
    "neb_backward_output": (c_int, [POINTER(NebNet), POINTER(c_void_p), c_int, c_int, c_void_p,
                                    c_int64, c_void_p, POINTER(c_void_p), POINTER(c_void_p), c_int,
                                    c_void_p, c_size_t, c_void_p]),
    "neb_backward_fields": (c_int, [POINTER(NebNet), POINTER(c_void_p), c_void_p, c_void_p,
                                    c_void_p, c_int64, c_void_p, POINTER(c_void_p),
                                    POINTER(c_void_p), c_int, c_void_p, c_size_t, c_void_p]),
    "neb_check_status": (c_int, [POINTER(NebNet), c_int64, c_void_p, c_size_t, c_void_p]),
    "neb_adam_workspace_bytes": (c_size_t, []),
    "neb_adam": (c_int, [c_int, c_int, POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p),
                         POINTER(c_void_p), POINTER(c_int64), c_int, c_void_p, c_void_p, c_double,
                         c_double, c_double, c_double, c_double, c_void_p, c_void_p, c_void_p,
                         c_size_t, c_void_p]),
    "neb_wait_selftest": (c_int, [c_int, ctypes.c_uint32, c_void_p, c_void_p]),
    "neb_envelope_product": (c_int, [POINTER(NebNet), c_void_p, c_int64, c_int, c_void_p, c_void_p,
                                     c_int, c_void_p]),
    "neb_modes_tape_bytes": (c_size_t, [POINTER(ModeNet), c_int, c_int64]),
    "neb_modes_workspace_bytes": (c_size_t, [POINTER(ModeNet), c_int, c_int64]),
    "neb_modes_forward": (c_int, [POINTER(ModeNet), c_int, c_int, _PP, _PP, _P, _P, c_int64, _P,
                                  c_size_t, _P, _P]),
    "neb_modes_eval_scratch_bytes": (c_size_t, [POINTER(ModeNet), c_int, c_int64]),
    "neb_modes_forward_eval": (c_int, [POINTER(ModeNet), c_int, c_int, _PP, _PP, _P, _P, c_int64,
                                       _P, c_size_t, _P, _P]),
    "neb_modes_backward": (c_int, [POINTER(ModeNet), c_int, c_int, _PP, _P, _P, c_int64, _P, _P,
                                   _PP, _PP, c_int, _P, c_size_t, _P]),
    "neb_velocity_fields": (c_int, [c_int, _P, c_int, c_int, c_int64, c_int, _P, _P, _P]),
    "neb_velocity_lift": (c_int, [c_int, _P, _P, c_int, c_int, c_int64, c_int, _P, _P]),
    "neb_potential_fields": (c_int, [c_int, _P, c_int, c_int, c_int64, c_int, _P, _P, _P]),
    "neb_potential_lift": (c_int, [c_int, _P, _P, c_int, c_int, c_int64, c_int, _P, _P]),
    "neb_column_center": (c_int, [c_int, c_int64, c_int, _P, _P]),
    "neb_periodic_features": (c_int, [c_int, c_int, c_int, c_double, c_double, _P, c_int64, _P,
                                      _P]),
    "neb_stream_fields": (c_int, [c_int, c_int, _P, c_int, c_int, c_int64, c_int, _P, _P, _P, _P]),
    "neb_normalize_pencil": (c_int, [c_int, _P, _P, _P, _P]),
    "neb_ritz_transform": (c_int, [c_int, _P, _P, _P, _P]),
    "neb_etdrk4_coefficients": (c_int, [c_int, _P, c_double, c_double, _P, _P]),
    "neb_rollout_workspace_bytes": (c_size_t, [c_int64, c_int]),
    "neb_rollout_rhs": (c_int, [c_int, c_int64, c_int, _P, _P, _P, c_double, _P, _P, _P,
                                c_size_t, _P]),
    "neb_etdrk4_step": (c_int, [c_int, c_int64, c_int, _P, _P, _P, c_double, _P, _P, _P,
                                c_size_t, _P]),
    "neb_rollout_project": (c_int, [c_int, c_int64, c_int, _P, _P, _P, _P, c_double, _P, _P,
                                    c_size_t, _P]),
    "neb_rollout_fields": (c_int, [c_int, c_int64, c_int, _P, _P, _P, _P, _P, _P, c_size_t, _P]),
    "neb_modes_adam_workspace_bytes": (c_size_t, [c_int]),
    "neb_modes_adam": (c_int, [c_int, c_int, c_int, _PP, _PP, _PP, _PP, POINTER(c_int64), _P,
                               c_int, _P, _P, c_double, c_double, _P, _P, _P, c_size_t, _P]),
    "neb_column_gram_workspace_bytes": (c_size_t, [c_int64, c_int]),
    "neb_column_gram": (c_int, [c_int, c_int64, c_int, _P, c_double, c_int, _P, _P, c_size_t,
                                _P]),
    "neb_column_apply_workspace_bytes": (c_size_t, [c_int64, c_int]),
    "neb_column_apply": (c_int, [c_int, c_int64, c_int, _P, _P, c_double, _P, _P, c_size_t, _P]),
    "neb_peel_workspace_bytes": (c_size_t, [c_int]),
    "neb_coefficient_peel": (c_int, [c_int, _P, _P, c_double, c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                     c_size_t, _P]),
}

EXPORTED = tuple(_SIGNATURES)

_lib = None


def load(path: Path | str = LIB_PATH):
    """Load the library (once) and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(path)
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build it with `python -m neb_gb300.build` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().neb_last_error().decode(errors="replace")


def check(status: int, what: str) -> None:
    if status == NEB_OK:
        return
    msg = f"{what}: {last_error()} (status {status})"
    if status == NEB_ERR_ARG:
        raise ValueError(msg)
    if status in (NEB_ERR_NONFINITE, NEB_ERR_NOT_PD, NEB_ERR_SOLVER):
        raise FloatingPointError(msg)
    if status == NEB_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def kernel_launches() -> int:
    return int(load().neb_kernel_launches())


def timing_begin() -> None:
    call("neb_timing_begin")


def timing_end(max_kernels: int = 64) -> dict:
    """Per-kernel {name: (launches, total_ms, flops, bytes)} since timing_begin."""
    name_len = 64
    names = ctypes.create_string_buffer(max_kernels * name_len)
    launches = (c_int * max_kernels)()
    ms = (c_double * max_kernels)()
    fl = (c_double * max_kernels)()
    by = (c_double * max_kernels)()
    n = c_int(0)
    call("neb_timing_end", max_kernels, names, name_len, launches, ms, fl, by, ctypes.byref(n))
    out = {}
    for k in range(n.value):
        name = names.raw[k * name_len:(k + 1) * name_len].split(b"\0", 1)[0].decode()
        out[name] = (launches[k], ms[k], fl[k], by[k])
    return out


def ptr_array(tensors) -> ctypes.Array:
    """Host array of device pointers (None -> NULL)."""
    return (c_void_p * len(tensors))(*[0 if t is None else t.data_ptr() for t in tensors])
