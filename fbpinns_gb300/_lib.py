"""ctypes binding of ``libfbpgpu.so`` (the C ABI declared in include/fbpgpu.h).

The library is required: importing the engine without it raises
``FBPLibraryError`` and nothing falls back to a CPU or PyTorch path.
"""

import ctypes as C
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfbpgpu.so")

FBP_OK = 0
STATUS_BITS = {
    1: "pair overflow (more point-subdomain pairs than the pair capacity)",
    2: "slot overflow (more (point, level) slots than capacity)",
    4: "work-item overflow",
    8: "a point's POU levels are not in ascending subdomain order",
    16: "index out of range",
    32: "tensor-core kernel timed out waiting for its MMAs",
}

PROBLEM_NONE, PROBLEM_HO_HARDBC, PROBLEM_BURGERS, PROBLEM_POISSON2D, PROBLEM_WAVE_C, PROBLEM_HELMHOLTZ2D = range(6)
D2_LAPLACIAN = 8  # FBP_D2_LAPLACIAN: one jet slot for the sum of the masked second derivatives


def D2_GROUP(dims):
    """FBP_D2_GROUP: the masked dims in ``dims`` share one jet slot (their sum)."""
    return (int(dims) & 7) << 4


def d2_group(d2):
    """Dims summed into the group's jet slot of a d2mask (0: no group)."""
    return (d2 & 7) if d2 & D2_LAPLACIAN else ((d2 >> 4) & 7 & d2)
# FBP_ACT_*: hidden-layer activation of the compiled networks, and the number of
# trainable activation parameters per neuron that each layer adds to W, b
ACT_TANH, ACT_SIN, ACT_ADAPTIVE_TANH, ACT_ADAPTIVE_SIN, ACT_FOURIER = 0, 1, 2, 3, 4
ACTIVATIONS = {"tanh": ACT_TANH, "sin": ACT_SIN, "adaptive_tanh": ACT_ADAPTIVE_TANH, "adaptive_sin": ACT_ADAPTIVE_SIN,
               "fourier": ACT_FOURIER}
ACT_EXTRA = {"tanh": 0, "sin": 0, "adaptive_tanh": 1, "adaptive_sin": 2, "fourier": 0}
# FBP_WINDOW_*: the subdomain window (fbpinns/windows.py)
WINDOW_COSINE, WINDOW_SIGMOID, WINDOW_BUMP, WINDOW_WENDLAND, WINDOW_RBF = range(5)


class FBPLibraryError(RuntimeError):
    pass


class Boxes(C.Structure):
    _fields_ = [("xmins", C.c_void_p), ("xmaxs", C.c_void_p), ("pou", C.c_void_p), ("select", C.c_void_p),
                ("m", C.c_int64), ("xd", C.c_int32), ("ncell", C.c_int32 * 3), ("lo", C.c_double * 3),
                ("inv_h", C.c_double * 3), ("cell_start", C.c_void_p), ("cell_boxes", C.c_void_p)]


class Net(C.Structure):
    _fields_ = [("xd", C.c_int32), ("h1", C.c_int32), ("h2", C.c_int32), ("ud", C.c_int32), ("d2mask", C.c_int32),
                ("nparam", C.c_int32), ("act", C.c_int32), ("theta", C.c_void_p), ("xmins", C.c_void_p), ("xmaxs", C.c_void_p),
                ("flags", C.c_void_p), ("unnorms", C.c_void_p), ("m", C.c_int64), ("window", C.c_int32),
                ("wmins", C.c_void_p), ("wmaxs", C.c_void_p)]


class Pairs(C.Structure):
    _fields_ = [("sd_start", C.c_void_p), ("sd_rec", C.c_void_p),
                ("items", C.c_void_p), ("n_items", C.c_void_p), ("items_cap", C.c_int64), ("slots_cap", C.c_int64),
                ("item_ctr", C.c_void_p), ("zs", C.c_void_p), ("zs_cap", C.c_int64)]


class Problem(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_int", C.c_int32), ("p", C.c_float * 8), ("gauss", C.c_void_p),
                ("ng", C.c_int32), ("pt_keep", C.c_void_p), ("n_keep", C.c_void_p)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_SIG = {
    "fbp_abi_version": (C.c_int, []),
    "fbp_last_error": (C.c_char_p, []),
    "fbp_scan_scratch_bytes": (C.c_size_t, [_I64]),
    "fbp_scan_i32": (C.c_int, [_P, _P, _I64, _P, C.c_size_t, _P]),
    "fbp_scan_i32_noalloc": (C.c_int, [_P, _P, _I64, _P]),
    "fbp_inside_count": (C.c_int, [_P, _I64, C.POINTER(Boxes), _P, _P, _P, _P, _P, _P, _P]),
    "fbp_inside_fill": (C.c_int, [_P, _I64, C.POINTER(Boxes), _P, _P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P, _P]),
    "fbp_gather_i32": (C.c_int, [_P, _I64, _P, _P, _P, _P]),
    "fbp_compact_scratch_bytes": (C.c_size_t, [_I64]),
    "fbp_compact_flags": (C.c_int, [_P, _I64, _P, _P, _P, C.c_size_t, _P]),
    "fbp_sort_scratch_bytes": (C.c_size_t, [_I64, _I64]),
    "fbp_sort_pairs": (C.c_int, [_P, _P, _P, _P, _I64, _I64, _P, _P, _P, C.c_size_t, _P]),
    "fbp_sort_pairs_kept": (C.c_int, [_P, _P, _P, _P, _P, _I64, _I64, _P, _P, _P, C.c_size_t, _P]),
    "fbp_train_mask": (C.c_int, [_P, _P, _I64, _I64, _P, _I64, _P, _P, _P, _P, _P]),
    "fbp_work_scratch_bytes": (C.c_size_t, [_I64]),
    "fbp_build_work": (C.c_int, [_P, _I64, _P, _I32, _P, _P, _P, _I64, _P, _P, C.c_size_t, _P]),
    "fbp_forward_pairs": (C.c_int, [C.POINTER(Net), _P, C.POINTER(Pairs), _P, _I32, _P]),
    "fbp_forward_pairs_tc": (C.c_int, [C.POINTER(Net), _P, C.POINTER(Pairs), _P, _P, _I32, _P]),
    "fbp_pou_forward": (C.c_int, [_I32, _I32, _I64, _I32, _P, _P, _P, _P, _P, _I64, _I64, _P, _P]),
    "fbp_pou_backward": (C.c_int, [_I32, _I32, _I64, _I32, _P, _P, _P, _I64, _P]),
    "fbp_pou_loss": (C.c_int, [_I32, _I32, C.POINTER(Problem), _I64, _I32, _P, _P, _P, _P, _P, _P, _P, _I64, _I64,
                               _P, _I32, _P, _P]),
    "fbp_loss_finalize": (C.c_int, [_P, _I32, C.c_double, _P, _P]),
    "fbp_adjoint_pairs": (C.c_int, [C.POINTER(Net), _P, C.POINTER(Pairs), _P, _P, _I32, _P]),
    "fbp_adjoint_pairs_tc": (C.c_int, [C.POINTER(Net), _P, C.POINTER(Pairs), _P, _P, _P, _I32, _P]),
    "fbp_has_tc_adjoint_shape": (C.c_int, [_I32, _I32, _I32, _I32, _I32]),
    "fbp_grad_reduce": (C.c_int, [_P, _P, _I64, _I32, _P, _P]),
    "fbp_adam": (C.c_int, [_P, _P, _P, _P, _P, _I64, _I32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                           _P, _P]),
    "fbp_sample_uniform": (C.c_int, [_P, _I64, _I32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_uint64,
                                     C.c_uint64, _P, _P]),
    "fbp_sort_points_scratch_bytes": (C.c_size_t, [_I64, _I32]),
    "fbp_sort_points_cells": (C.c_int, [_P, _I64, _I32, C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P,
                                        C.c_size_t, _P]),
    "fbp_graph_instantiate": (C.c_int, [_P, _I32, C.POINTER(C.c_void_p)]),
    "fbp_graph_launch": (C.c_int, [_P, _P]),
    "fbp_graph_exec_destroy": (C.c_int, [_P]),
    "fbp_fma_probe": (C.c_int, [_P, _I32, _I32, C.POINTER(C.c_double), _P]),
    "fbp_tanh_probe": (C.c_int, [_P, _P, _I64, _P]),
    "fbp_has_shape": (C.c_int, [_I32, _I32, _I32, _I32, _I32]),
    "fbp_has_tc_shape": (C.c_int, [_I32, _I32, _I32, _I32, _I32]),
}

_lib = None


def declared_symbols():
    """Entry points declared in include/fbpgpu.h (parsed from the header)."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "fbpgpu.h")
    with open(hdr) as f:
        txt = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\*?\s+\*?(fbp_[a-z_0-9]+)\s*\(", txt, re.M)))


def load(build_if_missing=True):
    """Load (building it first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise FBPLibraryError(f"libfbpgpu.so not found at {LIB_PATH}: run `python -m fbpinns_gb300.build`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIG.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != FBP_OK:
        msg = load().fbp_last_error().decode(errors="replace")
        raise FBPLibraryError(f"{what or 'libfbpgpu'} failed (status {rc}): {msg}")


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return C.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def decode_status(word):
    msgs = [m for b, m in STATUS_BITS.items() if word & b]
    return "; ".join(msgs)
