"""Loader for the in-tree CUDA library (``lib/libpoyd_gb300.so``).

The library is the product: there is no CPU fallback.  ``lib()`` raises when
the library has not been built or cannot be loaded, and every wrapper raises
``PoydError`` when an entry point returns a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpoyd_gb300.so")

POYD_OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ERANGE", -4: "ENOMEM", -5: "EUNSUP", -6: "ESPACE"}
ESPACE = -6
DELTAW_DEFAULT, DELTAW_EXPLICIT, DELTAW_DOS_DISTANCE = 0, 1, 2
FLAG_DOS_EMPTY = 1
SANK_INF = 1 << 30


class PoydError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"poyd_gb300 error {ERRORS.get(code, code)}: {msg}")
        self.code = code


class PoydCM(C.Structure):
    """``poyd_cm`` (include/poyd_gb300.h)."""

    _fields_ = [
        ("lcm", C.c_int32), ("gap", C.c_int32), ("a_sz", C.c_int32),
        ("combinations", C.c_int32), ("cost_model", C.c_int32),
        ("gap_open", C.c_int32), ("is_metric", C.c_int32),
        ("all_elements", C.c_int32),
        ("cost", C.c_int32 * 1024), ("worst", C.c_int32 * 1024),
        ("prepend", C.c_int32 * 32), ("tail", C.c_int32 * 32),
        ("median", C.c_uint8 * 1024),
    ]


class PoydNodeStore(C.Structure):
    """``poyd_node_store`` (include/poyd_gb300.h): device node data of the
    level engine."""

    _fields_ = [
        ("pool", C.c_void_p), ("pool_size", C.c_int64),
        ("fitch", C.c_void_p), ("fitch_stride", C.c_int64), ("fitch_len", C.c_int32),
        ("sank_nchar", C.c_int32), ("sank", C.c_void_p), ("sank_tcm", C.c_void_p),
        ("sank_k", C.c_int32), ("pad", C.c_int32),
    ]


class PoydTuneResult(C.Structure):
    """``poyd_tune_result`` (include/poyd_gb300.h)."""

    _fields_ = [
        ("packed", C.c_int32), ("blocks_per_sm", C.c_int32), ("solo", C.c_int32),
        ("lg_pairs", C.c_int32), ("lg_width", C.c_int32), ("n_variants", C.c_int32),
        ("ms", C.c_float * 8), ("variant", (C.c_int32 * 3) * 8),
    ]


# Every entry point the public header declares (include/poyd_gb300.h);
# tests check the header's declarations against this list and that the
# library exports each of them.
EXPORTED = (
    "poyd_adam_step", "poyd_autotune_batch", "poyd_autotune_clear", "poyd_autotune_get",
    "poyd_autotune_set", "poyd_algn_align_2d", "poyd_algn_align_affine_3", "poyd_algn_ancestor_2",
    "poyd_algn_backtrack_2d", "poyd_algn_cost_affine_3", "poyd_algn_median_2_no_gaps",
    "poyd_algn_median_2_with_gaps", "poyd_algn_simple_2", "poyd_algn_verify_2",
    "poyd_algn_worst_2", "poyd_align_2_batch", "poyd_align_2_host", "poyd_ancestor_2_batch",
    "poyd_closest_batch", "poyd_cm_dna", "poyd_cm_median3", "poyd_cm_of_matrix5",
    "poyd_colsum_bf16",
    "poyd_cost_2_batch", "poyd_cost_2_batch_noalloc", "poyd_gemm_bf16", "poyd_int32_peak",
    "poyd_int_pipe_rate", "poyd_last_error", "poyd_launch_count", "poyd_matrix_create",
    "poyd_matrix_free", "poyd_median_2_no_gaps_batch", "poyd_median_2_with_gaps_batch",
    "poyd_median_levels",
    "poyd_mlp_forward", "poyd_mlp_head_backward", "poyd_mlp_head_forward", "poyd_nonadd16_distance_batch",
    "poyd_nonadd16_median_3_batch", "poyd_nonadd16_median_batch",
    "poyd_nonadd32_distance_batch", "poyd_nonadd32_median_3_batch",
    "poyd_nonadd32_median_batch", "poyd_nonadd8_distance_batch", "poyd_nonadd8_median_3_batch",
    "poyd_nonadd8_median_batch", "poyd_pack_alignments", "poyd_powell_3D_align",
    "poyd_powell_3d_batch", "poyd_profile_enable", "poyd_profile_read", "poyd_readjust_3d_batch",
    "poyd_relu_grad_bf16", "poyd_sank_distance_batch",
    "poyd_sank_median_3_batch", "poyd_sank_median_batch", "poyd_to_bf16", "poyd_verify_2_batch", "poyd_version",
    "poyd_workspace_release", "poyd_worst_2_batch",
)

# (name, restype, argtypes) of the entry points the Python mirror calls
# through typed ctypes signatures (a subset of EXPORTED; the others are set
# up where they are called).
_vp, _i32, _i64 = C.c_void_p, C.c_int32, C.c_int64
_cmp = C.POINTER(PoydCM)
SIGNATURES = [
    ("poyd_last_error", C.c_char_p, []),
    ("poyd_version", C.c_int, []),
    ("poyd_cm_dna", C.c_int, [_cmp, _i32, _i32, _i32]),
    ("poyd_cm_of_matrix5", C.c_int, [_cmp, _vp, _i32]),
    ("poyd_cost_2_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp]),
    ("poyd_align_2_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _i32, _vp]),
    ("poyd_median_levels", C.c_int, [_cmp, C.POINTER(PoydNodeStore), _i32, _vp, _vp, _i32, _vp,
                                     _vp, _vp, _vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     _vp, _vp]),
    ("poyd_autotune_batch", C.c_int, [_cmp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp,
                                      _vp, _vp, _i32, _i32, C.POINTER(PoydTuneResult), _vp]),
    ("poyd_autotune_set", C.c_int, [_i32] * 7),
    ("poyd_autotune_get", C.c_int, [_i32, _i32, _i32, _i32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("poyd_autotune_clear", C.c_int, []),
    ("poyd_profile_enable", C.c_int, [C.c_int]),
    ("poyd_profile_read", C.c_int, [C.c_char_p, C.POINTER(C.c_double), C.c_int]),
    ("poyd_launch_count", C.c_longlong, []),
    ("poyd_pack_alignments", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("poyd_align_2_host", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    C.c_int64, _vp, _vp, _i32]),
    ("poyd_algn_align_2d", C.c_int, [_vp, _i32, _vp, _i32, _cmp, _vp, _vp, _vp, _i32, _vp, _i32,
                                     _i32, _vp]),
    ("poyd_median_2_with_gaps_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                                _vp]),
    ("poyd_median_2_no_gaps_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("poyd_ancestor_2_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("poyd_worst_2_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("poyd_verify_2_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("poyd_algn_median_2_with_gaps", C.c_int, [_vp, _vp, _i32, _cmp, _vp, _vp]),
    ("poyd_algn_median_2_no_gaps", C.c_int, [_vp, _vp, _i32, _cmp, _vp, _vp]),
    ("poyd_algn_ancestor_2", C.c_int, [_vp, _vp, _i32, _cmp, _vp, _vp]),
    ("poyd_algn_worst_2", C.c_int, [_vp, _vp, _i32, _cmp, _vp]),
    ("poyd_algn_verify_2", C.c_int, [_vp, _vp, _i32, _cmp, _vp]),
    ("poyd_closest_batch", C.c_int, [_cmp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _i32, _vp]),
    ("poyd_cm_median3", C.c_int, [_cmp, _vp]),
    ("poyd_workspace_release", C.c_int, []),
    ("poyd_powell_3D_align", C.c_int, [_vp, _i32, _vp, _i32, _vp, _i32, _vp, _vp, _vp, _i32, _vp,
                                       _i32, _i32, _i32, _vp]),
    ("poyd_powell_3d_batch", C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32,
                                       _vp, _vp, _vp, _vp, _vp, _vp]),
    ("poyd_readjust_3d_batch", C.c_int, [_cmp, _i32] + [_vp] * 14 + [_vp]),
    ("poyd_int32_peak", C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("poyd_int_pipe_rate", C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
]


def profile_read(name=None, clear=True):
    """(total ms, launches) of recorded kernels named `name` (None = all)."""
    ms = C.c_double()
    n = lib().poyd_profile_read(name.encode() if name else None, C.byref(ms), 1 if clear else 0)
    return ms.value, n


def int32_peak():
    """Measured integer issue rate in Gop/s over both integer pipes (fused
    add-min on the ALU pipe interleaved with multiply-add adds on the FMA
    pipe): the denominator of the DP roofline."""
    g, ms = C.c_double(), C.c_double()
    check(lib().poyd_int32_peak(C.byref(g), C.byref(ms)))
    return g.value


def int_pipe_rate(mode):
    """Integer issue rate in Gop/s: 0 fused add-min (ALU pipe), 1 multiply-add
    adds (FMA pipe), 2 both interleaved."""
    g, ms = C.c_double(), C.c_double()
    check(lib().poyd_int_pipe_rate(int(mode), C.byref(g), C.byref(ms)))
    return g.value

_lib = None


def lib():
    """The loaded library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the GPU path has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != POYD_OK:
        msg = lib().poyd_last_error()
        raise PoydError(rc, msg.decode() if msg else "")
