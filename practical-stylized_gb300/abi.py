"""ctypes mirror of include/sty_gb300.h and the loader of libsty_gb300.so.

Structures here must stay byte-identical to the C header; tests check sizes against the
header's layout. Every wrapped call raises StyError on a non-zero status with the library's
own message (sty_last_error).
"""
from __future__ import annotations

import ctypes as C
import pathlib
from typing import Sequence

PKG_DIR = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libsty_gb300.so"

STY_OK = 0
STY_ERR_ARG = 1
STY_ERR_OOM = 2
STY_ERR_CUDA = 3
STY_ERR_ITER_LIMIT = 4
STY_ERR_NAN = 5
STY_ERR_UNSUPPORTED = 6

STY_STYLE_NONE = 0
STY_STYLE_TOON = 1
STY_STYLE_PALETTE = 2
STY_STYLE_SAT_ADJUST = 3
STY_STYLE_SAT_REX = 4
STY_STYLE_EIGHT_BIT = 5
STY_STYLE_TOON_STEPS = 7
STY_STYLE_RAMP_SMOOTH = 8
STY_STYLE_HALF_TONE = 9
STY_STYLE_MAX_NODES = 4
STY_STYLE_MAX_PARAMS = 60


STY_DEV_WAIT_TIMEOUT = 1


def device_status(clear: bool = True) -> int:
    """Read (and by default clear) the device status word of the current device."""
    v = C.c_uint32(0)
    check(lib().sty_device_status(C.byref(v), 1 if clear else 0))
    return v.value


class StyError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{status_name(status)}: {msg}")
        self.status = status


_NAMES = {0: "STY_OK", 1: "STY_ERR_ARG", 2: "STY_ERR_OOM", 3: "STY_ERR_CUDA",
          4: "STY_ERR_ITER_LIMIT", 5: "STY_ERR_NAN", 6: "STY_ERR_UNSUPPORTED"}


def status_name(s: int) -> str:
    return _NAMES.get(s, f"STY_ERR_{s}")


class StyleNode(C.Structure):
    _fields_ = [("kind", C.c_int32), ("depth_mask", C.c_uint32), ("n", C.c_int32),
                ("reserved", C.c_int32), ("p", C.c_float * STY_STYLE_MAX_PARAMS)]


class StyleProgram(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("reserved", C.c_int32 * 3),
                ("nodes", StyleNode * STY_STYLE_MAX_NODES)]


class PfRecords(C.Structure):
    _fields_ = [("pos", C.c_void_p * 3), ("nrm", C.c_void_p * 3), ("rad", C.c_void_p * 3),
                ("thr", C.c_void_p * 3), ("valid", C.c_void_p),
                ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("depths", C.c_int32)]


class PfScreenParams(C.Structure):
    _fields_ = [("radius", C.c_int32), ("sigma_pixel", C.c_float), ("sigma_pos", C.c_float),
                ("sigma_nrm", C.c_float)]


class Pcg32(C.Structure):
    _fields_ = [("state", C.c_uint64), ("inc", C.c_uint64)]


# (name, restype, argtypes) of every exported entry point declared in include/sty_gb300.h
_VP = C.c_void_p
SIGNATURES = {
    "sty_version": (C.c_int32, []),
    "sty_status_string": (C.c_char_p, [C.c_int32]),
    "sty_last_error": (C.c_char_p, []),
    "sty_launch_count": (C.c_uint64, []),
    "sty_struct_size": (C.c_uint64, [C.c_char_p]),
    "sty_wait_timeout_probe": (C.c_int32, [C.c_uint32, _VP]),
    "sty_device_status": (C.c_int32, [C.POINTER(C.c_uint32), C.c_int32]),
    "sty_style_apply": (C.c_int32, [C.POINTER(StyleProgram), C.c_uint32, _VP, _VP, C.c_uint64, _VP]),
    "sty_style_apply_at": (C.c_int32, [C.POINTER(StyleProgram), C.c_uint32, _VP, _VP, _VP, C.c_uint64, _VP]),
    "sty_pf_screen_filter_depth": (C.c_int32, [C.POINTER(PfRecords), C.c_uint32, C.POINTER(PfScreenParams),
                                               C.POINTER(StyleProgram), _VP, _VP, _VP, _VP]),
    "sty_pf_screen_filter": (C.c_int32, [C.POINTER(PfRecords), C.POINTER(PfScreenParams),
                                         C.POINTER(StyleProgram), _VP, _VP]),
    "sty_pf_screen_set_kernel": (C.c_int32, [C.c_int32]),
    "sty_film_accumulate": (C.c_int32, [_VP, C.c_int32, C.c_int32, C.c_int32, C.c_double, _VP, _VP]),
    "sty_pf_ref_create": (C.c_int32, [C.c_uint64, C.c_uint32, C.POINTER(C.c_void_p)]),
    "sty_pf_ref_destroy": (C.c_int32, [C.c_void_p]),
    "sty_pf_ref_filter": (C.c_int32, [C.c_void_p, _VP, _VP, _VP, _VP, C.c_uint32, _VP, C.c_uint32, _VP, _VP,
                                      _VP, _VP, _VP]),
    "sty_pf_adjoint": (C.c_int32, [C.POINTER(PfRecords), C.c_uint32, C.c_int32, C.POINTER(C.c_float * 36),
                                   C.c_uint32, _VP, _VP, _VP, C.POINTER(C.c_float), _VP]),
    "sty_pf_adjoint_noalloc": (C.c_int32, [C.POINTER(PfRecords), C.c_uint32, C.c_int32,
                                           C.POINTER(C.c_float * 36), C.c_uint32, _VP, _VP, _VP,
                                           C.POINTER(C.c_float), _VP]),
    "sty_scene_create": (C.c_int32, [_VP, _VP, C.c_uint32, _VP, C.c_uint32, _VP, C.POINTER(C.c_void_p)]),
    "sty_scene_destroy": (C.c_int32, [C.c_void_p]),
    "sty_scene_closest_hit": (C.c_int32, [C.c_void_p, _VP, C.c_uint64, _VP, _VP, _VP, _VP]),
    "sty_pf_render": (C.c_int32, [C.c_void_p, _VP, _VP, C.c_uint32, _VP, C.POINTER(C.c_uint64), _VP]),
    "sty_nrc_samples": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _VP, _VP,
                                    C.c_uint64, C.POINTER(C.c_uint64), _VP]),
    "sty_nrc_render": (C.c_int32, [C.c_void_p, C.c_void_p, _VP, _VP, C.c_uint32, _VP, _VP, _VP]),
    "sty_brpt_render": (C.c_int32, [C.c_void_p, _VP, _VP, C.c_uint32, _VP, _VP, _VP]),
    "sty_bsdf_eval": (C.c_int32, [_VP, C.c_uint64, _VP, _VP, _VP, _VP, _VP]),
    "sty_bsdf_sample": (C.c_int32, [_VP, C.c_uint64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sty_principled_table": (C.c_int32, [_VP]),
    "sty_nrc_create": (C.c_int32, [_VP, C.POINTER(C.c_void_p)]),
    "sty_nrc_create_grid": (C.c_int32, [_VP, C.POINTER(C.c_void_p)]),
    "sty_nrc_destroy": (C.c_int32, [C.c_void_p]),
    "sty_nrc_param_count": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "sty_nrc_save_params": (C.c_int32, [C.c_void_p, _VP]),
    "sty_nrc_load_params": (C.c_int32, [C.c_void_p, _VP]),
    "sty_nrc_set_learning_rate": (C.c_int32, [C.c_void_p, C.c_float]),
    "sty_nrc_get_learning_rate": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float)]),
    "sty_nrc_reset_optimizer": (C.c_int32, [C.c_void_p]),
    "sty_nrc_inference": (C.c_int32, [C.c_void_p, C.c_uint64, _VP, _VP, _VP]),
    "sty_nrc_train_inference": (C.c_int32, [C.c_void_p, C.c_uint64, _VP, _VP, _VP]),
    "sty_nrc_train": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint64, _VP, _VP, C.POINTER(C.c_float), _VP]),
    "sty_nrc_gradient": (C.c_int32, [C.c_void_p, C.c_uint32, _VP, _VP, _VP, C.POINTER(C.c_float), _VP]),
    "sty_nrc_set_train_kernel": (C.c_int32, [C.c_int32]),
    "sty_pcg32_streams": (C.c_int32, [_VP, C.c_uint64, C.c_uint64, C.c_uint32, _VP, _VP, _VP]),
    "sty_std_rng_u64": (C.c_int32, [C.c_uint64, C.c_uint64, C.c_uint64, _VP, _VP]),
    "sty_pf_trace_records": (C.c_int32, [C.c_void_p, _VP, _VP, C.c_uint32, _VP, C.POINTER(C.c_uint64), _VP]),
    "sty_scene_camera_rays": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint64, _VP, _VP]),
    "sty_pf_nrc_render": (C.c_int32, [C.c_void_p, C.c_void_p, _VP, _VP, C.c_uint32, _VP, _VP, _VP]),
    "sty_hash_cells": (C.c_int32, [_VP, C.c_uint64, C.POINTER(C.c_float * 3), C.POINTER(C.c_float * 3),
                                   C.POINTER(C.c_uint32 * 3), C.c_uint32, _VP, _VP, _VP]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libsty_gb300.so (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"libsty_gb300.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != STY_OK:
        msg = lib().sty_last_error().decode(errors="replace")
        raise StyError(status, msg)


def style_node(kind: int, params: Sequence[float] = (), n: int = 0, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    nd = StyleNode()
    nd.kind = kind
    nd.depth_mask = depth_mask & 0xFFFFFFFF
    nd.n = n
    for i, v in enumerate(params):
        nd.p[i] = float(v)
    return nd


def style_program(nodes: Sequence[StyleNode] = ()) -> StyleProgram:
    if len(nodes) > STY_STYLE_MAX_NODES:
        raise ValueError("too many style nodes")
    p = StyleProgram()
    p.n_nodes = len(nodes)
    for i, nd in enumerate(nodes):
        p.nodes[i] = nd
    return p


# ---- constructors of the individual nodes (parameter layouts of include/sty_gb300.h) --------
def toon(color_band_width: float, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    return style_node(STY_STYLE_TOON, [color_band_width], 0, depth_mask)


def palette(colors, indirect_scale: float = 1.0, gamma: float = 1.0, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    colors = [tuple(c) for c in colors]
    if len(colors) > 19:
        raise ValueError("palette holds at most 19 colours")
    flat = [indirect_scale, gamma] + [v for c in colors for v in c]
    return style_node(STY_STYLE_PALETTE, flat, len(colors), depth_mask)


def sat_adjust(power: float, indirect_scale: float = 1.0, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    return style_node(STY_STYLE_SAT_ADJUST, [power, indirect_scale], 0, depth_mask)


def sat_rex(blend: float, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    return style_node(STY_STYLE_SAT_REX, [blend], 0, depth_mask)


def eight_bit(indirect_scale: float = 1.0, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    return style_node(STY_STYLE_EIGHT_BIT, [indirect_scale], 0, depth_mask)


def toon_steps(thresholds, levels, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    thresholds = list(thresholds)
    levels = list(levels)
    n = len(thresholds)
    if not 1 <= n <= 8 or len(levels) != n + 1:
        raise ValueError("toon_steps wants 1..8 thresholds and len(thresholds)+1 levels")
    p = [0.0] * 17
    p[:n] = thresholds
    p[8:8 + n + 1] = levels
    return style_node(STY_STYLE_TOON_STEPS, p, n, depth_mask)


def ramp_smooth(sharpness: float, thresholds, colors, depth_mask: int = 0xFFFFFFFF) -> StyleNode:
    thresholds = list(thresholds)
    colors = [tuple(c) for c in colors]
    n = len(thresholds)
    if not 1 <= n <= 8 or len(colors) != n:
        raise ValueError("ramp_smooth wants 1..8 thresholds and as many colours")
    p = [0.0] * 33
    p[0] = sharpness
    p[1:1 + n] = thresholds
    for k, c in enumerate(colors):
        p[9 + 3 * k:12 + 3 * k] = c
    return style_node(STY_STYLE_RAMP_SMOOTH, p, n, depth_mask)


def half_tone(radius_scale: float, radius: float, grid_distance: float, dark_tone, light_tone,
              indirect_scale: float = 1.0, blend: float = 1.0, max_depth: int = 0, affine=None) -> StyleNode:
    """sty_half_tone (svm/surface/mod.rs:1091-1233): a world-space dot screen of spacing
    `grid_distance`. `affine` is the node's TRS matrix (4 x 4 or 3 x 4, row-major); like
    AffineTransform::from_matrix (geometry.rs:216-222) a matrix within 1e-4 of the identity is
    applied as the identity. The node applies at depths <= max_depth."""
    if grid_distance <= 0:
        raise ValueError("half_tone wants grid_distance > 0")
    m = [[1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0]]
    if affine is not None:
        rows = [list(map(float, r)) for r in affine]
        if len(rows) == 4 and any(abs(a - b) > 1e-12 for a, b in zip(rows[3], (0.0, 0.0, 0.0, 1.0))):
            raise ValueError("half_tone wants an affine map (last row 0 0 0 1)")
        eye = [[float(i == j) for j in range(4)] for i in range(4)]
        if any(abs(rows[i][j] - eye[i][j]) > 1e-4 for i in range(len(rows)) for j in range(4)):
            m = rows[:3]
    p = [indirect_scale, radius_scale, radius, grid_distance, float(max_depth), blend,
         *map(float, dark_tone), *map(float, light_tone)] + [x for r in m for x in r]
    mask = 0xFFFFFFFF if max_depth >= 31 else (1 << (max_depth + 1)) - 1
    return style_node(STY_STYLE_HALF_TONE, p, 0, mask)
