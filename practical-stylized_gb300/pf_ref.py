"""Reference-mode NL-PF host wrapper (world-space hash grid + clustering + SMIS, one depth).

Mirrors PathFiltering::render's per-depth steps (crates/akari_integrator/src/
lm_path_filtering.rs:1673-1774): build grid, cluster, filter. The context owns the device
scratch; vertex arrays are caller-owned device tensors.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .abi import check, lib
from .synth import REF_FIELDS, REF_SCALARS

STY_MAT_DIFFUSE = 0
STY_MAT_GGX = 1
STY_MAT_PRINCIPLED = 2
STY_MAT_GLASS = 3


class PfMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("albedo", C.c_float * 3), ("alpha", C.c_float), ("style", C.c_int32 * 4),
                ("roughness", C.c_float), ("metallic", C.c_float), ("ior", C.c_float), ("transmission", C.c_float),
                ("specular_ior_level", C.c_float), ("specular_tint", C.c_float * 3), ("coat_weight", C.c_float),
                ("coat_roughness", C.c_float), ("coat_ior", C.c_float), ("coat_tint", C.c_float * 3)]


class PfVertices(C.Structure):
    _fields_ = [("active", C.c_void_p), ("p", C.c_void_p * 3), ("wo", C.c_void_p * 3), ("ns", C.c_void_p * 3),
                ("ng", C.c_void_p * 3), ("le", C.c_void_p * 3), ("mis", C.c_void_p), ("dir_wi", C.c_void_p * 3),
                ("dir_l", C.c_void_p * 3), ("dir_pdf", C.c_void_p), ("ind_wi", C.c_void_p * 3),
                ("ind_mis", C.c_void_p), ("flags", C.c_void_p), ("material", C.c_void_p), ("n", C.c_uint64)]


class PfRefParams(C.Structure):
    _fields_ = [("depth", C.c_uint32), ("radius", C.c_float), ("reuse", C.c_uint32), ("smis", C.c_int32),
                ("cluster", C.c_int32), ("disable_flag_check", C.c_int32), ("no_first_hit_stylization", C.c_int32),
                ("table_size", C.c_uint32), ("pmin", C.c_float * 3), ("pmax", C.c_float * 3),
                ("max_cluster_rounds", C.c_uint32)]


@dataclass
class RefParams:
    """Fields of lm_path_filtering::Config that the per-depth filter consumes."""
    depth: int = 1
    radius: float = 0.05
    reuse: int = 64
    smis: bool = True
    cluster: bool = False
    disable_flag_check: bool = False
    no_first_hit_stylization: bool = False
    table_size: int = 1 << 26
    pmin: tuple = (-1.0, -1.0, -1.0)
    pmax: tuple = (1.0, 1.0, 1.0)
    max_cluster_rounds: int = 64

    def c(self) -> PfRefParams:
        return PfRefParams(self.depth, self.radius, self.reuse, int(self.smis), int(self.cluster),
                           int(self.disable_flag_check), int(self.no_first_hit_stylization), self.table_size,
                           (C.c_float * 3)(*self.pmin), (C.c_float * 3)(*self.pmax), self.max_cluster_rounds)


def materials(specs) -> "C.Array":
    """specs: iterable of (kind, albedo rgb, alpha, style program per style index (4 ints, -1 none))."""
    specs = list(specs)
    arr = (PfMaterial * len(specs))()
    for i, (kind, alb, alpha, style) in enumerate(specs):
        arr[i].kind = kind
        arr[i].albedo[:] = list(alb)
        arr[i].alpha = alpha
        arr[i].style[:] = list(style)
    return arr


def programs(progs) -> "C.Array":
    progs = list(progs)
    arr = (abi.StyleProgram * max(1, len(progs)))()
    for i, p in enumerate(progs):
        arr[i] = p
    return arr


def vertices_struct(arrays: dict, ptr=lambda a: a.data_ptr()) -> PfVertices:
    """PfVertices over a dict of arrays (device tensors by default; pass
    ptr=lambda a: a.ctypes.data for host numpy arrays)."""
    for k, a in arrays.items():
        if isinstance(a, np.ndarray) and not a.flags["C_CONTIGUOUS"]:
            raise ValueError(f"vertex field {k} must be C-contiguous")
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError(f"vertex field {k} must be contiguous")
    v = PfVertices()
    v.active = ptr(arrays["active"])
    for name in REF_FIELDS:
        a = arrays[name]
        dst = getattr(v, name)
        for k in range(3):
            dst[k] = ptr(a[k])
    for name in REF_SCALARS:
        setattr(v, name, ptr(arrays[name]))
    v.flags = ptr(arrays["flags"])
    v.material = ptr(arrays["material"])
    v.n = int(arrays["active"].shape[0])
    return v


class RefContext:
    def __init__(self, max_vertices: int, table_size: int = 1 << 26):
        self.h = C.c_void_p()
        check(lib().sty_pf_ref_create(max_vertices, table_size, C.byref(self.h)))
        self.table_size = table_size

    def close(self):
        if self.h:
            lib().sty_pf_ref_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def filter(self, dev: dict, params: RefParams, mats, progs, n_progs: int, rng, in_next=None, out=None,
               neighbours=None, cluster_id=None, stream=None):
        import torch
        n = int(dev["active"].shape[0])
        if out is None:
            out = torch.empty((3, n), dtype=torch.float32, device=dev["active"].device)
        v = vertices_struct(dev)
        prm = params.c()
        from .pf import _stream_ptr
        check(lib().sty_pf_ref_filter(self.h, C.byref(v), in_next.data_ptr() if in_next is not None else None,
                                      C.byref(prm), mats, len(mats), progs if n_progs else None, n_progs,
                                      rng.data_ptr(), out.data_ptr(),
                                      neighbours.data_ptr() if neighbours is not None else None,
                                      cluster_id.data_ptr() if cluster_id is not None else None,
                                      _stream_ptr(stream)))
        return out


def to_device(arrays: dict, device="cuda") -> dict:
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in arrays.items()}
