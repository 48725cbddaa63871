"""Screen-space NL-PF host wrapper: records resident in device memory, per-depth filter calls.

Mirrors the per-depth backward pass of the reference's PathFiltering::render
(crates/akari_integrator/src/lm_path_filtering.rs:1673-1774): depths are filtered from the
deepest to 0 and each depth's styled result feeds the parent depth's incoming radiance.
PyTorch is used only to own device memory and to provide the current CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .abi import check, lib


@dataclass
class ScreenParams:
    radius: int = 16
    sigma_pixel: float = 8.0
    sigma_pos: float = 0.5
    sigma_nrm: float = 0.2

    def c(self) -> abi.PfScreenParams:
        return abi.PfScreenParams(int(self.radius), float(self.sigma_pixel), float(self.sigma_pos),
                                  float(self.sigma_nrm))


def c2_params() -> ScreenParams:
    """Filter parameters of the 1920x1080 x 4 spp x 5 depth synthetic workload."""
    return ScreenParams(radius=16, sigma_pixel=8.0, sigma_pos=0.5, sigma_nrm=0.2)


def c2_style() -> abi.StyleProgram:
    """4-level toon on the first-bounce radiance (depth 1): thresholds 0.1 / 0.3 / 0.6."""
    return abi.style_program([abi.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0], depth_mask=1 << 1)])


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream or None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


class RecordSet:
    """Path-vertex records in device memory: one float32 slab [12, n] (FIELDS order of
    synth.py) plus int32 valid [n], n = depths*height*width*spp."""

    def __init__(self, planes, valid, width: int, height: int, spp: int, depths: int):
        self.planes, self.valid = planes, valid
        self.width, self.height, self.spp, self.depths = width, height, spp, depths
        n = width * height * spp * depths
        assert tuple(planes.shape) == (12, n) and tuple(valid.shape) == (n,)

    @classmethod
    def from_numpy(cls, planes: np.ndarray, valid: np.ndarray, width, height, spp, depths, device="cuda"):
        import torch
        return cls(torch.from_numpy(np.ascontiguousarray(planes)).to(device),
                   torch.from_numpy(np.ascontiguousarray(valid)).to(device), width, height, spp, depths)

    @property
    def n_per_depth(self) -> int:
        return self.width * self.height * self.spp

    def c(self) -> abi.PfRecords:
        r = abi.PfRecords()
        base = self.planes.data_ptr()
        stride = self.planes.stride(0) * self.planes.element_size()
        for k in range(3):
            r.pos[k] = base + (0 + k) * stride
            r.nrm[k] = base + (3 + k) * stride
            r.rad[k] = base + (6 + k) * stride
            r.thr[k] = base + (9 + k) * stride
        r.valid = self.valid.data_ptr()
        r.width, r.height, r.spp, r.depths = self.width, self.height, self.spp, self.depths
        return r


def host_records(planes: np.ndarray, valid: np.ndarray, width, height, spp, depths) -> abi.PfRecords:
    """PfRecords over HOST numpy arrays (for the CPU oracle)."""
    r = abi.PfRecords()
    for k in range(3):
        r.pos[k] = planes[0 + k].ctypes.data
        r.nrm[k] = planes[3 + k].ctypes.data
        r.rad[k] = planes[6 + k].ctypes.data
        r.thr[k] = planes[9 + k].ctypes.data
    r.valid = valid.ctypes.data
    r.width, r.height, r.spp, r.depths = width, height, spp, depths
    return r


SCREEN_KERNEL_AUTO, SCREEN_KERNEL_FP32, SCREEN_KERNEL_TENSOR = 0, 1, 2


def set_screen_kernel(kernel: int) -> None:
    """Process-wide choice of the screen filter's kernel (sty_pf_screen_set_kernel): AUTO, FP32 (the
    CUDA-core kernels) or TENSOR (the tcgen05 split-TF32 kernel where it serves the configuration)."""
    check(lib().sty_pf_screen_set_kernel(int(kernel)))


def pf_screen_filter_depth(rs: RecordSet, depth: int, params: ScreenParams, style=None, out_next=None,
                           out=None, filtered=None, stream=None):
    """Filter one depth; returns `out` (device float32 [3, W*H*S])."""
    import torch
    if out is None:
        out = torch.empty((3, rs.n_per_depth), dtype=torch.float32, device=rs.planes.device)
    rec = rs.c()
    prm = params.c()
    sp = C.byref(style) if style is not None else None
    check(lib().sty_pf_screen_filter_depth(C.byref(rec), depth, C.byref(prm), sp,
                                           out_next.data_ptr() if out_next is not None else None,
                                           out.data_ptr(),
                                           filtered.data_ptr() if filtered is not None else None,
                                           _stream_ptr(stream)))
    return out


def pf_screen_filter(rs: RecordSet, params: ScreenParams, style=None, out=None, stream=None):
    """All depths, deepest first; returns device float32 [depths, 3, W*H*S]."""
    import torch
    if out is None:
        out = torch.empty((rs.depths, 3, rs.n_per_depth), dtype=torch.float32, device=rs.planes.device)
    rec = rs.c()
    prm = params.c()
    sp = C.byref(style) if style is not None else None
    check(lib().sty_pf_screen_filter(C.byref(rec), C.byref(prm), sp, out.data_ptr(), _stream_ptr(stream)))
    return out


def film_accumulate(out0, width: int, height: int, spp: int, weight: float, film, stream=None):
    check(lib().sty_film_accumulate(out0.data_ptr(), width, height, spp, float(weight), film.data_ptr(),
                                    _stream_ptr(stream)))
    return film
