"""Neural radiance cache host wrapper: the reference's TinyCudaNRC API (crates/akari_integrator/src/
nrc.rs:98-185) over the sty_nrc_* C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, lib

STY_NRC_FP32 = 0
STY_NRC_BF16 = 1
GRID_LAYERED = 1  # STY_NRC_GRID_LAYERED
GRID_FP16 = 2     # STY_NRC_GRID_FP16

# the spherical row layout's frequency table: pos 3, dir 2, normal 2, roughness 1, albedo 3
# -> 3*8 + 4*6 + 4*4 = 64 encoded columns
C4_FREQS = (4, 4, 4, 3, 3, 3, 3, 2, 2, 2, 2)


class NrcConfig(C.Structure):
    _fields_ = [("input_dims", C.c_uint32), ("output_dims", C.c_uint32), ("batch_size", C.c_uint32),
                ("hidden_layers", C.c_uint32), ("precision", C.c_uint32), ("freqs", C.c_uint32 * 16),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("ema_decay", C.c_float), ("decay_base", C.c_float), ("decay_interval", C.c_uint32),
                ("seed", C.c_uint64)]


def config(freqs=C4_FREQS, output_dims=3, batch_size=1 << 16, hidden_layers=5, precision=STY_NRC_BF16,
           learning_rate=1e-2, beta1=0.9, beta2=0.99, epsilon=1e-8, ema_decay=0.95, decay_base=1.0,
           decay_interval=100, seed=1337) -> NrcConfig:
    c = NrcConfig()
    c.input_dims = len(freqs)
    c.output_dims = output_dims
    c.batch_size = batch_size
    c.hidden_layers = hidden_layers
    c.precision = precision
    for i, f in enumerate(freqs):
        c.freqs[i] = f
    c.learning_rate, c.beta1, c.beta2, c.epsilon = learning_rate, beta1, beta2, epsilon
    c.ema_decay, c.decay_base, c.decay_interval, c.seed = ema_decay, decay_base, decay_interval, seed
    return c


class NrcGridConfig(C.Structure):
    _fields_ = [("input_dims", C.c_uint32), ("output_dims", C.c_uint32), ("batch_size", C.c_uint32),
                ("hidden_layers", C.c_uint32), ("hidden_units", C.c_uint32), ("grid_levels", C.c_uint32),
                ("grid_features", C.c_uint32), ("log2_table", C.c_uint32), ("base_resolution", C.c_uint32),
                ("per_level_scale", C.c_float), ("blob_dims", C.c_uint32), ("blob_bins", C.c_uint32),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("ema_decay", C.c_float), ("decay_base", C.c_float), ("decay_interval", C.c_uint32),
                ("flags", C.c_uint32), ("seed", C.c_uint64)]


def grid_config(max_depth=12, output_dims=3, batch_size=1 << 16, hidden_layers=5, hidden_units=128, grid_levels=22,
                grid_features=4, log2_table=19, base_resolution=16, per_level_scale=2.0, blob_dims=7, blob_bins=4,
                learning_rate=1e-3, beta1=0.9, beta2=0.99, epsilon=1e-8, ema_decay=0.95, decay_base=1.0,
                decay_interval=100, seed=1337, layered=False, fp16=False) -> NrcGridConfig:
    """The reference's NL-NRC network (nrc_pt.rs:1159-1352; defaults of configs/teaser/nl-nrc.json):
    rows of 20 + max_depth inputs in the reference layout. `layered` forces the layer-by-layer
    inference path instead of the fused tensor-core path (tile encoder + on-chip MLP kernel);
    `fp16` makes the MLP operands FP16 (tiny-cuda-nn's precision) instead of BF16."""
    c = NrcGridConfig()
    c.input_dims, c.output_dims, c.batch_size = 20 + max_depth, output_dims, batch_size
    c.hidden_layers, c.hidden_units = hidden_layers, hidden_units
    c.grid_levels, c.grid_features, c.log2_table = grid_levels, grid_features, log2_table
    c.base_resolution, c.per_level_scale = base_resolution, per_level_scale
    c.blob_dims, c.blob_bins = blob_dims, blob_bins
    c.learning_rate, c.beta1, c.beta2, c.epsilon = learning_rate, beta1, beta2, epsilon
    c.ema_decay, c.decay_base, c.decay_interval, c.seed = ema_decay, decay_base, decay_interval, seed
    c.flags = (GRID_LAYERED if layered else 0) | (GRID_FP16 if fp16 else 0)
    return c


TRAIN_KERNEL_AUTO, TRAIN_KERNEL_ONE_TILE = 0, 1


def set_train_kernel(kernel: int) -> None:
    """Process-wide choice of the BF16 training kernel (sty_nrc_set_train_kernel): AUTO (two tiles
    in flight per SM where the network has at most 5 hidden layers) or ONE_TILE. Both give the same
    gradients bit for bit."""
    check(lib().sty_nrc_set_train_kernel(int(kernel)))


def _sp(stream):
    from .pf import _stream_ptr
    return _stream_ptr(stream)


class NRC:
    """Mirror of TinyCudaNRC: train / inference / train_inference on device matrices (torch
    tensors, sample-major rows)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = C.c_void_p()
        if isinstance(cfg, NrcGridConfig):
            check(lib().sty_nrc_create_grid(C.byref(cfg), C.byref(self.h)))
        else:
            check(lib().sty_nrc_create(C.byref(cfg), C.byref(self.h)))

    def close(self):
        if self.h:
            lib().sty_nrc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def param_count(self) -> int:
        n = C.c_uint64()
        check(lib().sty_nrc_param_count(self.h, C.byref(n)))
        return n.value

    def save_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), dtype=np.float32)
        check(lib().sty_nrc_save_params(self.h, p.ctypes.data))
        return p

    def load_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.param_count()
        check(lib().sty_nrc_load_params(self.h, p.ctypes.data))

    @property
    def learning_rate(self) -> float:
        v = C.c_float()
        check(lib().sty_nrc_get_learning_rate(self.h, C.byref(v)))
        return v.value

    @learning_rate.setter
    def learning_rate(self, lr: float):
        check(lib().sty_nrc_set_learning_rate(self.h, lr))

    def reset_optimizer(self):
        check(lib().sty_nrc_reset_optimizer(self.h))

    def inference(self, x, out=None, stream=None, ema=True):
        import torch
        n = x.shape[0]
        if out is None:
            out = torch.empty((n, self.cfg.output_dims), dtype=torch.float32, device=x.device)
        fn = lib().sty_nrc_inference if ema else lib().sty_nrc_train_inference
        check(fn(self.h, n, x.data_ptr(), out.data_ptr(), _sp(stream)))
        return out

    def train(self, x, target, n_iters: int, stream=None, want_loss=True) -> float | None:
        loss = C.c_float()
        check(lib().sty_nrc_train(self.h, x.shape[0], n_iters, x.data_ptr(), target.data_ptr(),
                                  C.byref(loss) if want_loss else None, _sp(stream)))
        return loss.value if want_loss else None

    def gradient(self, x, target, stream=None):
        import torch
        g = torch.empty(self.param_count(), dtype=torch.float32, device=x.device)
        loss = C.c_float()
        check(lib().sty_nrc_gradient(self.h, x.shape[0], x.data_ptr(), target.data_ptr(), g.data_ptr(),
                                     C.byref(loss), _sp(stream)))
        return g, loss.value
