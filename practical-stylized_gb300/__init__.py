"""Host-side mirror of the reference's NL-PF / NL-NRC interface over the libsty_gb300 C ABI.

The compute path is the CUDA library `lib/libsty_gb300.so` (built by `build.py`); this module
only marshals arguments through ctypes. There is no CPU fallback: if the library is missing,
every call raises `RuntimeError`.

Import name: the directory is `practical-stylized_gb300`; `__graft_entry__.package()` (or
`load()` below) registers it as the module `practical_stylized_gb300`.
"""
from __future__ import annotations

import ctypes as C
import pathlib

from . import abi  # noqa: F401  (ctypes mirror of include/sty_gb300.h)
from .abi import (  # noqa: F401
    STY_OK, STY_ERR_ARG, STY_ERR_OOM, STY_ERR_CUDA, STY_ERR_ITER_LIMIT, STY_ERR_NAN,
    STY_ERR_UNSUPPORTED, StyError, lib, check, style_program, style_node,
)
from .pf import (  # noqa: F401
    ScreenParams, RecordSet, pf_screen_filter, pf_screen_filter_depth, film_accumulate,
    c2_params, c2_style, set_screen_kernel, SCREEN_KERNEL_AUTO, SCREEN_KERNEL_FP32, SCREEN_KERNEL_TENSOR,
)
from . import synth  # noqa: F401
from . import pf_ref  # noqa: F401
from . import nrc  # noqa: F401
from . import scene  # noqa: F401
from . import scenegraph  # noqa: F401
from . import replicas  # noqa: F401

PKG_DIR = pathlib.Path(__file__).resolve().parent
