"""Host-side checks of the C ABI: the library loads, exports every declared entry point, struct
layouts match the header, and argument validation fails cleanly without touching the GPU."""
import ctypes as C
import re

import pytest

from conftest import ROOT


def declared_functions():
    txt = (ROOT / "include" / "sty_gb300.h").read_text()
    return sorted(set(re.findall(r"STY_API\s+[\w\s\*]+?\b(sty_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sty_pf_screen_filter_depth" in names and "sty_version" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(sty):
    lib = sty.abi.lib()
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/sty_gb300.h but not exported"
        assert name in sty.abi.SIGNATURES, f"{name} has no ctypes signature"


def test_struct_layouts(sty):
    a = sty.abi
    assert C.sizeof(a.StyleNode) == 16 + 4 * a.STY_STYLE_MAX_PARAMS
    assert C.sizeof(a.StyleProgram) == 16 + a.STY_STYLE_MAX_NODES * C.sizeof(a.StyleNode)
    assert C.sizeof(a.PfRecords) == 13 * 8 + 16
    assert C.sizeof(a.PfScreenParams) == 16
    assert C.sizeof(a.Pcg32) == 16


def test_struct_sizes_match_the_library(sty):
    """Every struct the header declares has a ctypes mirror of the size the library was built with."""
    from importlib import import_module
    pkg = sty.__name__
    mirrors = {"sty_pcg32": "abi.Pcg32", "sty_style_node": "abi.StyleNode", "sty_style_program": "abi.StyleProgram",
               "sty_pf_records": "abi.PfRecords", "sty_pf_screen_params": "abi.PfScreenParams",
               "sty_pf_material": "pf_ref.PfMaterial", "sty_pf_vertices": "pf_ref.PfVertices",
               "sty_pf_ref_params": "pf_ref.PfRefParams", "sty_nrc_config": "nrc.NrcConfig",
               "sty_nrc_grid_config": "nrc.NrcGridConfig", "sty_scene_material": "scene.SceneMaterial",
               "sty_camera": "scene.Camera", "sty_pf_render_config": "scene.RenderConfig",
               "sty_nrc_render_config": "scene.NrcRenderConfig", "sty_nrc_render_stats": "scene.NrcRenderStats",
               "sty_brpt_config": "scene.BrptConfig", "sty_brpt_stats": "scene.BrptStats",
               "sty_pf_records_out": "scene.RecordsOut", "sty_pf_nrc_config": "scene.PfNrcConfig"}
    declared = set(re.findall(r"\}\s*(sty_\w+)\s*;", (ROOT / "include" / "sty_gb300.h").read_text()))
    assert declared == set(mirrors), declared ^ set(mirrors)
    lib = sty.abi.lib()
    for name, path in mirrors.items():
        mod, cls = path.split(".")
        size = C.sizeof(getattr(import_module(f"{pkg}.{mod}"), cls))
        assert lib.sty_struct_size(name.encode()) == size, (name, lib.sty_struct_size(name.encode()), size)
    assert lib.sty_struct_size(b"no_such_struct") == 0


def test_version_and_status_strings(sty):
    lib = sty.abi.lib()
    assert lib.sty_version() >= 100
    assert lib.sty_status_string(0) == b"STY_OK"
    assert lib.sty_status_string(1) == b"STY_ERR_ARG"
    assert lib.sty_status_string(99) == b"STY_ERR_UNKNOWN"


def test_argument_validation_without_gpu(sty):
    """Null / inconsistent arguments are rejected before any CUDA call (no GPU needed)."""
    a = sty.abi
    lib = a.lib()
    prm = a.PfScreenParams(16, 8.0, 0.5, 0.2)
    st = lib.sty_pf_screen_filter_depth(None, 0, C.byref(prm), None, None, None, None, None)
    assert st == a.STY_ERR_ARG
    assert b"null" in lib.sty_last_error()
    rec = a.PfRecords()
    rec.width, rec.height, rec.spp, rec.depths = 8, 8, 3, 1  # spp 3 unsupported
    for k in range(3):
        rec.pos[k] = rec.nrm[k] = rec.rad[k] = rec.thr[k] = 16
    rec.valid = 16
    st = lib.sty_pf_screen_filter_depth(C.byref(rec), 0, C.byref(prm), None, None, 16, None, None)
    assert st == a.STY_ERR_ARG and b"spp" in lib.sty_last_error()
    rec.spp = 4
    bad = a.PfScreenParams(40, 8.0, 0.5, 0.2)
    st = lib.sty_pf_screen_filter_depth(C.byref(rec), 0, C.byref(bad), None, None, 16, None, None)
    assert st == a.STY_ERR_ARG and b"radius" in lib.sty_last_error()
    st = lib.sty_pf_screen_filter_depth(C.byref(rec), 5, C.byref(prm), None, None, 16, None, None)
    assert st == a.STY_ERR_ARG and b"depth" in lib.sty_last_error()
    prog = a.style_program([a.style_node(99)])
    st = lib.sty_pf_screen_filter_depth(C.byref(rec), 0, C.byref(prm), C.byref(prog), None, 16, None, None)
    assert st == a.STY_ERR_ARG and b"style" in lib.sty_last_error()
    with pytest.raises(a.StyError) as ei:
        a.check(a.STY_ERR_ARG)
    assert ei.value.status == a.STY_ERR_ARG


def test_screen_kernel_choice_without_gpu(sty):
    """sty_pf_screen_set_kernel takes the three kernel families and rejects anything else (no GPU)."""
    lib = sty.abi.lib()
    for k in (sty.SCREEN_KERNEL_FP32, sty.SCREEN_KERNEL_TENSOR, sty.SCREEN_KERNEL_AUTO):
        assert lib.sty_pf_screen_set_kernel(k) == sty.abi.STY_OK
    assert lib.sty_pf_screen_set_kernel(3) == sty.abi.STY_ERR_ARG
    assert b"unknown kernel" in lib.sty_last_error()
    with pytest.raises(sty.StyError):
        sty.set_screen_kernel(-1)
    lib.sty_pf_screen_set_kernel(sty.SCREEN_KERNEL_AUTO)


def test_train_kernel_choice_without_gpu(sty):
    """sty_nrc_set_train_kernel takes AUTO and ONE_TILE and rejects anything else (no GPU)."""
    lib = sty.abi.lib()
    for k in (sty.nrc.TRAIN_KERNEL_ONE_TILE, sty.nrc.TRAIN_KERNEL_AUTO):
        assert lib.sty_nrc_set_train_kernel(k) == sty.abi.STY_OK
    assert lib.sty_nrc_set_train_kernel(2) == sty.abi.STY_ERR_ARG
    assert b"unknown kernel" in lib.sty_last_error()
    with pytest.raises(sty.StyError):
        sty.nrc.set_train_kernel(-1)
    lib.sty_nrc_set_train_kernel(sty.nrc.TRAIN_KERNEL_AUTO)


def test_style_builders_validate(sty):
    a = sty.abi
    with pytest.raises(ValueError):
        a.toon_steps([0.1, 0.2], [0.0, 1.0])
    with pytest.raises(ValueError):
        a.palette([(0, 0, 0)] * 20)
    p = a.style_program([a.toon(0.2), a.sat_rex(0.3)])
    assert p.n_nodes == 2 and abs(p.nodes[0].p[0] - 0.2) < 1e-7


def test_missing_library_fails_loudly(tmp_path):
    """Without the CUDA library the package raises on first use: there is no CPU fallback."""
    import subprocess
    import sys
    code = (
        "import sys, pathlib; sys.path.insert(0, %r)\n"
        "import __graft_entry__ as g\n"
        "sty = g.package()\n"
        "sty.abi.LIB_PATH = pathlib.Path(%r) / 'libsty_gb300.so'\n"
        "sty.abi._lib = None\n"
        "try:\n"
        "    sty.abi.lib()\n"
        "except RuntimeError as e:\n"
        "    print('raised:', e)\n"
        "    sys.exit(0)\n"
        "sys.exit(3)\n" % (str(ROOT), str(tmp_path)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "not built" in r.stdout
