"""CPU oracle of the stylized NL-PF hot path -- TEST INFRASTRUCTURE ONLY.

ctypes binding of oracle/_build/liboracle.so (built by oracle/build.py from sty_oracle.cpp).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package;
the product library never calls it. See sty_oracle.h for the parity status.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build as _b
            _b.build()
        L = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        L.orc_num_threads.restype = C.c_int32
        L.orc_set_num_threads.argtypes = [C.c_int32]
        L.orc_style_apply_f64.argtypes = [vp, C.c_uint32, vp, vp, C.c_uint64]
        L.orc_style_apply_at_f64.argtypes = [vp, C.c_uint32, vp, vp, vp, C.c_uint64]
        L.orc_pf_screen_filter_records_f64.argtypes = [vp, C.c_uint32, vp, vp, vp, vp, C.c_uint64, vp, vp]
        L.orc_pf_screen_filter_depth_f64.argtypes = [vp, C.c_uint32, vp, vp, vp, vp, vp]
        L.orc_pf_screen_filter_depth_f32.argtypes = [vp, C.c_uint32, vp, vp, vp, vp, vp, C.c_int32, C.c_int32]
        L.orc_pcg32_streams.argtypes = [vp, C.c_uint64, C.c_uint64, C.c_uint32, vp, vp]
        L.orc_hash_cells.argtypes = [vp, C.c_uint64, vp, vp, vp, C.c_uint32, vp, vp]
        L.orc_chacha_block.argtypes = [vp, vp, C.c_int32]
        L.orc_std_rng_key.argtypes = [C.c_uint64, vp]
        L.orc_std_rng_u64.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, vp]
        L.orc_camera_rays.argtypes = [vp, C.c_uint32, C.c_uint64, vp]
        L.orc_pf_adjoint_loss_f64.restype = C.c_double
        L.orc_pf_adjoint_loss_f64.argtypes = [vp, C.c_uint32, C.c_int32, vp, C.c_uint32, vp, vp]
        L.orc_pf_adjoint_f64.restype = C.c_double
        L.orc_pf_adjoint_f64.argtypes = [vp, C.c_uint32, C.c_int32, vp, C.c_uint32, vp, vp, vp]
        L.orc_pf_adjoint_image_f64.restype = C.c_double
        L.orc_pf_adjoint_image_f64.argtypes = [vp, C.c_uint32, C.c_int32, vp, C.c_uint32, vp, vp]
        L.orc_closest_hit.argtypes = [vp, C.c_uint32, vp, C.c_uint64, vp, vp, vp]
        L.orc_path_trace.argtypes = [vp, vp, C.c_uint32, vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint64, vp]
        L.orc_brpt.argtypes = [vp, vp, C.c_uint32, vp, vp, vp, C.c_uint32, C.c_uint32, vp, C.c_uint32, C.c_uint32,
                               C.c_uint32, C.c_uint64, vp]
        L.orc_principled_table.argtypes = [vp]
        L.orc_principled_eval.argtypes = [vp, C.c_uint64, vp, vp, vp, vp]
        L.orc_principled_sample.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, vp]
        L.orc_pf_ref_filter.restype = C.c_int32
        L.orc_pf_ref_filter.argtypes = [vp, vp, vp, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, vp]
        L.orc_pf_ref_filter_select.restype = C.c_int32
        L.orc_pf_ref_filter_select.argtypes = [vp, vp, vp, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def style_apply(program, depth: int, rgb: np.ndarray) -> np.ndarray:
    rgb = np.ascontiguousarray(rgb, dtype=np.float64).reshape(-1, 3)
    out = np.empty_like(rgb)
    lib().orc_style_apply_f64(C.addressof(program) if program is not None else None, depth, _p(rgb), _p(out),
                              rgb.shape[0])
    return out


def style_apply_at(program, depth: int, rgb: np.ndarray, pos: np.ndarray) -> np.ndarray:
    """style_apply with the shaded point of each colour (read by the half-tone node)."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float64).reshape(-1, 3)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    out = np.empty_like(rgb)
    lib().orc_style_apply_at_f64(C.addressof(program), depth, _p(rgb), _p(pos), _p(out), rgb.shape[0])
    return out


def pf_screen_filter_depth(rec, depth, params, style, out_next=None, want_filtered=False):
    """FP64 filter of one depth on host records (abi.PfRecords over numpy arrays).
    Returns (out [3, n], filtered [3, n] or None) as float64."""
    n = rec.width * rec.height * rec.spp
    out = np.zeros((3, n), dtype=np.float64)
    filt = np.zeros((3, n), dtype=np.float64) if want_filtered else None
    nxt = None if out_next is None else np.ascontiguousarray(out_next, dtype=np.float64)
    lib().orc_pf_screen_filter_depth_f64(C.addressof(rec), depth, C.addressof(params),
                                         C.addressof(style) if style is not None else None,
                                         _p(nxt), _p(out), _p(filt))
    return out, filt


def pf_screen_filter_records(rec, depth, params, style, idx, out_next=None):
    """The FP64 filter at the given record indices of one depth only; returns (out, filtered) [3, len(idx)]."""
    idx = np.ascontiguousarray(idx, dtype=np.uint64)
    out = np.zeros((3, idx.size), dtype=np.float64)
    filt = np.zeros((3, idx.size), dtype=np.float64)
    nxt = None if out_next is None else np.ascontiguousarray(out_next, dtype=np.float64)
    lib().orc_pf_screen_filter_records_f64(C.addressof(rec), depth, C.addressof(params),
                                           C.addressof(style) if style is not None else None,
                                           _p(nxt), _p(idx), idx.size, _p(out), _p(filt))
    return out, filt


def pf_screen_filter_depth_f32(rec, depth, params, style, out_next=None, y0=0, y1=None):
    n = rec.width * rec.height * rec.spp
    out = np.zeros((3, n), dtype=np.float32)
    nxt = None if out_next is None else np.ascontiguousarray(out_next, dtype=np.float32)
    lib().orc_pf_screen_filter_depth_f32(C.addressof(rec), depth, C.addressof(params),
                                         C.addressof(style) if style is not None else None,
                                         _p(nxt), _p(out), None, y0, rec.height if y1 is None else y1)
    return out


def pcg32_streams(seeds: np.ndarray, first_seq: int, draws: int):
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    out = np.zeros((seeds.size, draws), dtype=np.uint32)
    states = np.zeros((seeds.size, 2), dtype=np.uint64)
    lib().orc_pcg32_streams(_p(seeds), first_seq, seeds.size, draws, _p(out), _p(states))
    return out, states


def chacha_block(words, rounds: int = 20) -> np.ndarray:
    """ChaCha block function of a 16-word input state (rounds of it, plus the input)."""
    w = np.ascontiguousarray(words, dtype=np.uint32).reshape(16)
    out = np.zeros(16, dtype=np.uint32)
    lib().orc_chacha_block(_p(w), _p(out), rounds)
    return out


def std_rng_key(seed: int) -> np.ndarray:
    key = np.zeros(8, dtype=np.uint32)
    lib().orc_std_rng_key(seed, _p(key))
    return key


def std_rng_u64(seed: int, first: int, n: int) -> np.ndarray:
    """gen::<u64>() outputs first .. first+n-1 of rand's StdRng::seed_from_u64(seed)."""
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_std_rng_u64(seed, first, n, _p(out))
    return out


def camera_rays(cam, branch: int, seed: int) -> np.ndarray:
    """Depth-0 rays [W*H*branch, 8] of every path slot (slot = b * W * H + pixel)."""
    out = np.zeros((cam.width * cam.height * branch, 8), dtype=np.float32)
    lib().orc_camera_rays(C.addressof(cam), branch, seed, _p(out))
    return out


def hash_cells(points: np.ndarray, pmin, pmax, res, table_size: int):
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    pmin = np.asarray(pmin, dtype=np.float32)
    pmax = np.asarray(pmax, dtype=np.float32)
    res = np.asarray(res, dtype=np.uint32)
    cells = np.zeros((pts.shape[0], 3), dtype=np.uint32)
    idx = np.zeros(pts.shape[0], dtype=np.uint32)
    lib().orc_hash_cells(_p(pts), pts.shape[0], _p(pmin), _p(pmax), _p(res), table_size, _p(cells), _p(idx))
    return cells, idx


def pf_ref_filter(arrays: dict, params_c, mats, progs, n_progs: int, rng_states: np.ndarray, in_next=None,
                  select=None):
    """Reference-mode filter of one depth on host arrays (dict from synth.ref_vertices).
    Returns (status, out [3, n] float64, neighbours [n], cluster_id [n], rng_states_after).
    select (bool [n], optional): filter only those vertices (the rest stay 0 / untouched)."""
    import importlib
    pfr = importlib.import_module(__package_name__() + ".pf_ref")
    n = int(arrays["active"].shape[0])
    v = pfr.vertices_struct(arrays, ptr=lambda a: a.ctypes.data)
    out = np.zeros((3, n), dtype=np.float64)
    nb = np.zeros(n, dtype=np.uint32)
    cid = np.zeros(n, dtype=np.uint32)
    st = np.ascontiguousarray(rng_states.copy())
    nxt = None if in_next is None else np.ascontiguousarray(in_next, dtype=np.float32)
    sel = None if select is None else np.ascontiguousarray(select, dtype=np.uint8)
    status = lib().orc_pf_ref_filter_select(C.addressof(v), _p(nxt), C.addressof(params_c), C.addressof(mats),
                                            len(mats), C.addressof(progs) if progs is not None else None, n_progs,
                                            _p(st), _p(out), _p(nb), _p(cid), _p(sel))
    return status, out, nb, cid, st


def __package_name__() -> str:
    return "practical_stylized_gb300"


def pf_adjoint_loss(rec, depth, radius, params, n_steps, target, in_next=None) -> float:
    prm = np.ascontiguousarray(params, dtype=np.float64)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    nxt = None if in_next is None else np.ascontiguousarray(in_next, dtype=np.float64)
    return lib().orc_pf_adjoint_loss_f64(C.addressof(rec), depth, radius, _p(prm), n_steps, _p(nxt), _p(tg))


def pf_adjoint_image(rec, depth, radius, params, n_steps, in_next=None) -> np.ndarray:
    """FP64 image (pixel-mean over spp of the ramp-styled filter output), interleaved rgb."""
    prm = np.ascontiguousarray(params, dtype=np.float64)
    nxt = None if in_next is None else np.ascontiguousarray(in_next, dtype=np.float64)
    img = np.zeros(3 * rec.width * rec.height, dtype=np.float64)
    lib().orc_pf_adjoint_image_f64(C.addressof(rec), depth, radius, _p(prm), n_steps, _p(nxt), _p(img))
    return img


def pf_adjoint(rec, depth, radius, params, n_steps, target, in_next=None):
    """(loss, grad[36]) in FP64 (analytic adjoint)."""
    prm = np.ascontiguousarray(params, dtype=np.float64)
    tg = np.ascontiguousarray(target, dtype=np.float64)
    nxt = None if in_next is None else np.ascontiguousarray(in_next, dtype=np.float64)
    g = np.zeros(36, dtype=np.float64)
    loss = lib().orc_pf_adjoint_f64(C.addressof(rec), depth, radius, _p(prm), n_steps, _p(nxt), _p(tg), _p(g))
    return loss, g


def closest_hit(tri_pos: np.ndarray, rays: np.ndarray):
    """Brute-force closest hit: (prim [n] uint32, t [n], bary [n,2])."""
    pos = np.ascontiguousarray(tri_pos, dtype=np.float32).reshape(-1)
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    n = r.shape[0]
    prim = np.zeros(n, dtype=np.uint32)
    t = np.zeros(n, dtype=np.float32)
    b = np.zeros((n, 2), dtype=np.float32)
    lib().orc_closest_hit(_p(pos), pos.size // 9, _p(r), n, _p(prim), _p(t), _p(b))
    return prim, t, b


def path_trace(tri_pos, mat_ids, albedo, emission, cam, spp: int, max_depth: int, seed: int = 0):
    """Independent FP64 CPU path tracer (NEE + balance MIS, diffuse, black emitters) -> image
    [H, W, 3]. cam = (eye3, target3, up3, fov_y, W, H, filter_radius)."""
    pos = np.ascontiguousarray(tri_pos, dtype=np.float32).reshape(-1)
    m = np.ascontiguousarray(mat_ids, dtype=np.uint32)
    alb = np.ascontiguousarray(albedo, dtype=np.float32).reshape(-1)
    em = np.ascontiguousarray(emission, dtype=np.float32).reshape(-1)
    c = np.ascontiguousarray(cam, dtype=np.float32)
    W, H = int(c[10]), int(c[11])
    img = np.zeros((H, W, 3), dtype=np.float64)
    lib().orc_path_trace(_p(pos), _p(m), m.size, _p(alb), _p(em), _p(c), spp, max_depth, seed, _p(img))
    return img


def brpt(tri_pos, mat_ids, materials, cam, programs, max_depth: int, inner_samples, repeats: int = 1,
         seed: int = 0, first_repeat: int = 0):
    """Recursive FP64 branching path tracer on the same sampling keys as sty_brpt_render (diffuse
    surfaces) -> image [H, W, 3]. `materials` is a ctypes array of sty_scene_material, `programs` a
    sequence of sty_style_program, cam = (eye3, target3, up3, fov_y, W, H, filter_radius)."""
    pos = np.ascontiguousarray(tri_pos, dtype=np.float32).reshape(-1)
    m = np.ascontiguousarray(mat_ids, dtype=np.uint32)
    c = np.ascontiguousarray(cam, dtype=np.float32)
    inner = np.ascontiguousarray(inner_samples, dtype=np.uint32)
    progs = list(programs)
    parr = None
    if progs:
        parr = (type(progs[0]) * len(progs))(*progs)
    W, H = int(c[10]), int(c[11])
    img = np.zeros((H, W, 3), dtype=np.float64)
    lib().orc_brpt(_p(pos), _p(m), m.size, C.addressof(materials), _p(c), None if parr is None else C.addressof(parr),
                   len(progs), max_depth, _p(inner), inner.size, repeats, first_repeat, seed, _p(img))
    return img


def principled_table() -> np.ndarray:
    """The FP64 ggx_dielectric_s table [z, mu, roughness] (16^3)."""
    t = np.zeros(16 ** 3, dtype=np.float64)
    lib().orc_principled_table(_p(t))
    return t.reshape(16, 16, 16)


def principled_eval(material, wo, wi):
    """FP64 principled closure in the shading frame: (f * |cos_i| [n, 3], pdf [n])."""
    wo = np.ascontiguousarray(wo, dtype=np.float64).reshape(-1, 3)
    wi = np.ascontiguousarray(wi, dtype=np.float64).reshape(-1, 3)
    f = np.zeros_like(wo)
    pdf = np.zeros(wo.shape[0])
    lib().orc_principled_eval(C.addressof(material), wo.shape[0], _p(wo), _p(wi), _p(f), _p(pdf))
    return f, pdf


def principled_sample(material, wo, u):
    """FP64 SurfaceClosure::sample of the principled closure: (wi [n, 3], f [n, 3], pdf [n])."""
    wo = np.ascontiguousarray(wo, dtype=np.float64).reshape(-1, 3)
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 3)
    wi = np.zeros_like(wo)
    f = np.zeros_like(wo)
    pdf = np.zeros(wo.shape[0])
    lib().orc_principled_sample(C.addressof(material), wo.shape[0], _p(wo), _p(u), _p(wi), _p(f), _p(pdf))
    return wi, f, pdf


def num_threads() -> int:
    return lib().orc_num_threads()
