"""Loader for the reference's scene format: the akari_scenegraph JSON (camera, instances, geometries,
materials as shader-node graphs, buffers / buffer views) plus its binary buffer
(crates/akari_render/src/load.rs:64-700, crates/akari_scenegraph/src/{scene,shader}.rs).

What the GPU path needs from a scene is extracted here on the host:
  * triangles in world space (mesh buffer views: vertices [f32; 3], indices [u32; 3], per-triangle
    material slots u32, load.rs:481-530; instance transforms as row-major 4x4 matrices or TRS in the
    Akari / Blender coordinate systems, scene.rs:31-60);
  * the camera (perspective TRS; camera space looks down -z and `fov` spans the longer image side,
    camera/mod.rs:129-151) as a look-at sty_camera;
  * materials: the surface under the style wrappers (principled -> STY_MAT_PRINCIPLED, the
    reference's principled closure with the node's roughness, metallic, ior, transmission,
    specular and coat inputs, principled.rs:118-330; glass -> STY_MAT_GLASS, glass.rs:13-44;
    diffuse -> Lambert; emission -> emitter, the
    mesh lights of load.rs:95-128); constant inputs only -- textured inputs (and normal maps) fall
    back to constants and are listed in `warnings`;
  * the style graphs: for each style index s = 0..3 the ordered list of style nodes the graph
    applies (every sty_* node applies its inner surface's stylization first, then its own:
    svm/surface/mod.rs:275-285, 573-585; sty_enable_if follows `surface` when the path's style
    index is `idx`, else its `else` branch or nothing, mod.rs:933-976, svm/compiler.rs:459-476;
    sty_set_idx sets the index for the rest of the path), turned into sty_style_program entries.
    Palette entries are "0xRRGGBB" -> (R, G, B) / 255 (compiler.rs:420-449).
"""
from __future__ import annotations

import json
import math
import pathlib
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .scene import MAT_DIFFUSE, MAT_GLASS, MAT_PRINCIPLED, camera, glass, material, principled


class UnsupportedNode(ValueError):
    pass


# ---------------------------------------------------------------- constant node inputs
def _node(nodes, ref):
    if ref is None:
        return None
    return nodes[ref["id"]] if isinstance(ref, dict) else nodes[ref]


def const_float(nodes, ref, default=None):
    n = _node(nodes, ref)
    if n is None:
        return default
    t = n["type"]
    if t == "float":
        return float(n["value"])
    if t in ("rgb", "float3"):
        return float(np.mean(n["value"]))
    if t == "spectral_uplift":
        return const_float(nodes, n["rgb"], default)
    raise UnsupportedNode(f"non-constant float input ({t})")


def const_rgb(nodes, ref, default=None):
    n = _node(nodes, ref)
    if n is None:
        return default
    t = n["type"]
    if t in ("rgb", "float3"):
        return tuple(float(v) for v in n["value"])
    if t == "float":
        return (float(n["value"]),) * 3
    if t == "spectral_uplift":
        return const_rgb(nodes, n["rgb"], default)
    raise UnsupportedNode(f"non-constant colour input ({t})")


def _palette_rgb(s: str):
    x = int(s[2:] if s.lower().startswith("0x") else s, 16)
    return ((x >> 16) & 0xFF) / 255.0, ((x >> 8) & 0xFF) / 255.0, (x & 0xFF) / 255.0


# ---------------------------------------------------------------- style graphs
STYLE_TYPES = {"sty_toon", "sty_color_palette", "sty_8bit", "sty_saturation_adjust", "sty_saturation_adjust_rex",
               "sty_enable_if", "sty_set_idx", "sty_hue_shift", "sty_half_tone"}


def style_ops(nodes, node_id, s: int):
    """Style nodes the graph rooted at `node_id` applies for style index `s`, innermost first."""
    n = nodes[node_id]
    t = n["type"]
    if t == "output":
        return style_ops(nodes, n["node"]["id"], s)
    if t not in STYLE_TYPES:
        return []  # a BSDF / emission / null surface leaves the colour as it is
    if t == "sty_enable_if":
        if s == int(n["idx"]):
            return style_ops(nodes, n["surface"]["id"], s)
        e = n.get("else")
        return style_ops(nodes, e["id"], s) if e else []
    inner = style_ops(nodes, n["surface"]["id"], s)
    if t == "sty_set_idx":
        return inner
    if t == "sty_toon":
        return inner + [abi.toon(const_float(nodes, n["color_band_width"]))]
    if t == "sty_color_palette":
        cols = [_palette_rgb(c) for c in n["palette"]]
        return inner + [abi.palette(cols, indirect_scale=const_float(nodes, n.get("indirect_scale"), 1.0),
                                    gamma=const_float(nodes, n.get("gamma"), 1.0))]
    if t == "sty_8bit":
        return inner + [abi.eight_bit(const_float(nodes, n.get("indirect_scale"), 1.0))]
    if t == "sty_saturation_adjust":
        return inner + [abi.sat_adjust(const_float(nodes, n["power"]),
                                       const_float(nodes, n.get("indirect_scale"), 1.0))]
    if t == "sty_saturation_adjust_rex":
        return inner + [abi.sat_rex(const_float(nodes, n["blend"]))]
    if t == "sty_half_tone":
        m = trs_matrix(n["trs"])
        return inner + [abi.half_tone(const_float(nodes, n["radius_scale"]), const_float(nodes, n["radius"]),
                                      const_float(nodes, n["grid_distance"]), const_rgb(nodes, n["dark_tone"]),
                                      const_rgb(nodes, n["light_tone"]),
                                      indirect_scale=const_float(nodes, n["indirect_scale"]),
                                      blend=const_float(nodes, n["blend"]), max_depth=int(n["max_depth"]),
                                      affine=m.tolist())]
    raise UnsupportedNode(f"style node {t} has no GPU counterpart")


def set_style_index(nodes, node_id):
    """The index a sty_set_idx on the material's surface chain assigns, or -1."""
    n = nodes[node_id]
    t = n["type"]
    if t == "output":
        return set_style_index(nodes, n["node"]["id"])
    if t == "sty_set_idx":
        return int(n["idx"])
    if t in STYLE_TYPES and "surface" in n:
        return set_style_index(nodes, n["surface"]["id"])
    return -1


def base_surface(nodes, node_id):
    """The surface under the style wrappers (through enable_if's `surface`)."""
    n = nodes[node_id]
    t = n["type"]
    if t == "output":
        return base_surface(nodes, n["node"]["id"])
    if t in STYLE_TYPES:
        return base_surface(nodes, n["surface"]["id"])
    if t == "mix":
        return base_surface(nodes, n["first"]["id"])
    return node_id


def output_id(mat) -> str:
    g = mat["shader"]
    nodes = g["nodes"]
    out = g.get("output")
    if isinstance(out, dict):
        return out["id"]
    if isinstance(out, str):
        return out
    for k, n in nodes.items():
        if n["type"] == "output":
            return k
    raise ValueError("material without an output node")


@dataclass
class LoadedMaterial:
    name: str
    kind: int
    albedo: tuple
    alpha: float
    emission: tuple
    ops: list  # per style index: list of StyleNode
    set_style: int
    warnings: list = field(default_factory=list)
    params: dict = field(default_factory=dict)  # principled inputs (scene.principled keywords)


def convert_material(name, mat) -> LoadedMaterial:
    nodes = mat["shader"]["nodes"]
    out = output_id(mat)
    warn = []
    base = nodes[base_surface(nodes, out)]
    t = base["type"]

    def rgb(ref, default):
        try:
            return const_rgb(nodes, ref, default)
        except UnsupportedNode as e:
            warn.append(f"{name}: {e}; using {default}")
            return default

    def flt(ref, default):
        try:
            return const_float(nodes, ref, default)
        except UnsupportedNode as e:
            warn.append(f"{name}: {e}; using {default}")
            return default

    kind, albedo, alpha, emission, params = MAT_DIFFUSE, (0.5, 0.5, 0.5), 1.0, (0.0, 0.0, 0.0), {}
    if t == "principled":
        kind = MAT_PRINCIPLED
        albedo = rgb(base.get("base_color"), (0.5, 0.5, 0.5))
        r = flt(base.get("roughness"), 0.5)
        alpha = max(r * r, 1e-4)
        params = dict(roughness=r, metallic=flt(base.get("metallic"), 0.0), ior=flt(base.get("ior"), 1.45),
                      transmission=flt(base.get("transmission_weight"), 0.0),
                      specular_ior_level=flt(base.get("specular_ior_level"), 0.5),
                      specular_tint=rgb(base.get("specular_tint"), (1.0, 1.0, 1.0)),
                      coat_weight=flt(base.get("coat_weight"), 0.0), coat_roughness=flt(base.get("coat_roughness"), 0.03),
                      coat_ior=flt(base.get("coat_ior"), 1.5), coat_tint=rgb(base.get("coat_tint"), (1.0, 1.0, 1.0)))
        if base.get("normal") is not None and _node(nodes, base.get("normal")) is not None and \
                _node(nodes, base.get("normal")).get("type") == "normal_map":
            warn.append(f"{name}: normal map ignored (flat shading)")
        strength = flt(base.get("emission_strength"), 0.0)
        if strength and strength > 0:
            e = rgb(base.get("emission_color"), (0.0, 0.0, 0.0))
            emission = tuple(c * strength for c in e)
    elif t == "glass":  # svm/compiler.rs:249-263 -> glass.rs
        kind = MAT_GLASS
        albedo = rgb(base.get("color"), (1.0, 1.0, 1.0))
        r = flt(base.get("roughness"), 0.0)
        alpha = max(r * r, 1e-4)
        params = dict(roughness=r, ior=flt(base.get("ior"), 1.5))
    elif t == "diffuse":
        albedo = rgb(base.get("color"), (0.5, 0.5, 0.5))
    elif t == "emission":
        e = rgb(base.get("color"), (1.0, 1.0, 1.0))
        st = flt(base.get("strength"), 1.0)
        albedo, emission = (0.0, 0.0, 0.0), tuple(c * st for c in e)
    elif t == "null":
        albedo = (0.0, 0.0, 0.0)
    else:
        warn.append(f"{name}: surface {t} mapped to a grey Lambert")
    ops = [style_ops(nodes, out, s) for s in range(4)]
    for s, o in enumerate(ops):
        if len(o) > abi.STY_STYLE_MAX_NODES:
            raise UnsupportedNode(f"{name}: style index {s} applies {len(o)} nodes (max {abi.STY_STYLE_MAX_NODES})")
    return LoadedMaterial(name, kind, albedo, alpha, emission, ops, set_style_index(nodes, out), warn, params)


def _program_key(nodes):
    return tuple((n.kind, n.depth_mask, n.n, tuple(round(float(x), 9) for x in n.p[: 60])) for n in nodes)


def build_style_table(mats):
    """Deduplicated style programs and each material's style[4] slot indices (-1: no node)."""
    table, index, slots = [], {}, []
    for m in mats:
        sl = []
        for ops in m.ops:
            if not ops:
                sl.append(-1)
                continue
            k = _program_key(ops)
            if k not in index:
                index[k] = len(table)
                table.append(abi.style_program(ops))
            sl.append(index[k])
        slots.append(tuple(sl))
    return table, slots


# ---------------------------------------------------------------- transforms and camera
def _rot(axis, a):
    c, s = math.cos(a), math.sin(a)
    x, y, z = axis
    R = np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                  [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                  [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])
    M = np.eye(4)
    M[:3, :3] = R
    return M


def trs_matrix(trs, is_camera=False):
    """TRS::to_matrix (scene.rs:31-60): scale (not for cameras), rotations, translation; the
    Blender system maps (x, y, z) -> (x, z, -y) and turns cameras to look down -z."""
    t, r, s = (np.asarray(trs[k], dtype=np.float64) for k in ("translation", "rotation", "scale"))
    cs = trs.get("coordinate_system", "Akari")
    M = np.eye(4)
    if not is_camera:
        M = np.diag([s[0], s[1], s[2], 1.0]) @ M
    T = np.eye(4)
    if cs == "Akari":
        M = _rot((0, 0, 1), r[2]) @ M
        M = _rot((1, 0, 0), r[0]) @ M
        M = _rot((0, 1, 0), r[1]) @ M
        T[:3, 3] = t
    elif cs == "Blender":
        if is_camera:
            M = _rot((1, 0, 0), -math.pi / 2) @ M
        M = _rot((1, 0, 0), r[0]) @ M
        M = _rot((0, 0, 1), -r[1]) @ M
        M = _rot((0, 1, 0), r[2]) @ M
        T[:3, 3] = (t[0], t[2], -t[1])
    else:
        raise ValueError(f"unknown coordinate system {cs}")
    return T @ M


def transform_matrix(tr, is_camera=False):
    if tr["type"] == "matrix":
        return np.asarray(tr["data"], dtype=np.float64)  # rows as written (load.rs:140-143)
    if tr["type"] == "trs":
        return trs_matrix(tr["data"], is_camera)
    raise ValueError(f"unknown transform {tr['type']}")


def apply_film_filter(cam, method_config):
    """The pixel filter of a method config's `film.filter` (PixelFilter, film.rs:20-48: {"type": "box"
    | "gaussian", "radius": r}) set on a loaded camera; no `film.filter` keeps the reference's default,
    the Gaussian of radius 1.5 (film.rs:50-54). Returns the camera."""
    from .scene import FILTER_BOX, FILTER_GAUSSIAN
    filt = ((method_config or {}).get("film") or {}).get("filter") or {"type": "gaussian", "radius": 1.5}
    kinds = {"box": FILTER_BOX, "gaussian": FILTER_GAUSSIAN}
    if filt.get("type") not in kinds:
        raise UnsupportedNode(f"pixel filter {filt.get('type')}")
    cam.filter = kinds[filt["type"]]
    cam.filter_radius = float(filt.get("radius", 1.5))
    return cam


def load_camera(cam, width=None, height=None):
    if cam["type"] != "perspective":
        raise UnsupportedNode(f"camera {cam['type']}")
    d = cam["data"]
    M = transform_matrix(d["transform"], is_camera=True)
    W = int(width or d["sensor_width"])
    H = int(height or d["sensor_height"])
    eye = M[:3, 3]
    fwd = M[:3, :3] @ np.array([0.0, 0.0, -1.0])
    up = M[:3, :3] @ np.array([0.0, 1.0, 0.0])
    fwd /= np.linalg.norm(fwd)
    up /= np.linalg.norm(up)
    fov = math.radians(float(d["fov"]))
    fov_y = fov if W <= H else 2.0 * math.atan(math.tan(fov / 2.0) * H / W)
    return camera(tuple(eye), tuple(eye + fwd), tuple(up), fov_y=math.degrees(fov_y), width=W, height=H)


# ---------------------------------------------------------------- the whole scene
def _buffer_reader(graph, base_dir, bin_paths):
    cache = {}

    def view(ref):
        bv = graph["buffer_views"][ref["id"]]
        bid = bv["buffer"]["id"]
        if bid not in cache:
            b = graph["buffers"][bid]
            p = bin_paths.get(bid) if bin_paths else None
            if p is None:
                p = pathlib.Path(b["path"])
                if not p.is_absolute() or not p.exists():
                    p = pathlib.Path(base_dir) / pathlib.Path(b["path"]).name
            cache[bid] = np.memmap(p, dtype=np.uint8, mode="r")
        raw = cache[bid]
        o, n = int(bv["offset"]), int(bv["length"])
        if o + n > raw.size:
            raise ValueError(f"buffer view {ref['id']} runs past its buffer")
        return np.asarray(raw[o:o + n])

    return view


def load(path, bin_paths=None, width=None, height=None):
    """Read a scene; returns dict(positions [n, 9] f32, mat_ids u32, materials [SceneMaterial],
    programs [StyleProgram], camera, names, warnings)."""
    if isinstance(path, dict):
        graph, base_dir = path, pathlib.Path(".")
    else:
        graph = json.loads(pathlib.Path(path).read_text())
        base_dir = pathlib.Path(path).parent
    view = _buffer_reader(graph, base_dir, bin_paths or {})
    names = list(graph["materials"].keys())
    loaded = [convert_material(k, graph["materials"][k]) for k in names]
    table, slots = build_style_table(loaded)
    def build(i, m):
        if m.kind == MAT_PRINCIPLED:
            return principled(m.albedo, emission=m.emission, style=slots[i], set_style=m.set_style, **m.params)
        if m.kind == MAT_GLASS:
            return glass(m.albedo, emission=m.emission, style=slots[i], set_style=m.set_style, **m.params)
        return material(m.kind, m.albedo, m.alpha, m.emission, slots[i], m.set_style)
    mats = [build(i, m) for i, m in enumerate(loaded)]
    mindex = {k: i for i, k in enumerate(names)}
    tris, mids = [], []
    for iname, inst in graph["instances"].items():
        geo = graph["geometries"][inst["geometry"]["id"]]
        if geo["type"] != "mesh":
            raise UnsupportedNode(f"geometry {geo['type']}")
        v = view(geo["vertices"]).view(np.float32).reshape(-1, 3).astype(np.float64)
        idx = view(geo["indices"]).view(np.uint32).reshape(-1, 3)
        slots_t = view(geo["materials"]).view(np.uint32) if geo.get("materials") else np.zeros(1, np.uint32)
        M = transform_matrix(inst["transform"])
        vw = v @ M[:3, :3].T + M[:3, 3]
        t = vw[idx].reshape(-1, 9)
        inst_mats = [mindex[m["id"]] for m in inst["materials"]]
        per = slots_t if slots_t.size == idx.shape[0] else np.zeros(idx.shape[0], np.uint32)
        if per.size and per.max() >= len(inst_mats):
            raise ValueError(f"instance {iname}: material slot out of range")
        tris.append(t)
        mids.append(np.asarray(inst_mats, np.uint32)[per])
    warnings = [w for m in loaded for w in m.warnings]
    return {"positions": np.concatenate(tris).astype(np.float32), "mat_ids": np.concatenate(mids),
            "materials": mats, "programs": table, "camera": load_camera(graph["camera"], width, height),
            "names": names, "warnings": warnings}
