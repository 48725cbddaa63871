"""Scenes, the wavefront tracer and the end-to-end NL-PF render (sty_scene_*, sty_pf_render).

Procedural scenes stand in for the reference's scene files (its teaser geometry is not
available): the Cornell box of the plain NL-PF workload and an emissive "furnace" box whose
radiance is known in closed form.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .abi import check, lib

MAT_DIFFUSE = 0
MAT_GGX = 1
MAT_PRINCIPLED = 2
MAT_GLASS = 3
NRC_SAMPLES_TRAIN = 0
NRC_SAMPLES_QUERY = 1
NRC_ROWS_REF = 0
NRC_ROWS_SPHERICAL = 1


class SceneMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("albedo", C.c_float * 3), ("alpha", C.c_float), ("emission", C.c_float * 3),
                ("style", C.c_int32 * 4), ("set_style", C.c_int32),
                ("roughness", C.c_float), ("metallic", C.c_float), ("ior", C.c_float), ("transmission", C.c_float),
                ("specular_ior_level", C.c_float), ("specular_tint", C.c_float * 3), ("coat_weight", C.c_float),
                ("coat_roughness", C.c_float), ("coat_ior", C.c_float), ("coat_tint", C.c_float * 3)]


FILTER_BOX = 0
FILTER_GAUSSIAN = 1
PF_MODE_REF = 0
PF_MODE_SCREEN = 1


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("fov_y", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32), ("filter_radius", C.c_float), ("filter", C.c_int32)]


class RenderConfig(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("branch", C.c_uint32), ("repeats", C.c_uint32),
                ("radius_scale", C.c_float * 16), ("n_radius_scale", C.c_uint32), ("reuse", C.c_uint32 * 16),
                ("n_reuse", C.c_uint32), ("smis", C.c_int32), ("cluster", C.c_int32),
                ("disable_flag_check", C.c_int32), ("no_first_hit_stylization", C.c_int32),
                ("has_scene_bounds", C.c_int32), ("scene_bounds", C.c_float * 6), ("seed", C.c_uint64),
                ("mode", C.c_int32), ("screen_style", C.c_int32), ("screen", abi.PfScreenParams)]


class RecordsOut(C.Structure):
    _fields_ = [("pos", C.c_void_p * 3), ("nrm", C.c_void_p * 3), ("rad", C.c_void_p * 3), ("thr", C.c_void_p * 3),
                ("valid", C.c_void_p), ("prim", C.c_void_p)]


class NrcRenderConfig(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("training_iters", C.c_uint32), ("batches_per_iter", C.c_uint32),
                ("training_paths", C.c_uint32), ("repeats", C.c_uint32), ("per_level_training", C.c_uint32),
                ("no_first_hit_stylization", C.c_int32), ("learn_stylized_radiance", C.c_int32),
                ("final_gather", C.c_uint32), ("reserved", C.c_uint32), ("seed", C.c_uint64)]


class PfNrcConfig(C.Structure):
    _fields_ = [("pf", RenderConfig), ("nrc", NrcRenderConfig), ("cache_depth", C.c_uint32), ("reserved", C.c_uint32)]


class NrcRenderStats(C.Structure):
    _fields_ = [("training_rows", C.c_uint64), ("inference_queries", C.c_uint64), ("last_loss", C.c_float),
                ("reserved", C.c_uint32)]


class BrptConfig(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("n_levels", C.c_uint32), ("inner_samples", C.c_uint32 * 8),
                ("repeats", C.c_uint32), ("vram_mb", C.c_uint32), ("seed", C.c_uint64),
                ("first_repeat", C.c_uint32), ("reserved", C.c_uint32)]


class BrptStats(C.Structure):
    _fields_ = [("vertices", C.c_uint64), ("slots", C.c_uint64), ("passes", C.c_uint64),
                ("pixels_per_pass", C.c_uint64), ("max_pass_slots", C.c_uint64)]


def brpt_config(max_depth=7, inner_samples=(256, 32, 8, 1), repeats=1, vram_mb=8192, seed=0,
                first_repeat=0) -> BrptConfig:
    """The branching path tracer's configuration (branching_pt.rs Config :77-100; the defaults are
    the reference's). first_repeat: this call's share of a render split over replicas."""
    c = BrptConfig()
    c.max_depth, c.repeats, c.vram_mb, c.seed = max_depth, repeats, vram_mb, seed
    c.first_repeat = first_repeat
    c.n_levels = len(inner_samples)
    for i, v in enumerate(inner_samples):
        c.inner_samples[i] = v
    return c


def nrc_render_config(max_depth=5, training_iters=64, batches_per_iter=16, training_paths=0, repeats=1,
                      per_level_training=0, no_first_hit_stylization=False, learn_stylized_radiance=False,
                      final_gather=0, seed=0) -> NrcRenderConfig:
    c = NrcRenderConfig()
    c.max_depth, c.training_iters, c.batches_per_iter = max_depth, training_iters, batches_per_iter
    c.training_paths, c.repeats, c.per_level_training = training_paths, repeats, per_level_training
    c.no_first_hit_stylization, c.learn_stylized_radiance = int(no_first_hit_stylization), int(learn_stylized_radiance)
    c.final_gather = final_gather
    c.seed = seed
    return c


def material(kind=MAT_DIFFUSE, albedo=(0.75, 0.75, 0.75), alpha=0.3, emission=(0, 0, 0), style=(-1, -1, -1, -1),
             set_style=-1) -> SceneMaterial:
    m = SceneMaterial()
    m.kind = kind
    m.albedo[:] = list(albedo)
    m.alpha = alpha
    m.emission[:] = list(emission)
    m.style[:] = list(style)
    m.set_style = set_style
    m.ior, m.specular_ior_level, m.coat_ior = 1.5, 0.5, 1.5
    m.specular_tint[:] = [1.0, 1.0, 1.0]
    m.coat_tint[:] = [1.0, 1.0, 1.0]
    return m


def principled(base_color=(0.8, 0.8, 0.8), roughness=0.5, metallic=0.0, ior=1.5, transmission=0.0,
               specular_ior_level=0.5, specular_tint=(1, 1, 1), coat_weight=0.0, coat_roughness=0.03, coat_ior=1.5,
               coat_tint=(1, 1, 1), emission=(0, 0, 0), style=(-1, -1, -1, -1), set_style=-1) -> SceneMaterial:
    """The reference's principled BSDF (svm/surface/principled.rs; Blender's Principled BSDF inputs;
    emission = emission colour x strength)."""
    m = material(MAT_PRINCIPLED, base_color, alpha=max(roughness * roughness, 1e-4), emission=emission,
                 style=style, set_style=set_style)
    m.roughness, m.metallic, m.ior, m.transmission = roughness, metallic, ior, transmission
    m.specular_ior_level = specular_ior_level
    m.specular_tint[:] = list(specular_tint)
    m.coat_weight, m.coat_roughness, m.coat_ior = coat_weight, coat_roughness, coat_ior
    m.coat_tint[:] = list(coat_tint)
    return m


def glass(color=(1.0, 1.0, 1.0), ior=1.5, roughness=0.0, emission=(0, 0, 0), style=(-1, -1, -1, -1),
          set_style=-1) -> SceneMaterial:
    """The reference's glass node (svm/surface/glass.rs): rough dielectric reflection and
    transmission, both tinted by `color`."""
    m = material(MAT_GLASS, color, alpha=max(roughness * roughness, 1e-4), emission=emission, style=style,
                 set_style=set_style)
    m.roughness, m.ior = roughness, ior
    return m


def camera(eye, target, up=(0, 1, 0), fov_y=40.0, width=256, height=256, filter_radius=1.0,
           filter=FILTER_BOX) -> Camera:
    """Pinhole camera; `filter` is the pixel filter (FILTER_BOX or FILTER_GAUSSIAN, film.rs:20-48)
    of radius `filter_radius` pixels."""
    c = Camera()
    c.eye[:] = list(eye)
    c.target[:] = list(target)
    c.up[:] = list(up)
    c.fov_y, c.width, c.height, c.filter_radius = fov_y, width, height, filter_radius
    c.filter = filter
    return c


def screen_render_config(max_depth=5, branch=16, repeats=1, radius=8, sigma_pixel=4.0, sigma_pos=0.05,
                         sigma_nrm=0.2, screen_style=0, seed=0) -> RenderConfig:
    """An NL-PF render with the screen-space bilateral filter (STY_PF_MODE_SCREEN): the tracer's
    vertex records of `branch` samples per pixel filtered over a (2 radius + 1)^2 pixel window with
    the program programs[screen_style] (-1: none)."""
    c = render_config(max_depth=max_depth, branch=branch, repeats=repeats, seed=seed)
    c.mode = PF_MODE_SCREEN
    c.screen_style = screen_style
    c.screen.radius, c.screen.sigma_pixel, c.screen.sigma_pos, c.screen.sigma_nrm = (radius, sigma_pixel, sigma_pos,
                                                                                     sigma_nrm)
    return c


def render_config(max_depth=5, branch=16, repeats=1, radius_scale=(5.0,), reuse=(64,), smis=True, cluster=False,
                  disable_flag_check=False, no_first_hit_stylization=False, scene_bounds=None, seed=0) -> RenderConfig:
    c = RenderConfig()
    c.max_depth, c.branch, c.repeats = max_depth, branch, repeats
    for i, v in enumerate(radius_scale):
        c.radius_scale[i] = v
    c.n_radius_scale = len(radius_scale)
    for i, v in enumerate(reuse):
        c.reuse[i] = v
    c.n_reuse = len(reuse)
    c.smis, c.cluster = int(smis), int(cluster)
    c.disable_flag_check, c.no_first_hit_stylization = int(disable_flag_check), int(no_first_hit_stylization)
    if scene_bounds is not None:
        c.has_scene_bounds = 1
        c.scene_bounds[:] = list(scene_bounds[0]) + list(scene_bounds[1])
    c.seed = seed
    return c


def _quad(a, b, c, d):
    """Two triangles (a, b, c), (a, c, d); counter-clockwise seen from the normal side."""
    return [a + b + c, a + c + d]


def _box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    p = lambda x, y, z: [x, y, z]  # noqa: E731
    tris = []
    tris += _quad(p(x0, y0, z1), p(x1, y0, z1), p(x1, y1, z1), p(x0, y1, z1))  # +z
    tris += _quad(p(x1, y0, z0), p(x0, y0, z0), p(x0, y1, z0), p(x1, y1, z0))  # -z
    tris += _quad(p(x1, y0, z1), p(x1, y0, z0), p(x1, y1, z0), p(x1, y1, z1))  # +x
    tris += _quad(p(x0, y0, z0), p(x0, y0, z1), p(x0, y1, z1), p(x0, y1, z0))  # -x
    tris += _quad(p(x0, y1, z1), p(x1, y1, z1), p(x1, y1, z0), p(x0, y1, z0))  # +y
    tris += _quad(p(x0, y0, z0), p(x1, y0, z0), p(x1, y0, z1), p(x0, y0, z1))  # -y
    return tris


def cornell_box(width=256, height=256, style=(-1, -1, -1, -1), light_style=(-1, -1, -1, -1)):
    """Unit Cornell box (y up, open towards +z): 5 diffuse walls (albedo 0.75 grey, left
    0.63/0.065/0.05, right 0.14/0.45/0.09), two axis-aligned boxes of 12 triangles, one 0.25 x 0.25
    area light of radiance 17 under the ceiling. Returns (positions [n, 9], material ids, materials,
    camera)."""
    P = lambda x, y, z: [x, y, z]  # noqa: E731
    tris, mids = [], []

    def add(ts, m):
        tris.extend(ts)
        mids.extend([m] * len(ts))

    add(_quad(P(0, 0, 1), P(1, 0, 1), P(1, 0, 0), P(0, 0, 0)), 0)  # floor (normal +y)
    add(_quad(P(0, 1, 0), P(1, 1, 0), P(1, 1, 1), P(0, 1, 1)), 0)  # ceiling (normal -y)
    add(_quad(P(0, 0, 0), P(1, 0, 0), P(1, 1, 0), P(0, 1, 0)), 0)  # back wall (normal +z)
    add(_quad(P(0, 0, 1), P(0, 0, 0), P(0, 1, 0), P(0, 1, 1)), 1)  # left wall (normal +x)
    add(_quad(P(1, 0, 0), P(1, 0, 1), P(1, 1, 1), P(1, 1, 0)), 2)  # right wall (normal -x)
    add(_box((0.55, 0.0, 0.15), (0.85, 0.3, 0.45)), 0)             # short box
    add(_box((0.15, 0.0, 0.35), (0.45, 0.6, 0.65)), 0)             # tall box
    ly = 1.0 - 1e-3
    add(_quad(P(0.375, ly, 0.375), P(0.625, ly, 0.375), P(0.625, ly, 0.625), P(0.375, ly, 0.625)), 3)  # light, -y
    mats = [material(MAT_DIFFUSE, (0.75, 0.75, 0.75), style=style),
            material(MAT_DIFFUSE, (0.63, 0.065, 0.05), style=style),
            material(MAT_DIFFUSE, (0.14, 0.45, 0.09), style=style),
            material(MAT_DIFFUSE, (0.0, 0.0, 0.0), emission=(17.0, 17.0, 17.0), style=light_style)]
    cam = camera((0.5, 0.5, 2.2), (0.5, 0.5, 0.0), fov_y=36.0, width=width, height=height)
    return np.array(tris, dtype=np.float32), np.array(mids, dtype=np.uint32), mats, cam


def furnace(albedo=0.5, le=1.0, width=32, height=32):
    """Closed unit cube whose 12 inward-facing triangles all emit `le` and reflect `albedo`
    (diffuse): the radiance of every path prefix of depth D is le * sum_{k<=D} albedo^k."""
    tris = _box((0, 0, 0), (1, 1, 1))
    # flip winding so the normals point into the cube
    tris = [t[0:3] + t[6:9] + t[3:6] for t in tris]
    mats = [material(MAT_DIFFUSE, (albedo,) * 3, emission=(le,) * 3)]
    cam = camera((0.5, 0.5, 0.5), (0.5, 0.5, 0.0), fov_y=60.0, width=width, height=height)
    return np.array(tris, dtype=np.float32), np.zeros(len(tris), dtype=np.uint32), mats, cam


def icosphere(subdiv=3):
    """Unit icosphere: the icosahedron with each face split into 4 `subdiv` times, vertices pushed
    to the sphere (20 * 4^subdiv outward-facing triangles). Returns [n, 3, 3] float64."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = np.array([[v[i] for i in face] for face in f], dtype=np.float64)
    tris /= np.linalg.norm(tris, axis=2, keepdims=True)
    for _ in range(subdiv):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.concatenate([np.stack(q, 1) for q in ((a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca))])
    return tris


def icosphere_grid(width=1920, height=1080, n=10, subdiv=3, seed=0, camera_fov=40.0):
    """Neural-cache workload scene: an n x n grid of subdivision-`subdiv` icospheres (radius 0.45,
    spacing 1.2; 1280 triangles each at subdivision 3, 128 000 for the 10 x 10 grid) on a 16 x 16
    ground quad (diffuse 0.5), each sphere GGX with alpha ~ U[0.05, 0.5] and albedo ~ U[0.2, 0.9]^3
    (seeded), one 3 x 3 area light of radiance 12 at height 6. Returns (positions [n, 9], material
    ids, materials, camera)."""
    rng = np.random.default_rng(seed)
    sph = icosphere(subdiv) * 0.45
    tris, mids, mats = [], [], []
    mats.append(material(MAT_DIFFUSE, (0.5, 0.5, 0.5)))
    g = 8.0
    ground = np.array(_quad([-g, 0, g], [g, 0, g], [g, 0, -g], [-g, 0, -g]), dtype=np.float64).reshape(-1, 3, 3)
    tris.append(ground)
    mids += [0, 0]
    for i in range(n):
        for j in range(n):
            c = np.array([(i - (n - 1) / 2) * 1.2, 0.45, (j - (n - 1) / 2) * 1.2])
            tris.append(sph + c)
            mids += [len(mats)] * len(sph)
            mats.append(material(MAT_GGX, tuple(rng.uniform(0.2, 0.9, 3)), alpha=float(rng.uniform(0.05, 0.5))))
    L, y = 1.5, 6.0
    light = np.array(_quad([-L, y, -L], [L, y, -L], [L, y, L], [-L, y, L]), dtype=np.float64).reshape(-1, 3, 3)
    tris.append(light)
    mids += [len(mats)] * 2
    mats.append(material(MAT_DIFFUSE, (0.0, 0.0, 0.0), emission=(12.0, 12.0, 12.0)))
    pos = np.concatenate(tris).reshape(-1, 9).astype(np.float32)
    cam = camera((0.0, 6.5, 10.5), (0.0, 0.3, 0.0), fov_y=camera_fov, width=width, height=height)
    return pos, np.array(mids, dtype=np.uint32), mats, cam


def _grid_quad(o, u, v, nu, nv):
    """A planar quad o + s*u + t*v (s, t in [0, 1]) tessellated into nu x nv cells (2 triangles
    each), counter-clockwise seen from the side u x v points to."""
    o, u, v = (np.asarray(x, dtype=np.float64) for x in (o, u, v))
    s = np.linspace(0.0, 1.0, nu + 1)
    t = np.linspace(0.0, 1.0, nv + 1)
    P = o[None, None] + s[:, None, None] * u[None, None] + t[None, :, None] * v[None, None]
    a, b, c, d = P[:-1, :-1], P[1:, :-1], P[1:, 1:], P[:-1, 1:]
    return np.concatenate([np.stack([a, b, c], 2).reshape(-1, 3, 3), np.stack([a, c, d], 2).reshape(-1, 3, 3)])


def _box_tris(lo, hi, inward=False):
    t = np.array(_box(lo, hi), dtype=np.float64).reshape(-1, 3, 3)
    return t[:, [0, 2, 1]] if inward else t


def room_with_door(width=320, height=180, cell=0.028, door_angle=20.0, seed=0):
    """Full-render workload scene: a 6 x 3 x 4 m room (x: 0..6, y: 0..3 up, z: 0..4) whose walls,
    floor and ceiling are tessellated into `cell`-sized quads (~125 k triangles at 5 cm, ~400 k at
    2.8 cm); a 1 x 2.1 m doorway in the wall x = 6 with a door panel turned `door_angle` degrees about
    its hinge; behind it a 2 m deep corridor whose ceiling holds the only emitter (1 x 2 m, radiance
    40), so most light reaches the room indirectly through the door gap. Furniture: 6 diffuse
    boxes and 8 GGX icospheres (alpha ~ U[0.05, 0.5], albedo ~ U[0.2, 0.9]^3, seeded); walls
    diffuse 0.7, floor GGX alpha 0.3. Style indices: every surface uses program slot 0.
    Returns (positions [n, 9], material ids, materials, camera)."""
    rng = np.random.default_rng(seed)
    tris, mids, mats = [], [], []

    def add(t, m):
        tris.append(np.asarray(t, dtype=np.float64).reshape(-1, 3, 3))
        mids.extend([m] * len(tris[-1]))

    sty0 = (0, -1, -1, -1)
    mats.append(material(MAT_DIFFUSE, (0.7, 0.7, 0.68), style=sty0))            # 0 walls
    mats.append(material(MAT_GGX, (0.55, 0.45, 0.35), alpha=0.3, style=sty0))  # 1 floor
    mats.append(material(MAT_DIFFUSE, (0.6, 0.35, 0.2), style=sty0))           # 2 door / boxes
    mats.append(material(MAT_DIFFUSE, (0.0, 0.0, 0.0), emission=(40.0, 40.0, 40.0), style=sty0))  # 3 light
    n = lambda L: max(1, int(round(L / cell)))  # noqa: E731
    X, Y, Z = 6.0, 3.0, 4.0
    # floor (normal +y) and ceiling (normal -y), room and corridor
    add(_grid_quad([0, 0, 0], [0, 0, Z], [X, 0, 0], n(Z), n(X)), 1)
    add(_grid_quad([0, Y, 0], [X, 0, 0], [0, 0, Z], n(X), n(Z)), 0)
    add(_grid_quad([X, 0, 0], [0, 0, Z], [2, 0, 0], n(Z), n(2)), 1)
    # corridor ceiling with the light in its middle
    add(_grid_quad([X, Y, 0], [2, 0, 0], [0, 0, 1], n(2), n(1)), 0)
    add(_grid_quad([X, Y, 3], [2, 0, 0], [0, 0, 1], n(2), n(1)), 0)
    add(_grid_quad([X, Y, 1], [0.5, 0, 0], [0, 0, 2], n(0.5), n(2)), 0)
    add(_grid_quad([X + 1.5, Y, 1], [0.5, 0, 0], [0, 0, 2], n(0.5), n(2)), 0)
    ly = Y - 1e-3
    add(_quad([X + 0.5, ly, 1], [X + 1.5, ly, 1], [X + 1.5, ly, 3], [X + 0.5, ly, 3]), 3)
    # room walls (inward): z = 0 (normal +z), z = Z (normal -z), x = 0 (normal +x)
    add(_grid_quad([0, 0, 0], [X, 0, 0], [0, Y, 0], n(X), n(Y)), 0)
    add(_grid_quad([X, 0, Z], [-X, 0, 0], [0, Y, 0], n(X), n(Y)), 0)
    add(_grid_quad([0, 0, Z], [0, 0, -Z], [0, Y, 0], n(Z), n(Y)), 0)
    # corridor walls: z = 0, z = Z, x = X + 2 (back)
    add(_grid_quad([X, 0, 0], [2, 0, 0], [0, Y, 0], n(2), n(Y)), 0)
    add(_grid_quad([X + 2, 0, Z], [-2, 0, 0], [0, Y, 0], n(2), n(Y)), 0)
    add(_grid_quad([X + 2, 0, 0], [0, 0, Z], [0, Y, 0], n(Z), n(Y)), 0)
    # the wall x = X around the doorway z in [1.5, 2.5], y in [0, 2.1], one face towards the room (the
    # BSDFs are two-sided, so the corridor sees the same triangles from behind)
    dz0, dz1, dh = 1.5, 2.5, 2.1
    for o, u, v, nu, nv in (([X, 0, 0], [0, 0, dz0], [0, Y, 0], n(dz0), n(Y)),
                            ([X, 0, dz1], [0, 0, Z - dz1], [0, Y, 0], n(Z - dz1), n(Y)),
                            ([X, dh, dz0], [0, 0, dz1 - dz0], [0, Y - dh, 0], n(dz1 - dz0), n(Y - dh))):
        add(_grid_quad(o, u, v, nu, nv), 0)
    # door panel: 1 x 2.1 x 0.04 m, hinged at (X, z = dz0), turned into the room by door_angle
    door = _box_tris((0.0, 0.0, 0.0), (0.04, dh, dz1 - dz0))
    th = np.radians(door_angle)
    R = np.array([[np.cos(th), 0, np.sin(th)], [0, 1, 0], [-np.sin(th), 0, np.cos(th)]])
    door = door @ R.T + np.array([X - 0.04, 0, dz0])
    add(door, 2)
    # furniture
    for k in range(6):
        cx, cz = rng.uniform(0.6, X - 1.2), rng.uniform(0.5, Z - 0.5)
        sx, sy, sz = rng.uniform(0.3, 0.8), rng.uniform(0.3, 1.2), rng.uniform(0.3, 0.8)
        add(_box_tris((cx, 0.0, cz), (cx + sx, sy, cz + sz)), 2)
    sph = icosphere(3)
    for k in range(8):
        r = rng.uniform(0.15, 0.4)
        c = np.array([rng.uniform(0.5, X - 0.8), r, rng.uniform(0.5, Z - 0.5)])
        mats.append(material(MAT_GGX, tuple(rng.uniform(0.2, 0.9, 3)), alpha=float(rng.uniform(0.05, 0.5)),
                             style=sty0))
        add(sph * r + c, len(mats) - 1)
    pos = np.concatenate(tris).reshape(-1, 9).astype(np.float32)
    cam = camera((0.6, 1.6, 2.0), (6.0, 1.1, 2.0), fov_y=60.0, width=width, height=height)
    return pos, np.array(mids, dtype=np.uint32), mats, cam


class Scene:
    def __init__(self, positions: np.ndarray, mat_ids: np.ndarray, materials, cam: Camera):
        self.positions = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 9)
        self.mat_ids = np.ascontiguousarray(mat_ids, dtype=np.uint32)
        self.materials = (SceneMaterial * len(materials))(*materials)
        self.camera = cam
        self.h = C.c_void_p()
        check(lib().sty_scene_create(self.positions.ctypes.data, self.mat_ids.ctypes.data, self.positions.shape[0],
                                     self.materials, len(materials), C.byref(cam), C.byref(self.h)))

    def close(self):
        if self.h:
            lib().sty_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def closest_hit(self, rays):
        """rays: device float32 [n, 8] (o, d, tmin, tmax) -> (prim, t, bary) device tensors."""
        import torch
        n = rays.shape[0]
        prim = torch.empty(n, dtype=torch.int32, device=rays.device)
        t = torch.empty(n, dtype=torch.float32, device=rays.device)
        b = torch.empty((n, 2), dtype=torch.float32, device=rays.device)
        check(lib().sty_scene_closest_hit(self.h, rays.data_ptr(), n, prim.data_ptr(), t.data_ptr(), b.data_ptr(),
                                          None))
        return prim, t, b

    def render(self, cfg: RenderConfig, programs=(), film=None, stream=None):
        """Full NL-PF render; returns (film [H, W, 3] float64 device tensor, vertex count)."""
        import torch
        from .pf import _stream_ptr
        W, H = self.camera.width, self.camera.height
        if film is None:
            film = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        progs = list(programs)
        arr = (abi.StyleProgram * max(1, len(progs)))(*progs) if progs else None
        vc = C.c_uint64()
        check(lib().sty_pf_render(self.h, C.byref(cfg), arr, len(progs), film.data_ptr(), C.byref(vc),
                                  _stream_ptr(stream)))
        return film, vc.value

    def trace_records(self, cfg: RenderConfig, programs=(), with_prim=False, stream=None):
        """The screen-space records a SCREEN-mode render filters (sty_pf_trace_records): returns
        (RecordSet over device planes, prim ids [depths, H, W, branch] or None, vertex count)."""
        import torch
        from .pf import RecordSet, _stream_ptr
        W, H, S, D = self.camera.width, self.camera.height, cfg.branch, cfg.max_depth + 1
        n = D * H * W * S
        planes = torch.empty((12, n), dtype=torch.float32, device="cuda")
        valid = torch.empty(n, dtype=torch.int32, device="cuda")
        prim = torch.empty((D, H, W, S), dtype=torch.int32, device="cuda") if with_prim else None
        ro = RecordsOut()
        for a in range(3):
            ro.pos[a] = planes[a].data_ptr()
            ro.nrm[a] = planes[3 + a].data_ptr()
            ro.rad[a] = planes[6 + a].data_ptr()
            ro.thr[a] = planes[9 + a].data_ptr()
        ro.valid = valid.data_ptr()
        ro.prim = prim.data_ptr() if prim is not None else None
        progs = list(programs)
        arr = (abi.StyleProgram * max(1, len(progs)))(*progs) if progs else None
        vc = C.c_uint64()
        check(lib().sty_pf_trace_records(self.h, C.byref(cfg), arr, len(progs), C.byref(ro), C.byref(vc),
                                         _stream_ptr(stream)))
        return RecordSet(planes, valid, W, H, S, D), prim, vc.value

    def camera_rays(self, branch: int, seed: int = 0, stream=None):
        """Depth-0 rays [W*H*branch, 8] (device) of every path slot (sty_scene_camera_rays)."""
        import torch
        from .pf import _stream_ptr
        n = self.camera.width * self.camera.height * branch
        rays = torch.empty((n, 8), dtype=torch.float32, device="cuda")
        check(lib().sty_scene_camera_rays(self.h, branch, seed, rays.data_ptr(), _stream_ptr(stream)))
        return rays

    def nrc_samples(self, mode: int, spp: int, max_depth: int, layout: int = NRC_ROWS_SPHERICAL, seed: int = 0,
                    capacity: int | None = None, stream=None):
        """NRC rows from the tracer (sty_nrc_samples): returns (inputs [rows, dims], targets
        [rows, 3]) float32 device tensors, dims = 11 (spherical layout) or 20 + max_depth (the
        reference's layout). Query mode gives spp * width * height rows."""
        import torch
        from .pf import _stream_ptr
        W, H = self.camera.width, self.camera.height
        if capacity is None:
            capacity = W * H * spp * (max_depth + 1 if mode == NRC_SAMPLES_TRAIN else 1)
        dims = 11 if layout == NRC_ROWS_SPHERICAL else 20 + max_depth
        x = torch.empty((capacity, dims), dtype=torch.float32, device="cuda")
        y = torch.empty((capacity, 3), dtype=torch.float32, device="cuda")
        cnt = C.c_uint64()
        check(lib().sty_nrc_samples(self.h, mode, layout, spp, max_depth, seed, x.data_ptr(), y.data_ptr(), capacity,
                                    C.byref(cnt), _stream_ptr(stream)))
        return x[:cnt.value], y[:cnt.value]

    def nrc_render(self, net, cfg: NrcRenderConfig, programs=(), film=None, stream=None):
        """The NL-NRC render (sty_nrc_render): trains `net` online on the scene's own paths and
        renders the cache at the first hit. Returns (film [H, W, 3] float64 device tensor, stats)."""
        import torch
        from .pf import _stream_ptr
        W, H = self.camera.width, self.camera.height
        if film is None:
            film = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        progs = list(programs)
        arr = (abi.StyleProgram * max(1, len(progs)))(*progs) if progs else None
        st = NrcRenderStats()
        check(lib().sty_nrc_render(self.h, net.h, C.byref(cfg), arr, len(progs), film.data_ptr(), C.byref(st),
                                   _stream_ptr(stream)))
        return film, st

    def pf_nrc_render(self, net, pf_cfg: RenderConfig, nrc_cfg: NrcRenderConfig, cache_depth: int, programs=(),
                      film=None, stream=None):
        """NL-PF with the neural cache at the path ends (sty_pf_nrc_render): `net` trained by the
        NL-NRC loop of `nrc_cfg`, then the SCREEN-mode render of `pf_cfg` traced to `cache_depth`,
        the cache's prediction there feeding the filter. Returns (film [H, W, 3] float64, stats)."""
        import torch
        from .pf import _stream_ptr
        W, H = self.camera.width, self.camera.height
        if film is None:
            film = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        cfg = PfNrcConfig()
        cfg.pf, cfg.nrc, cfg.cache_depth = pf_cfg, nrc_cfg, cache_depth
        progs = list(programs)
        arr = (abi.StyleProgram * max(1, len(progs)))(*progs) if progs else None
        st = NrcRenderStats()
        check(lib().sty_pf_nrc_render(self.h, net.h, C.byref(cfg), arr, len(progs), film.data_ptr(), C.byref(st),
                                      _stream_ptr(stream)))
        return film, st

    def brpt_render(self, cfg: BrptConfig, programs=(), film=None, stream=None):
        """The branching path tracer (sty_brpt_render): returns (film [H, W, 3] float64 device
        tensor, stats)."""
        import torch
        from .pf import _stream_ptr
        W, H = self.camera.width, self.camera.height
        if film is None:
            film = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        progs = list(programs)
        arr = (abi.StyleProgram * max(1, len(progs)))(*progs) if progs else None
        st = BrptStats()
        check(lib().sty_brpt_render(self.h, C.byref(cfg), arr, len(progs), film.data_ptr(), C.byref(st),
                                    _stream_ptr(stream)))
        return film, st
