"""The reference's scene format (akari_scenegraph JSON + binary buffer): style graphs of the real
stylized teaser scene (fixture: tests/golden/scene_sty_materials.json, made by
tests/golden/make_scene_fixture.py; its geometry buffer is not available), and a synthetic scene
written in the same format covering meshes, instance transforms, the Blender camera and emitters."""
import json
import math

import numpy as np
import pytest

from conftest import ROOT

FIX = ROOT / "tests" / "golden" / "scene_sty_materials.json"


def _teaser():
    return json.loads(FIX.read_text())


def test_teaser_style_graphs(sty):
    sg, a = sty.scenegraph, sty.abi
    d = _teaser()
    lm = {k: sg.convert_material(k, m) for k, m in d["materials"].items()}
    assert len(lm) == 33
    shapes = {}
    for k, m in lm.items():
        shapes[k] = tuple(tuple((n.kind, n.n) for n in ops) for ops in m.ops)
    pal14_toon = (((a.STY_STYLE_PALETTE, 14),), (), ((a.STY_STYLE_TOON, 0),), ())
    assert sum(s == pal14_toon for s in shapes.values()) == 26
    assert sum(s == ((), ((a.STY_STYLE_PALETTE, 17),), ((a.STY_STYLE_TOON, 0),), ()) for s in shapes.values()) == 2
    assert shapes["Dragon"] == (((a.STY_STYLE_SAT_REX, 0),), (), ((a.STY_STYLE_TOON, 0),), ())
    assert lm["Mirror"].set_style == 1 and lm["Mirror2"].set_style == 2
    assert all(m.set_style == -1 for k, m in lm.items() if k not in ("Mirror", "Mirror2"))
    # parameters are the graph's constants: palette hex -> rgb / 255, the toon band width node
    nodes = d["materials"]["BadBook"]["shader"]["nodes"]
    pal_node = next(n for n in nodes.values() if n["type"] == "sty_color_palette")
    toon_node = next(n for n in nodes.values() if n["type"] == "sty_toon")
    pal = lm["BadBook"].ops[0][0]
    hexes = pal_node["palette"]
    first = int(hexes[0], 16)
    assert pal.p[2:5] == pytest.approx([(first >> 16) / 255, ((first >> 8) & 255) / 255, (first & 255) / 255])
    assert pal.p[1] == pytest.approx(nodes[pal_node["gamma"]["id"]]["value"])
    assert lm["BadBook"].ops[2][0].p[0] == pytest.approx(nodes[toon_node["color_band_width"]["id"]]["value"])
    # emitters (load.rs:95-128): the 3 emission surfaces and the 2 principled surfaces with an
    # emission strength
    emit = sorted(k for k, m in lm.items() if max(m.emission) > 0)
    assert emit == ["Book_tittle", "Flashlight_Glass", "Material_001", "MiniLightLeft", "MiniLightRight"]
    assert lm["MiniLightLeft"].kind == sty.scene.MAT_DIFFUSE and max(lm["MiniLightLeft"].albedo) == 0
    table, slots = sg.build_style_table(list(lm.values()))
    assert 3 <= len(table) <= 8
    for m, sl in zip(lm.values(), slots):
        for s, ops in enumerate(m.ops):
            assert (sl[s] == -1) == (len(ops) == 0)


def test_teaser_camera(sty):
    cam = sty.scenegraph.load_camera(_teaser()["camera"])
    d = _teaser()["camera"]["data"]
    t = d["transform"]["data"]["translation"]
    assert list(cam.eye) == pytest.approx([t[0], t[2], -t[1]], abs=1e-5)  # Blender (x, y, z) -> (x, z, -y)
    fwd = np.array(cam.target) - np.array(cam.eye)
    assert np.linalg.norm(fwd) == pytest.approx(1.0, abs=1e-5)
    assert (cam.width, cam.height) == (d["sensor_width"], d["sensor_height"])
    # the fov spans the longer (horizontal) side
    assert math.degrees(2 * math.atan(math.tan(math.radians(cam.fov_y) / 2) * cam.width / cam.height)) == \
        pytest.approx(d["fov"], rel=1e-5)


def _write_scene(tmp_path):
    """A scene in the reference's format: one quad mesh with two material slots, instanced twice
    (row-major matrix; Akari TRS), an emissive quad, a Blender-TRS camera."""
    quad_v = np.array([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], np.float32)
    quad_i = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    slots = np.array([0, 1], np.uint32)
    light_v = np.array([[0, 2, 0], [1, 2, 0], [1, 2, 1], [0, 2, 1]], np.float32)
    light_i = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    blobs, views = [], {}
    off = 0
    for name, arr in (("qv", quad_v), ("qi", quad_i), ("qm", slots), ("lv", light_v), ("li", light_i)):
        b = arr.tobytes()
        views[name] = {"buffer": {"id": "Scene"}, "offset": off, "length": len(b)}
        blobs.append(b)
        off += len(b)
    (tmp_path / "Scene.bin").write_bytes(b"".join(blobs))
    f = lambda v: {"type": "float", "value": v}  # noqa: E731
    rgb = lambda v: {"type": "rgb", "value": v, "colorspace": "srgb"}  # noqa: E731
    mats = {
        "Grey": {"shader": {"nodes": {"c": rgb([0.6, 0.6, 0.6]), "d": {"type": "diffuse", "color": {"id": "c"}},
                                      "t": {"type": "sty_toon", "surface": {"id": "d"}, "color_band_width": {"id": "w"}},
                                      "w": f(0.25), "e": {"type": "sty_enable_if", "surface": {"id": "t"}, "idx": 0},
                                      "o": {"type": "output", "node": {"id": "e"}}}, "output": "o"}},
        "Metal": {"shader": {"nodes": {"c": rgb([0.9, 0.7, 0.4]), "r": f(0.5),
                                       "p": {"type": "principled", "base_color": {"id": "c"}, "roughness": {"id": "r"}},
                                       "o": {"type": "output", "node": {"id": "p"}}}, "output": "o"}},
        "Lamp": {"shader": {"nodes": {"c": rgb([1.0, 0.9, 0.8]), "s": f(5.0),
                                      "m": {"type": "emission", "color": {"id": "c"}, "strength": {"id": "s"}},
                                      "o": {"type": "output", "node": {"id": "m"}}}, "output": "o"}},
    }
    graph = {
        "camera": {"type": "perspective", "data": {
            "transform": {"type": "trs", "data": {"translation": [0.5, -3.0, 1.0], "rotation": [math.pi / 2, 0, 0],
                                                  "scale": [1, 1, 1], "coordinate_system": "Blender"}},
            "fov": 60.0, "focal_distance": 10.0, "fstop": 2.8, "sensor_width": 64, "sensor_height": 48,
            "depth_of_field": False}},
        "instances": {
            "floor": {"geometry": {"id": "quad"}, "materials": [{"id": "Grey"}, {"id": "Metal"}],
                      "transform": {"type": "matrix", "data": [[2, 0, 0, -0.5], [0, 1, 0, 0], [0, 0, 2, -0.5],
                                                               [0, 0, 0, 1]]}},
            "floor2": {"geometry": {"id": "quad"}, "materials": [{"id": "Metal"}, {"id": "Grey"}],
                       "transform": {"type": "trs", "data": {"translation": [0, 0.5, 0], "rotation": [0, 0, 0],
                                                             "scale": [1, 1, 1], "coordinate_system": "Akari"}}},
            "lamp": {"geometry": {"id": "light"}, "materials": [{"id": "Lamp"}],
                     "transform": {"type": "matrix", "data": np.eye(4).tolist()}},
        },
        "geometries": {
            "quad": {"type": "mesh", "vertices": {"id": "qv"}, "indices": {"id": "qi"}, "materials": {"id": "qm"}},
            "light": {"type": "mesh", "vertices": {"id": "lv"}, "indices": {"id": "li"}},
        },
        "materials": mats,
        "lights": {},
        "buffers": {"Scene": {"type": "path", "path": "/elsewhere/Scene.bin", "length": off}},
        "buffer_views": views,
    }
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(graph))
    return p


def test_synthetic_scene_load(sty, tmp_path):
    sc = sty.scenegraph.load(_write_scene(tmp_path))
    pos, mids, mats = sc["positions"].reshape(-1, 3, 3), sc["mat_ids"], sc["materials"]
    assert pos.shape == (6, 3, 3)
    # floor: matrix scale 2 and offset (-0.5, 0, -0.5); first triangle (0, 2, 1)
    np.testing.assert_allclose(pos[0], [[-0.5, 0, -0.5], [1.5, 0, 1.5], [1.5, 0, -0.5]], atol=1e-6)
    names = sc["names"]
    assert [names[m] for m in mids] == ["Grey", "Metal", "Metal", "Grey", "Lamp", "Lamp"]
    np.testing.assert_allclose(pos[2, 0], [0, 0.5, 0], atol=1e-6)  # Akari TRS translation
    grey, metal, lamp = (mats[names.index(k)] for k in ("Grey", "Metal", "Lamp"))
    assert metal.kind == sty.scene.MAT_PRINCIPLED and metal.roughness == pytest.approx(0.5)
    assert metal.alpha == pytest.approx(0.25) and metal.ior == pytest.approx(1.45) and metal.metallic == 0.0
    assert list(lamp.emission) == pytest.approx([5.0, 4.5, 4.0])
    assert grey.style[0] >= 0 and list(grey.style)[1:] == [-1, -1, -1]
    assert sc["programs"][grey.style[0]].nodes[0].kind == sty.abi.STY_STYLE_TOON
    cam = sc["camera"]
    assert list(cam.eye) == pytest.approx([0.5, 1.0, 3.0])  # Blender (0.5, -3, 1) -> (0.5, 1, 3)
    assert (np.array(cam.target) - np.array(cam.eye)).tolist() == pytest.approx([0, 0, -1], abs=1e-6)
    assert cam.fov_y == pytest.approx(math.degrees(2 * math.atan(math.tan(math.radians(30)) * 48 / 64)))


def test_synthetic_scene_rejects_bad_slots(sty, tmp_path):
    p = _write_scene(tmp_path)
    g = json.loads(p.read_text())
    g["instances"]["floor"]["materials"] = [{"id": "Grey"}]  # slot 1 has no material
    with pytest.raises(ValueError):
        sty.scenegraph.load(g, bin_paths={"Scene": tmp_path / "Scene.bin"})


@pytest.mark.gpu
def test_synthetic_scene_renders(sty, cuda, tmp_path):
    sc = sty.scenegraph.load(_write_scene(tmp_path))
    scene = sty.scene.Scene(sc["positions"], sc["mat_ids"], sc["materials"], sc["camera"])
    cfg = sty.scene.render_config(max_depth=3, branch=4, radius_scale=(2.0,), reuse=(16,), seed=1)
    film, nv = scene.render(cfg, sc["programs"])
    img = film.cpu().numpy()
    assert nv > 0 and np.isfinite(img).all() and img.mean() > 0


def test_film_filter_from_method_config(sty):
    """film.filter of a method config (the teaser configs select {"type": "gaussian", "radius": 1.5})
    sets the camera's pixel filter; no entry keeps the reference's default Gaussian of radius 1.5."""
    sg, sc = sty.scenegraph, sty.scene
    cam = sc.camera((0, 0, 1), (0, 0, 0))
    assert cam.filter == sc.FILTER_BOX
    sg.apply_film_filter(cam, {"film": {"filter": {"type": "gaussian", "radius": 1.5}}})
    assert cam.filter == sc.FILTER_GAUSSIAN and abs(cam.filter_radius - 1.5) < 1e-7
    sg.apply_film_filter(cam, {"film": {"filter": {"type": "box", "radius": 0.5}}})
    assert cam.filter == sc.FILTER_BOX and abs(cam.filter_radius - 0.5) < 1e-7
    sg.apply_film_filter(cam, {})
    assert cam.filter == sc.FILTER_GAUSSIAN and abs(cam.filter_radius - 1.5) < 1e-7
    import pytest
    with pytest.raises(sg.UnsupportedNode):
        sg.apply_film_filter(cam, {"film": {"filter": {"type": "mitchell"}}})
