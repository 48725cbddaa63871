"""Writes tests/golden/scene_sty_materials.json from the reference's stylized teaser scene
(scenes/veach-ajar-sty-v2/scene-sty.json): its camera and every material's shader graph, pruned to
the nodes reachable from the material's output node. Usage: python make_scene_fixture.py
<reference checkout> (or set STY_REFERENCE); the geometry buffer Scene.bin is not needed and not
read."""
import json
import os
import pathlib
import sys


def _source() -> pathlib.Path:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STY_REFERENCE")
    if not root:
        sys.exit("usage: make_scene_fixture.py <reference checkout>  (or set STY_REFERENCE)")
    return pathlib.Path(root) / "scenes/veach-ajar-sty-v2/scene-sty.json"


OUT = pathlib.Path(__file__).with_name("scene_sty_materials.json")


def reachable(nodes, root):
    seen, stack = set(), [root]
    while stack:
        k = stack.pop()
        if k in seen or k not in nodes:
            continue
        seen.add(k)
        def refs(v):
            if isinstance(v, dict):
                if set(v.keys()) == {"id"}:
                    yield v["id"]
                else:
                    for x in v.values():
                        yield from refs(x)
            elif isinstance(v, list):
                for x in v:
                    yield from refs(x)
        stack.extend(refs({kk: vv for kk, vv in nodes[k].items() if kk != "type"}))
    return seen


def main():
    g = json.loads(_source().read_text())
    mats = {}
    for name, m in g["materials"].items():
        nodes = m["shader"]["nodes"]
        out = next(k for k, n in nodes.items() if n["type"] == "output")
        keep = reachable(nodes, out)
        mats[name] = {"shader": {"nodes": {k: nodes[k] for k in sorted(keep)}, "output": out}}
    OUT.write_text(json.dumps({"camera": g["camera"], "materials": mats}, separators=(",", ":"), sort_keys=True))
    print(OUT, OUT.stat().st_size, "bytes,", len(mats), "materials")


if __name__ == "__main__":
    main()
