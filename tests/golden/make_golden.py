"""Generates tests/golden/golden.json by running the reference's own relight + mesher templates,
compiled from the reference sources by oracle/Makefile.ref, on every case of tests/cases.py.

Run where the reference sources are present:  python tests/golden/make_golden.py
The fixture holds digests only (inputs are regenerated from their seeds and checked by digest).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

from hypercraft_gb300.build import build  # noqa: E402
from oracle import bind  # noqa: E402
import cases  # noqa: E402


def registry_digest(reg: dict) -> dict:
    out = {}
    for k in ("tex", "transparency", "light", "collision"):
        out[k] = hashlib.sha256(np.ascontiguousarray(reg[k]).tobytes()).hexdigest()
    # custom meshes by content: per raw value the face records (empty for none, "flow" for dynamic)
    h = hashlib.sha256()
    for raw in range(65536):
        key = int(reg["mesh_key"][raw])
        if key == 0:
            h.update(b"-")
        elif key == 0xFFFF:
            h.update(b"flow")
        else:
            h.update(reg["meshes"][key - 1].tobytes())
    out["custom_meshes"] = h.hexdigest()
    return out


def main():
    build()
    ref = bind.reference()
    if ref is None:
        raise SystemExit("reference sources not present")
    golden = {"registry": registry_digest(bind.reference_registry()), "cases": {}}
    for name, make in cases.CASES.items():
        b, h = make()
        meshes = ref.mesh_chunk(b, h)
        light = ref.relight_window(b, h)
        golden["cases"][name] = {
            "input": cases.input_digest(b, h),
            "meshes": cases.mesh_digest(meshes),
            "mesh_count": len(meshes),
            "quads": sum(len(m.vertices) for m in meshes) // 4,
            "light62": hashlib.sha256(light.tobytes()).hexdigest(),
            "light34": hashlib.sha256(cases.light34_from_window(light).tobytes()).hexdigest(),
        }
        print(name, golden["cases"][name]["mesh_count"], golden["cases"][name]["quads"])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
