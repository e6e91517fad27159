"""Generates tests/golden/tank_scene.npz from the reference checkout: the
reference's `tank` scene (apps/simulator/src/scene/tank.js:47-83) voxelised
by vsim.voxelize (the restated asset preparation and voxelisers), and the
node positions the reference recorded for it on its own GPU path
(apps/simulator/test/motion-reference/recorded/tank.json, with the script
of apps/simulator/test/motion-reference/scenarios.js:32-35).

Run from the repository root, naming the reference checkout's root:

    python tests/golden/make_tank_fixture.py REFERENCE_ROOT

The OBJ meshes and tank.json are read only here; the tests read the npz.
"""
import base64
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "visionary-sim_gb300"))

from vsim import voxelize as vz  # noqa: E402

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_tank_fixture.py REFERENCE_ROOT")
REF = Path(sys.argv[1])
APP = REF / "apps" / "simulator"

# tank.js:33-36 (JELLY, RUBBER) over material.js:69-77 (DEFAULT_MATERIAL).
DEFAULT = dict(youngs_modulus=1.2e5, poisson_ratio=0.40, density=1000.0, friction=0.4, damping=0.6,
               relaxation=0.012, max_stretch=0.0)
JELLY = dict(DEFAULT, youngs_modulus=1.5e4, poisson_ratio=0.42, density=1050.0, friction=0.35)
RUBBER = dict(DEFAULT, youngs_modulus=4e4, poisson_ratio=0.45, density=1100.0, friction=0.6)


def mesh_body(path, size, position, element_size):
    """factory.js:41-51 with voxelLattice.js:366-371 (mesh branch)."""
    mesh = vz.parse_obj(path.read_text())
    mesh = vz.translate_mesh(vz.normalize_mesh(mesh, size), position)
    return vz.voxelize_mesh(mesh, vz.mesh_bounds(mesh.positions), element_size)


def shape_body(shape, position, element_size):
    """factory.js:63-73 with voxelLattice.js:366-371 (shape branch)."""
    return vz.voxelize_sdf(vz.translate_shape(vz.rest_on_ground(shape), position), element_size)


def main():
    bodies = [
        ("spot", mesh_body(APP / "public/models/spot.obj", 0.17, [-0.15, 0.18, -0.05], 0.0142), JELLY),
        ("suzanne", mesh_body(APP / "public/models/suzanne.obj", 0.15, [0.14, 0.21, 0.06], 0.0125), RUBBER),
        ("torus", shape_body(vz.torus(0.052, 0.022), [0.0, 0.33, 0.0], 0.0124), JELLY),
        ("sphere", shape_body(vz.sphere(0.05), [-0.16, 0.36, 0.09], 0.0112), JELLY),
        ("cube", shape_body(vz.box([0.045, 0.045, 0.045]), [0.17, 0.35, -0.09], 0.0113), RUBBER),
    ]
    rec = json.loads((APP / "test/motion-reference/recorded/tank.json").read_text())
    out = {"names": np.array([b[0] for b in bodies]),
           "dt": np.float64(rec["dt"]), "batch": np.int64(rec["batch"]), "nodes": np.int64(rec["nodes"]),
           "steps": np.array([int(c["step"]) for c in rec["checkpoints"]], np.int64),
           "tank_min": np.array([-0.30, 0.0, -0.20]), "tank_max": np.array([0.30, 0.50, 0.20])}
    for b, (name, grid, mat) in enumerate(bodies):
        out[f"dims{b}"] = np.array(grid.dims, np.int64)
        out[f"origin{b}"] = np.array(grid.origin, np.float64)
        out[f"h{b}"] = np.float64(grid.h)
        out[f"occupancy{b}"] = np.packbits(grid.occupancy)
        out[f"material{b}"] = np.array([mat[k] for k in ("youngs_modulus", "poisson_ratio", "density", "friction",
                                                         "damping", "relaxation", "max_stretch")])
        print(name, grid.dims, int(grid.occupancy.sum()), "cells",
              int(np.prod(np.asarray(grid.dims) + 1)), "node slots")
    for c, cp in enumerate(rec["checkpoints"]):
        out[f"positions{c}"] = np.frombuffer(base64.b64decode(cp["positions"]), np.float32).reshape(-1, 3)
    np.savez_compressed(Path(__file__).with_name("tank_scene.npz"), **out)
    print("nodes", sum(int(np.prod(np.asarray(g.dims) + 1)) for _, g, _ in bodies), "recorded", rec["nodes"])


if __name__ == "__main__":
    main()
