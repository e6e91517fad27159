"""The reference's own recorded trajectory: the `tank` scene (two meshes and
three analytic shapes falling into a tank and onto each other) as the
reference recorded it on its GPU path (RTX 4090, WebGPU;
apps/simulator/test/motion-reference/recorded/tank.json), replayed here with
the recorded script -- 1440 fixed steps in frames of at most 24, node
positions read at steps 0, 480, 960 and 1440.

What must hold exactly: the node count and every rest position (the
voxelisers and lattice builder are restated operation by operation), and
the step duration the CFL rule picks. What can only agree closely: the
motion, because the reference's recording is one GPU's rounding -- its own
README measures 0.1 / 1.5 / 2.1 mm between two GPUs at the same commit at
steps 480 / 960 / 1440, growing through contact. The bounds below are
those of that cross-GPU spread.

The CPU test replays the float oracle (pinning it to the reference's own
run); the GPU test replays libvsim through the C ABI and also requires
equality with the oracle at every checkpoint.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

FIXTURE = Path(__file__).with_name("golden") / "tank_scene.npz"
# Largest node distance allowed from the recording at steps 0, 480, 960, 1440.
BOUND_M = (0.0, 0.5e-3, 5e-3, 5e-3)


def _scene():
    import vsim.scenes as sc

    return sc.tank_scene(FIXTURE), np.load(FIXTURE)


def _cfl_step(scene):
    """stableStepDuration of the fastest body's wave rate (simulator.js:162-186)."""
    from vsim import _ffi
    from vsim.scenes import Descs

    lib = _ffi.lib()
    descs = Descs(scene)
    rate = max(lib.vsim_wave_speed(C.byref(descs.bodies[b].material)) / b_.h for b, b_ in enumerate(scene.bodies))
    out = C.c_double()
    assert lib.vsim_stable_step_duration(rate, C.byref(out)) == 0
    return out.value


def _furthest(a, b):
    return float(np.max(np.linalg.norm(a.astype(np.float64) - b.astype(np.float64), axis=1)))


def _replay(sim, z, read):
    """The recorded script: checkpoints after 0, 480, 960, 1440 steps, frames
    of at most `batch` steps. Returns the largest node distance from the
    recording at each checkpoint, and the positions read."""
    batch = int(z["batch"])
    done, distances, seen = 0, [], []
    for c, step in enumerate(z["steps"]):
        while done < step:
            n = min(batch, int(step) - done)
            sim.dispatch(n)
            done += n
        pos = read()
        seen.append(pos)
        distances.append(_furthest(pos, z[f"positions{c}"]))
    return distances, seen


def test_tank_cells_and_step_match_the_recording():
    scene, z = _scene()
    assert sum(int(np.prod(np.asarray(b.cell_dims) + 1)) for b in scene.bodies) == int(z["nodes"]) == 14104
    assert _cfl_step(scene) == float(z["dt"])


def test_oracle_replays_the_recorded_tank_run():
    import pyoracle

    scene, z = _scene()
    orc = pyoracle.Oracle(scene, 32)
    orc.set_step_duration(float(z["dt"]))
    distances, _ = _replay(orc, z, lambda: orc.state()[0][:, :3].copy())
    assert distances[0] == 0.0, "rest positions differ from the recording"
    for d, bound, step in zip(distances, BOUND_M, z["steps"]):
        assert d <= bound, f"step {step}: {1e3 * d:.4f} mm from the recording"


@pytest.mark.gpu
def test_gpu_replays_the_recorded_tank_run(vsimlib, gpu):
    import pyoracle
    from vsim import Simulator

    scene, z = _scene()
    sim = Simulator(scene)
    assert sim.node_count == int(z["nodes"])
    assert sim.stats()["step_duration"] == float(z["dt"])
    orc = pyoracle.Oracle(scene, 32)
    orc.set_step_duration(float(z["dt"]))
    distances, seen = _replay(sim, z, lambda: sim.read_positions()[:, :3].copy())
    _, oracle_seen = _replay(orc, z, lambda: orc.state()[0][:, :3].copy())
    for g, o, step in zip(seen, oracle_seen, z["steps"]):
        assert np.array_equal(g, o), f"step {step}: GPU differs from the oracle"
    for d, bound, step in zip(distances, BOUND_M, z["steps"]):
        assert d <= bound, f"step {step}: {1e3 * d:.4f} mm from the recording"
    sim.destroy()
