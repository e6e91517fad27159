"""GPU parity at the workloads' full sizes: the bench's single large body
with its 1M splats, the 256-body batch, and the stress scene (one substep
from rest, and one whole frame once the sheet has landed on the blob), each
compared with the float oracle node for node (`==`).

These run the same kernels as tests/test_gpu_parity.py but at the launch
shapes the bench uses (block sizes, gather mapping, streamed colour passes),
so a shape-dependent fault cannot hide behind small test scenes.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same, make

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(vsimlib, gpu):
    return vsimlib


def test_headline_body_frames_and_splats(lib):
    """64^3 noise blob (126,535 cells), ground and self contact, 1M splats:
    five frames, then the contact pairs, the deformed splats and their depth
    order."""
    import pyoracle
    import vsim.scenes as sc

    scene = sc.noise_blob(n=64, seed=1, splats=1_000_000)
    sim, orc = make(scene)
    for frame in range(5):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")
    assert np.array_equal(sim.contact_pairs(), orc.contact_pairs())
    view = (0.0, 0.0, -1.0)
    sim.deform_splats(view)
    sim.sort_splats()
    means, cov, order = sim.read_splats()
    m, q, s, *_ = scene.splats[0]
    om, oc, keys = orc.splat_deform(0, m, q, s, view)
    assert np.array_equal(means, om)
    assert np.array_equal(cov, oc)
    assert np.array_equal(order, pyoracle.stable_sort(keys))


def test_batch_of_256_uneven_boxes(lib):
    """The batching workload: 256 boxes with sides log-uniform 4-48 cells
    (1.5M cells), one pinned face each, ground contact; two frames."""
    import vsim.scenes as sc

    scene = sc.box_batch(256, seed=2)
    sim, orc = make(scene)
    for frame in range(2):
        sim.dispatch(scene.substeps)
        orc.dispatch(scene.substeps)
        assert_same(sim, orc, scene, f"frame {frame}")


def test_stress_scene_one_substep(lib):
    """The stress workload (192^3 blob + 192 x 192 x 2 sheet, 4.1M cells,
    two Gauss-Seidel sweeps, self and body contact): one substep, which runs
    the streamed colour pass and the thread-per-record gather."""
    import vsim.scenes as sc

    scene = sc.blob_and_sheet(192, seed=4, splats=0)
    sim, orc = make(scene)
    assert min(sim.color_counts()) >= 155_648
    sim.dispatch(1)
    orc.dispatch(1)
    assert_same(sim, orc, scene, "substep 1")


def test_stress_scene_full_frame_in_contact(lib):
    """The stress workload once the sheet lies on the blob (30 frames run on
    the GPU first): the oracle takes that state, and both run one whole frame
    -- 20 substeps of 2 Gauss-Seidel sweeps (lambda restarting each sweep,
    xpbdCouple.wgsl:9-13) with dense self and body contact. Positions,
    previous positions and velocities node for node, then the contact pairs
    of the state reached."""
    import vsim.scenes as sc

    scene = sc.blob_and_sheet(192, seed=4, splats=0)
    sim, orc = make(scene)
    for _ in range(30):
        sim.dispatch(scene.substeps)
    pos, prev, vel = sim.read_state()
    orc.set_state(pos, prev, vel)
    sim.dispatch(scene.substeps)
    orc.dispatch(scene.substeps)
    assert_same(sim, orc, scene, "frame 31 (20 substeps x 2 sweeps)")
    pairs = sim.contact_pairs()
    assert len(pairs) > 10_000, "the sheet and blob are not in contact yet"
    assert np.array_equal(pairs, orc.contact_pairs())
