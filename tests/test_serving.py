"""Isolated bodies, partial frames and the session server, on the GPU.

- Isolated scenes (every body its own contact grid) equal the oracle's
  isolated mode frame by frame.
- A body that sits a frame out is untouched; the bodies that ran equal the
  oracle run of each alone.
- Serving: a request's result is the same whether its session ran alone or
  among others (continuous batching does not change arithmetic), and a
  served session equals the oracle stepping that body alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(vsimlib, gpu):
    return vsimlib


def small_pool(count, seed=5):
    import vsim.scenes as sc

    return sc.session_pool(count, seed=seed, min_n=6, max_n=14)


def test_isolated_batch_matches_oracle(lib):
    import pyoracle
    import vsim.scenes as sc
    from vsim import Simulator

    bodies, tank = small_pool(5)
    scene = sc.Scene(bodies, tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True,
                     isolated=True)
    sim, orc = Simulator(scene), pyoracle.Oracle(scene, 32)
    for frame in range(6):
        sim.dispatch(10)
        orc.dispatch(10)
        g, o = sim.read_state(), orc.state()
        for a, b in zip(g, o):
            assert np.array_equal(a, b), f"frame {frame}"


def test_inactive_bodies_are_untouched(lib):
    import pyoracle
    import vsim.scenes as sc
    from vsim import Simulator

    bodies, tank = small_pool(4, seed=9)
    scene = sc.Scene(bodies, tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True,
                     isolated=True)
    sim = Simulator(scene)
    before = sim.read_state()
    active = [True, False, True, False]
    sim.set_bodies_active(active)
    for _ in range(3):
        sim.dispatch(10)
    after = sim.read_state()
    for b, on in enumerate(active):
        lo, hi = sim.offsets[b], sim.offsets[b] + bodies[b].node_count
        if not on:
            for x, y in zip(before, after):
                assert np.array_equal(x[lo:hi], y[lo:hi])
            continue
        alone = sc.Scene([bodies[b]], tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True,
                         isolated=True)
        orc = pyoracle.Oracle(alone, 32)
        for _ in range(3):
            orc.dispatch(10)
        for x, y in zip(after, orc.state()):
            assert np.array_equal(x[lo:hi], y)


def serve(bodies, tank, requests, budget=150e9):
    """Submit all `requests` (session, frames, drag) then tick until done;
    returns the server (for reads) and the completions."""
    from vsim.server import Server

    server = Server(bodies, tank, budget_bytes=budget)
    for session, frames, drag in requests:
        server.submit(session, frames, drag)
    done = []
    while server.stats()["pending"]:
        server.tick()
        done += server.poll()
    return server, done


def test_served_result_same_alone_and_in_the_mix(lib):
    import vsim.scenes as sc

    bodies, tank = small_pool(6, seed=11)
    rng = np.random.default_rng(3)
    drag0 = sc.drag_request(bodies[0], rng)
    alone, _ = serve(bodies, tank, [(0, 4, drag0)])
    mix_requests = [(0, 4, drag0)]
    for s in range(1, 6):
        mix_requests.append((s, int(rng.integers(1, 5)), sc.drag_request(bodies[s], rng) if s % 2 else None))
    mixed, done = serve(bodies, tank, mix_requests)
    assert len(done) == 6
    assert np.array_equal(alone.read_positions(0), mixed.read_positions(0))
    # Sessions without a request stayed at rest in the solo run.
    for s in range(1, 6):
        assert not np.array_equal(alone.read_positions(s), mixed.read_positions(s))


def test_requests_join_at_frame_boundaries(lib):
    """A request submitted while another runs starts at the next tick and
    shares frames with it; both finish with the frames they asked for."""
    bodies, tank = small_pool(3, seed=13)
    from vsim.server import Server

    server = Server(bodies, tank)
    first = server.submit(0, 4)
    server.tick()
    second = server.submit(1, 2)
    server.tick()
    server.tick()
    done = {c["request"]: c for c in server.poll()}
    assert second in done and first not in done
    assert done[second]["first_tick"] == 1 and done[second]["last_tick"] == 2
    server.tick()
    done = {c["request"]: c for c in server.poll()}
    assert done[first]["first_tick"] == 0 and done[first]["last_tick"] == 3
    assert server.stats()["session_frames"] == 6


def test_tick_budget_admits_started_then_oldest(lib):
    """Under a tick budget a tick runs the sessions whose requests already
    started (oldest first), then waiting requests in arrival order, while
    their cells fit; the first always runs. Results do not depend on the
    budget: each session ends where an unbudgeted server leaves it."""
    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = small_pool(6, seed=23)
    cells = [b.cell_count for b in bodies]
    rng = np.random.default_rng(5)
    requests = [(0, 3, sc.drag_request(bodies[0], rng)), (1, 1, None), (2, 2, None), (3, 1, None)]
    server = Server(bodies, tank)
    server.set_tick_budget(cells[0])  # session 0 alone fills a tick
    for session, frames, drag in requests:
        server.submit(session, frames, drag)
    stepped = []
    while server.stats()["pending"]:
        stepped.append(server.tick())
        server.poll()
    assert server.stats()["session_frames"] == 7
    assert len(stepped) > 3  # the free server needs three ticks
    free, _ = serve(bodies, tank, requests)
    for s in range(4):
        assert np.array_equal(server.read_positions(s), free.read_positions(s)), f"session {s}"


def test_tick_budget_order(lib):
    """Started requests keep their place; a later arrival waits while the
    budget is spent."""
    from vsim.server import Server

    bodies, tank = small_pool(4, seed=29)
    cells = [b.cell_count for b in bodies]
    server = Server(bodies, tank)
    server.set_tick_budget(max(cells[0], cells[1]))  # one of session 0 or 1 per tick
    a = server.submit(0, 2)
    b = server.submit(1, 1)
    assert server.tick() == 1  # session 0 (earliest)
    assert server.tick() == 1  # session 0 again: started requests go first
    done = {c["request"]: c for c in server.poll()}
    assert a in done and done[a]["first_tick"] == 0 and done[a]["last_tick"] == 1
    assert server.tick() == 1  # now session 1
    done = {c["request"]: c for c in server.poll()}
    assert b in done and done[b]["first_tick"] == 2
    server.set_tick_budget(0)
    server.submit(2, 1)
    server.submit(3, 1)
    assert server.tick() == 2  # no cap: both together


def test_native_request_loop(lib):
    """vsim_server_run: an open-loop schedule served by the library's loop
    ends every session exactly where submitting the same requests by hand
    and ticking does; completions carry the scheduled arrivals; a closed
    loop keeps every session busy for its span and reports its counts."""
    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = small_pool(5, seed=31)
    rng = np.random.default_rng(4)
    drags = [sc.drag_request(b, rng) for b in bodies]
    arrivals = np.array([0.0, 0.0005, 0.001, 0.02, 0.021])
    sessions = np.array([0, 1, 2, 0, 3])
    frames = np.array([2, 1, 3, 1, 2])
    flags = np.array([1, 0, 1, 0, 1])
    served = Server(bodies, tank)
    done, report = served.run(arrivals, sessions, frames, flags, drags)
    assert report["requests"] == 5 and report["returned"] == 5 and report["frames"] == 9
    assert sorted(c["frames"] for c in done) == sorted(frames.tolist())
    for c in done:
        assert c["completed"] >= c["submitted"]
    t0 = min(c["submitted"] for c in done)
    assert np.allclose(sorted(c["submitted"] - t0 for c in done), arrivals, atol=1e-9)
    by_hand, _ = serve(bodies, tank, [(int(q), int(k), drags[int(q)] if f else None)
                                      for q, k, f in zip(sessions, frames, flags)])
    # Same requests per session in the same order: the same end state.
    for q in range(4):
        assert np.array_equal(served.read_positions(q), by_hand.read_positions(q)), f"session {q}"
    closed = Server(bodies, tank)
    _, rep = closed.run(None, None, np.array([1, 2]), np.array([0, 1]), drags, closed_loop_seconds=0.05)
    assert rep["requests"] > 0 and rep["ticks"] > 0 and rep["seconds"] >= 0.05
    assert closed.stats()["pending"] == 0


@pytest.mark.parametrize("engine,block_cells,cluster_cells",
                         [(0, 0, 0), (1, 32, 512), (1, 1 << 30, 0), (1, 0, 1 << 30), (1, 60, 120)],
                         ids=["frames", "sessions-default", "sessions-all-block", "sessions-all-cluster",
                              "sessions-block-cluster-ticks"])
def test_engines_give_the_same_result(lib, engine, block_cells, cluster_cells):
    """vsim_server_run's engines -- ticks of shared frames; the session
    kernel with every session in one block, or on a cluster of blocks; and a
    mix of block, cluster and tick sessions running side by side -- leave
    every session exactly where submitting the same requests by hand and
    ticking leaves it, multi-frame drags and back-to-back requests of one
    session included; a closed loop then keeps them all busy and drains."""
    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = small_pool(7, seed=41)
    rng = np.random.default_rng(9)
    drags = [sc.drag_request(b, rng) for b in bodies]
    arrivals = np.array([0.0, 0.0, 0.0001, 0.0002, 0.0003, 0.0004, 0.0005, 0.002, 0.0021, 0.0022])
    sessions = np.array([0, 1, 2, 3, 4, 5, 6, 0, 2, 0])
    frames = np.array([3, 1, 2, 4, 1, 2, 3, 2, 1, 1])
    flags = np.array([1, 0, 1, 1, 0, 0, 1, 0, 1, 1])
    by_hand, _ = serve(bodies, tank, [(int(q), int(k), drags[int(q)] if f else None)
                                      for q, k, f in zip(sessions, frames, flags)])
    server = Server(bodies, tank)
    server.set_engine(engine, block_cells, cluster_cells)
    done, report = server.run(arrivals, sessions, frames, flags, drags)
    assert report["requests"] == 10 and report["frames"] == int(frames.sum())
    assert sorted(c["request"] for c in done) == sorted(set(c["request"] for c in done))
    for c in done:
        assert c["completed"] >= c["submitted"]
    for q in range(7):
        for a, b in zip(server.read_state(q), by_hand.read_state(q)):
            assert np.array_equal(a, b), f"session {q}"
    # The pool's hold list follows the run: ticking on afterwards matches.
    for q in (0, 3):
        server.submit(q, 2)
        by_hand.submit(q, 2)
    for srv in (server, by_hand):
        while srv.stats()["pending"]:
            srv.tick()
        srv.poll()
    for q in (0, 3):
        assert np.array_equal(server.read_positions(q), by_hand.read_positions(q)), f"ticked session {q}"
    _, rep = server.run(None, None, np.array([1, 3, 2]), np.array([1, 0, 1]), drags, closed_loop_seconds=0.03)
    assert rep["requests"] > 0 and rep["seconds"] >= 0.03 and server.stats()["pending"] == 0
    for srv in (server, by_hand):
        srv.destroy()


def test_server_on_a_caller_stream(lib):
    """A server given the caller's stream (vsim_server_create's `stream`)
    runs its ticks there -- the session engine's launch slots on their own
    streams as always -- and leaves every session where a server on a stream
    of its own (made at the device's greatest priority) leaves it; the
    caller's stream outlives the server."""
    import torch
    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = small_pool(7, seed=41)
    rng = np.random.default_rng(9)
    drags = [sc.drag_request(b, rng) for b in bodies]
    arrivals = np.array([0.0, 0.0, 0.0001, 0.0002, 0.0003, 0.0004, 0.0005, 0.002])
    sessions = np.array([0, 1, 2, 3, 4, 5, 6, 0])
    frames = np.array([3, 1, 2, 4, 1, 2, 3, 2])
    flags = np.array([1, 0, 1, 1, 0, 0, 1, 0])
    caller = torch.cuda.Stream()
    states = []
    for stream in (None, caller.cuda_stream):
        server = Server(bodies, tank, stream=stream)
        server.set_engine(1, 60, 120)  # blocks, clusters and ticks side by side
        _, report = server.run(arrivals, sessions, frames, flags, drags)
        assert report["requests"] == len(frames)
        states.append([server.read_state(q) for q in range(7)])
        server.destroy()
    for q in range(7):
        for a, b in zip(states[0][q], states[1][q]):
            assert np.array_equal(a, b), f"session {q}"
    with torch.cuda.stream(caller):
        x = torch.ones(4, device="cuda") * 2
    caller.synchronize()
    assert float(x.sum()) == 8.0


def test_session_kernel_stretch_limit_and_engine_checks(lib):
    """Sessions whose material limits stretch (maxStretch > 1: three limit-only
    sweeps of the eight colours every substep) leave the session kernel --
    in one block and on a cluster -- where the ticks leave them; unknown
    engines are refused."""
    import dataclasses

    import vsim.scenes as sc
    from vsim import _ffi
    from vsim.server import Server

    bodies, tank = small_pool(5, seed=43)
    bodies = [dataclasses.replace(b, material=dict(b.material, max_stretch=1.05)) for b in bodies]
    rng = np.random.default_rng(12)
    drags = [sc.drag_request(b, rng) for b in bodies]
    requests = [(q, 3, drags[q] if q % 2 else None) for q in range(5)]
    by_hand, _ = serve(bodies, tank, requests)
    for block, cluster in ((1 << 30, 0), (0, 1 << 30)):
        server = Server(bodies, tank)
        server.set_engine(server.SESSIONS, block, cluster)
        server.run(np.zeros(5), np.arange(5), np.full(5, 3), np.array([q % 2 for q in range(5)]), drags)
        for q in range(5):
            for a, b in zip(server.read_state(q), by_hand.read_state(q)):
                assert np.array_equal(a, b), f"block {block} cluster {cluster} session {q}"
        with pytest.raises(_ffi.VsimError):
            server.set_engine(7)
        server.destroy()
    by_hand.destroy()


def test_default_engine_on_the_serving_pool(lib):
    """The serving workload's 64-session pool (noise blobs on 8^3-64^3 grids:
    block, cluster and tick sessions under the default thresholds), settled
    for 20 frames into self contact, then 200 seeded requests (k ~ U{1..4},
    half dragging) arriving as a Poisson schedule: the session engine and
    the frames engine leave every session's state equal bit for bit, and
    the session engine's jobs pass their own checks."""
    import vsim.scenes as sc
    from vsim.server import Server

    bodies, tank = sc.session_pool(64, seed=3)
    rng = np.random.default_rng(21)
    drags = [sc.drag_request(b, rng) for b in bodies]
    arrivals = np.cumsum(rng.exponential(1 / 4000, 200))
    sessions = rng.integers(0, 64, 200)
    frames = rng.integers(1, 5, 200)
    flags = (rng.random(200) < 0.5).astype(np.int64)
    states = []
    for engine in (Server.SESSIONS, Server.FRAMES):
        server = Server(bodies, tank)
        for q in range(64):
            server.submit(q, 20)
        while server.stats()["pending"]:
            server.tick()
        server.poll()
        server.set_engine(engine)
        done, report = server.run(arrivals, sessions, frames, flags, drags)
        assert report["requests"] == 200 and report["frames"] == int(frames.sum())
        states.append([server.read_state(q) for q in range(64)])
        server.destroy()
    for q in range(64):
        for a, b, what in zip(states[0][q], states[1][q], ("pos", "prev", "vel")):
            assert np.array_equal(a, b), f"session {q} {what}"


def test_served_session_matches_oracle(lib):
    import pyoracle
    import vsim.scenes as sc

    bodies, tank = small_pool(3, seed=17)
    server, _ = serve(bodies, tank, [(1, 5, None), (2, 2, None)])
    alone = sc.Scene([bodies[1]], tank, step_duration=1 / 600, substeps=10, contact=True, self_contact=True,
                     isolated=True)
    orc = pyoracle.Oracle(alone, 32)
    for _ in range(5):
        orc.dispatch(10)
    assert np.array_equal(server.read_positions(1), orc.state()[0])


def test_budget_admission(lib):
    from vsim.server import Server

    bodies, tank = small_pool(8, seed=19)
    everyone = Server(bodies, tank)
    assert everyone.admitted == 8
    per = everyone.stats()["resident_bytes"] / 8
    tight = Server(bodies, tank, budget_bytes=per * 3)
    st = tight.stats()
    assert 1 <= tight.admitted < 8 and st["rejected"] == 8 - tight.admitted
    assert st["resident_bytes"] <= per * 3


def test_session_checkpoint_restore_and_reset(lib):
    """A session read out, run on, written back and run again with the same
    requests ends exactly where the first run did; a pending session refuses
    to be overwritten; reset returns it to rest."""
    import vsim.scenes as sc
    from vsim import _ffi
    from vsim.server import Server

    bodies, tank = small_pool(3, seed=17)
    rng = np.random.default_rng(4)
    drag = sc.drag_request(bodies[1], rng)
    server = Server(bodies, tank)
    rest = server.read_state(1)

    def run(requests):
        for session, frames, d in requests:
            server.submit(session, frames, d)
        while server.stats()["pending"]:
            server.tick()
        server.poll()

    run([(1, 3, drag), (2, 2, None)])
    checkpoint = server.read_state(1)
    run([(1, 4, drag), (0, 1, None)])
    first = server.read_state(1)
    assert not np.array_equal(first[0], checkpoint[0])

    server.write_state(1, *checkpoint)
    assert all(np.array_equal(a, b) for a, b in zip(server.read_state(1), checkpoint))
    run([(1, 4, drag), (2, 3, None)])  # other sessions' work differs; session 1's must not
    second = server.read_state(1)
    for a, b in zip(first, second):
        assert np.array_equal(a, b)

    server.submit(1, 1)
    with pytest.raises(_ffi.VsimError):
        server.write_state(1, *checkpoint)
    while server.stats()["pending"]:
        server.tick()
    server.reset_session(1)
    for a, b in zip(server.read_state(1), rest):
        assert np.array_equal(a, b)
    server.destroy()


def test_eviction_and_readmission(lib):
    """Sessions evicted to the host and made resident again -- in another
    pool order, beside other sessions -- continue exactly as in a server
    that never moved them; a session with requests pending cannot leave; a
    set over the budget is refused and changes nothing; a session that is
    not resident takes no requests; a session never run arrives at rest."""
    import vsim.scenes as sc
    from vsim import _ffi
    from vsim.server import Server

    bodies, tank = small_pool(6, seed=23)
    rng = np.random.default_rng(8)
    drags = {s: sc.drag_request(bodies[s], rng) for s in (1, 4)}
    plan1 = [(0, 3, None), (1, 2, drags[1]), (2, 4, None), (3, 1, None), (4, 2, drags[4]), (5, 3, None)]
    plan2 = [(0, 2, None), (1, 3, drags[1]), (3, 2, None), (4, 1, drags[4])]

    def run(server, requests):
        for session, frames, d in requests:
            server.submit(session, frames, d)
        while server.stats()["pending"]:
            server.tick()
        server.poll()

    kept = Server(bodies, tank)
    run(kept, plan1)
    run(kept, plan2)

    moved = Server(bodies, tank)
    run(moved, plan1)
    moved.set_resident([5, 2])
    assert moved.resident == [5, 2] and moved.admitted == 2 and moved.stats()["sessions"] == 2
    with pytest.raises(_ffi.VsimError):
        moved.submit(0, 1)
    moved.set_resident([4, 3, 1, 0, 2])
    run(moved, plan2)
    for s in range(5):
        for a, b in zip(kept.read_state(s), moved.read_state(s)):
            assert np.array_equal(a, b), f"session {s}"

    moved.submit(0, 1)
    with pytest.raises(_ffi.VsimError):
        moved.set_resident([1, 2])
    run(moved, [])
    assert moved.resident == [4, 3, 1, 0, 2]

    per = kept.stats()["resident_bytes"] / 6
    tight = Server(bodies, tank, budget_bytes=per * 2.5)
    before = tight.resident
    with pytest.raises(_ffi.VsimError):
        tight.set_resident([0, 1, 2, 3, 4, 5])
    assert tight.resident == before == list(range(tight.admitted))

    fresh = Server(bodies, tank)
    rest = fresh.read_state(5)
    fresh.set_resident([])
    assert fresh.admitted == 0 and fresh.resident == []
    fresh.set_resident([5])
    for a, b in zip(fresh.read_state(5), rest):
        assert np.array_equal(a, b)
    for server in (kept, moved, tight, fresh):
        server.destroy()
