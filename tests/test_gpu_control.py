"""The server loop (bcs_run) around the control messages: frames until a
handled stopRendering message, or max_frames + 1 frames as main.cu:158-245
counts them, then streamSuccessfullyEnded queued for the client."""
import numpy as np
import pytest

import bcs
import bcs_scenes as S

pytestmark = pytest.mark.gpu

E = bcs.EVENT


def make():
    sc = S.tiny_scene(cells=6, seed=3)
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    return sc, sim


def test_run_counts_frames_like_the_reference(lib):
    sc, sim = make()
    assert sim.run(4) == 5
    other = bcs.Simulation(sc)
    other.set_particles(sc.positions, sc.velocities)
    other.step(5)
    for a, b in zip(sim.get_particles(), other.get_particles()):
        np.testing.assert_array_equal(a, b)


def test_run_stops_on_stop_rendering(lib):
    _, sim = make()
    c = bcs.Control()
    c.post(bytes([E["camera_left"] | 0x80]))
    c.post(bytes([E["stop_rendering"] | 0x80]))
    c.post(bytes([E["stop_rendering"]]))   # the stop message acts (msg_controller.cpp:40-45)
    assert sim.run(100, c) == 3
    assert sim.refresh_info().steps_done == 3
    assert c.take_outgoing() == [E["stream_successfully_ended"]]
    s = c.handle()
    assert s["stop_requested"] == 1 and s["held"] == 1 << E["camera_left"]
