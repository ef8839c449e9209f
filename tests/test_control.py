"""The streaming server's control messages (bcs_control), headless.

The reference's client sends one byte per message (server_endpoint.cpp:6-8,
140-185): the low seven bits name the event, the high bit marks "start".
Its MsgController (msg_controller.cpp:27-148) handles one message per call:
a start adds the event to the held set, a stop removes it and then, through
the missing break of its switch, also takes the single-message path (render
toggles, abort on stopRendering, held set cleared on disconnect).  These
tests need no GPU; the server loop around it is in test_gpu_control.py.
"""
import pytest

import bcs

E = bcs.EVENT


def test_decode_follows_parse_event(lib):
    assert bcs.decode_event(bytes([E["camera_left"] | 0x80])) == ("camera_left", bcs.EVENT_START)
    assert bcs.decode_event(bytes([E["camera_left"]])) == ("camera_left", bcs.EVENT_STOP)
    assert bcs.decode_event(bytes([E["stop_rendering"]])) == ("stop_rendering", bcs.EVENT_STOP)
    # unknown event numbers, the invalid marker itself and wrong lengths are invalid
    for bad in (bytes([E["invalid_message"]]), bytes([0x7F]), bytes([0xFF]), b"", bytes([1, 2])):
        assert bcs.decode_event(bad) == ("invalid_message", bcs.EVENT_NOT_RELEVANT)


def test_encode_round_trip_and_channels(lib):
    for name in bcs.EVENT_NAMES[:-1]:
        for state in (bcs.EVENT_START, bcs.EVENT_STOP):
            b, ch = bcs.encode_event(name, state)
            assert bcs.decode_event(bytes([b])) == (name, state)
            assert ch == (2 if name in ("stream_successfully_ended", "stop_rendering") else 1)
    # a not-relevant state encodes like a stop (no start bit)
    assert bcs.encode_event("stream_successfully_ended", bcs.EVENT_NOT_RELEVANT) == (E["stream_successfully_ended"], 2)
    assert bcs.encode_event("no_message", 7) == (None, 0)


def test_held_events_one_message_per_call(lib):
    c = bcs.Control()
    c.post(bytes([E["camera_left"] | 0x80]))
    c.post(bytes([E["camera_rotate_up"] | 0x80]))
    c.post(bytes([E["camera_left"]]))
    s = c.handle()
    assert s["held"] == 1 << E["camera_left"] and s["handled"] == 1
    s = c.handle()
    assert s["held"] == (1 << E["camera_left"]) | (1 << E["camera_rotate_up"])
    s = c.handle()
    assert s["held"] == 1 << E["camera_rotate_up"]
    s = c.handle()   # empty queue: nothing changes
    assert s["handled"] == 3


def test_toggles_act_on_the_stop_message(lib):
    c = bcs.Control()
    s = c.handle()
    assert (s["polygon_mode_line"], s["springs_rendering"], s["spheres_rendering"]) == (0, 1, 1)
    for name in ("toggle_polygon_mode", "toggle_springs_rendering", "toggle_spheres_rendering"):
        c.post(bytes([E[name] | 0x80]))   # key down: held, no toggle
        c.post(bytes([E[name]]))          # key up: released, toggled
    states = [c.handle() for _ in range(6)]
    assert states[0]["polygon_mode_line"] == 0 and states[1]["polygon_mode_line"] == 1
    assert states[3]["springs_rendering"] == 0 and states[5]["spheres_rendering"] == 0
    assert states[5]["held"] == 0


def test_stop_rendering_and_connections(lib):
    c = bcs.Control()
    c.post_event("new_connection")
    c.post(bytes([E["camera_back"] | 0x80]))
    c.post_event("peer_disconnected")
    c.post(bytes([E["stop_rendering"] | 0x80]))
    c.post(bytes([E["stop_rendering"]]))
    s = [c.handle() for _ in range(5)]
    assert s[0]["connected"] == 1 and s[1]["held"] == 1 << E["camera_back"]
    assert s[2]["connected"] == 0 and s[2]["held"] == 0
    assert s[3]["stop_requested"] == 0 and s[4]["stop_requested"] == 1
    with pytest.raises(bcs.BcsError):
        c.post_event("camera_left", 9)


def test_outgoing_queue(lib):
    c = bcs.Control()
    c.send("stream_successfully_ended")
    c.send("camera_left", bcs.EVENT_START)
    assert c.take_outgoing() == [E["stream_successfully_ended"], E["camera_left"] | 0x80]
    assert c.take_outgoing() == []
