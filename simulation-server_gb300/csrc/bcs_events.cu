// bcs_events.cu — the streaming server's control messages without the
// network and the renderer (host code only).
//
// The reference's server takes one-byte messages from its client over ENet
// (src/communication/server_endpoint.cpp:6-8,168-185): the low seven bits
// name the event, the high bit is set for "start" (a key pressed) and clear
// for "stop" (released).  Its MsgController (msg_controller.cpp:27-148)
// handles at most one message per frame: a start adds the event to the set
// of held events, a stop removes it and then, like the connection events,
// goes through the single-message handling (render toggles, abort on
// stopRendering, held set cleared on disconnect).  bcs_control keeps that
// state machine and queue; a transport of the application's choosing posts
// the received bytes and takes the outgoing ones, and a renderer reads the
// held events and toggles.  bcs_run (bcs_api.cu) is the server loop around
// it.
#include <cstdint>
#include <deque>
#include <mutex>
#include <new>

#include "../../include/bcs.h"

struct bcs_control {
    std::mutex lock;
    std::deque<bcs_event> in;     // decoded, not yet handled
    std::deque<uint8_t> out;      // encoded, not yet taken by the transport
    bcs_control_state state{};
};

namespace {
constexpr uint8_t kStartBit = 0x80;                  // START_EVENT_MASK of the reference
constexpr uint8_t kPayload = (uint8_t)~kStartBit;    // EVENT_PAYLOAD

bool valid(const bcs_event& e) {
    return e.type >= BCS_EVENT_NO_MESSAGE && e.type <= BCS_EVENT_INVALID_MESSAGE &&
           e.state >= BCS_EVENT_START && e.state <= BCS_EVENT_NOT_RELEVANT;
}

// handleSingleMsgs (msg_controller.cpp:114-148), headless
void handle_single(bcs_control_state& s, const bcs_event& e) {
    switch (e.type) {
        case BCS_EVENT_NEW_CONNECTION: s.connected = 1; break;
        case BCS_EVENT_PEER_DISCONNECTED:
            s.held = 0u;
            s.connected = 0;
            break;
        case BCS_EVENT_TOGGLE_POLYGON_MODE: s.polygon_mode_line ^= 1; break;
        case BCS_EVENT_TOGGLE_SPRINGS_RENDERING: s.springs_rendering ^= 1; break;
        case BCS_EVENT_TOGGLE_SPHERES_RENDERING: s.spheres_rendering ^= 1; break;
        case BCS_EVENT_STOP_RENDERING: s.stop_requested = 1; break;
        default: break;   // other messages are ignored
    }
}
}  // namespace

extern "C" {

bcs_event bcs_event_decode(const uint8_t* data, size_t length) {
    bcs_event e{BCS_EVENT_INVALID_MESSAGE, BCS_EVENT_NOT_RELEVANT};
    if (!data || length != 1) return e;
    const uint8_t payload = data[0] & kPayload;
    if (payload >= (uint8_t)BCS_EVENT_INVALID_MESSAGE) return e;
    e.type = payload;
    e.state = (data[0] & kStartBit) ? BCS_EVENT_START : BCS_EVENT_STOP;
    return e;
}

int bcs_event_encode(bcs_event event, uint8_t* byte) {
    if (!byte || !valid(event)) return 0;
    uint8_t b = (uint8_t)event.type;
    if (event.state == BCS_EVENT_START) b |= kStartBit;
    *byte = b;
    return event.type == BCS_EVENT_STREAM_SUCCESSFULLY_ENDED || event.type == BCS_EVENT_STOP_RENDERING ? 2 : 1;
}

bcs_status bcs_control_create(bcs_control** out) {
    if (!out) return BCS_ERR_INVALID_ARGUMENT;
    bcs_control* c = new (std::nothrow) bcs_control();
    if (!c) return BCS_ERR_OUT_OF_MEMORY;
    c->state.springs_rendering = 1;
    c->state.spheres_rendering = 1;
    *out = c;
    return BCS_OK;
}

void bcs_control_destroy(bcs_control* c) { delete c; }

bcs_status bcs_control_post(bcs_control* c, const uint8_t* data, size_t length) {
    if (!c) return BCS_ERR_INVALID_ARGUMENT;
    const bcs_event e = bcs_event_decode(data, length);
    std::lock_guard<std::mutex> g(c->lock);
    c->in.push_back(e);
    return BCS_OK;
}

bcs_status bcs_control_post_event(bcs_control* c, bcs_event event) {
    if (!c || !valid(event)) return BCS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(c->lock);
    c->in.push_back(event);
    return BCS_OK;
}

bcs_status bcs_control_handle(bcs_control* c, bcs_control_state* state_out) {
    if (!c) return BCS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(c->lock);
    if (!c->in.empty()) {
        const bcs_event e = c->in.front();
        c->in.pop_front();
        bcs_control_state& s = c->state;
        if (e.type != BCS_EVENT_NO_MESSAGE && e.type != BCS_EVENT_INVALID_MESSAGE) {
            switch (e.state) {
                case BCS_EVENT_START: s.held |= 1u << e.type; break;
                case BCS_EVENT_STOP:
                    s.held &= ~(1u << e.type);
                    handle_single(s, e);   // as in the reference, a stop also takes the single-message path
                    break;
                default: handle_single(s, e); break;
            }
        }
        ++s.handled;
    }
    if (state_out) *state_out = c->state;
    return BCS_OK;
}

bcs_status bcs_control_send(bcs_control* c, bcs_event event) {
    uint8_t b = 0;
    if (!c || !bcs_event_encode(event, &b)) return BCS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(c->lock);
    c->out.push_back(b);
    return BCS_OK;
}

int bcs_control_take_outgoing(bcs_control* c, uint8_t* byte) {
    if (!c || !byte) return 0;
    std::lock_guard<std::mutex> g(c->lock);
    if (c->out.empty()) return 0;
    *byte = c->out.front();
    c->out.pop_front();
    return 1;
}

}  // extern "C"
