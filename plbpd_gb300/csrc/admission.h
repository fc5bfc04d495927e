// The solve server's admission policy, free of CUDA so that it is testable
// on its own (tests/cpp/test_admission.cpp).
//
// Under overload the device-memory budget fills with admitted requests that
// then share the device, and each finishes late.  Requests are therefore
// admitted while (1) their device bytes fit the budget and (2) the running
// requests hold fewer than `cap_cells` cells (a request larger than the cap
// runs once nothing else runs), taking the queued request with the fewest
// cell updates first -- unless the oldest has waited `max_wait` seconds, or
// the order is FIFO, when the oldest goes first.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace plb {

struct AdmissionView {      // one queued request, in arrival order
    double t_submit;        // seconds
    double work;            // cells x steps
    int64_t cells;
    int64_t bytes;          // device bytes it needs
};

struct AdmissionState {
    int64_t budget = 0, used = 0;        // device bytes
    int64_t cap_cells = 0, active_cells = 0;
    double max_wait = 30.0;
    bool fifo = false;
};

enum class Admit { kTake, kWait, kReject };

// The index (into `queue`, arrival order) of the request to consider next.
inline size_t admission_pick(const std::vector<AdmissionView>& queue, const AdmissionState& st, double now) {
    if (queue.empty() || st.fifo || now - queue.front().t_submit >= st.max_wait) return 0;
    size_t pick = 0;
    for (size_t i = 1; i < queue.size(); ++i)
        if (queue[i].work < queue[pick].work) pick = i;
    return pick;
}

// What to do with the picked request: take it, wait for room, or reject it
// (it needs more than the whole budget).
inline Admit admission_decide(const AdmissionView& r, const AdmissionState& st) {
    if (r.bytes > st.budget) return Admit::kReject;
    if (st.used + r.bytes > st.budget) return Admit::kWait;
    if (st.active_cells > 0 && st.active_cells + r.cells > st.cap_cells) return Admit::kWait;
    return Admit::kTake;
}

}  // namespace plb
