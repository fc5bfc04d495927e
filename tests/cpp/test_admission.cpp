// Unit test of the solve server's admission policy (plbpd_gb300/csrc/admission.h);
// no GPU.  Prints "ok" and exits 0, or names the failed check and exits 1.
#include <cstdio>
#include <vector>

#include "admission.h"

using plb::Admit;
using plb::AdmissionState;
using plb::AdmissionView;

static int failures = 0;
#define CHECK(c)                                                    \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                             \
        }                                                           \
    } while (0)

int main() {
    AdmissionState st;
    st.budget = 1000;
    st.cap_cells = 100;
    st.max_wait = 30.0;
    // arrival order: big, small, medium
    const std::vector<AdmissionView> q = {{0.0, 5e9, 80, 400}, {1.0, 1e6, 10, 50}, {2.0, 1e8, 40, 200}};

    // smallest work first
    CHECK(plb::admission_pick(q, st, 5.0) == 1);
    // the oldest goes first once it has waited max_wait
    CHECK(plb::admission_pick(q, st, 30.0) == 0);
    CHECK(plb::admission_pick(q, st, 29.999) == 1);
    // FIFO order
    AdmissionState fifo = st;
    fifo.fifo = true;
    CHECK(plb::admission_pick(q, fifo, 5.0) == 0);
    CHECK(plb::admission_pick({}, st, 0.0) == 0);
    // ties keep arrival order
    const std::vector<AdmissionView> tie = {{0.0, 7.0, 1, 1}, {1.0, 7.0, 1, 1}};
    CHECK(plb::admission_pick(tie, st, 2.0) == 0);

    // budget: fits, waits for room, rejected outright
    CHECK(plb::admission_decide(q[1], st) == Admit::kTake);
    AdmissionState full = st;
    full.used = 980;
    CHECK(plb::admission_decide(q[1], full) == Admit::kWait);
    const AdmissionView huge = {0.0, 1.0, 1, 1001};
    CHECK(plb::admission_decide(huge, st) == Admit::kReject);

    // running-cells cap: waits while others run and it would exceed the cap
    AdmissionState busy = st;
    busy.active_cells = 70;
    CHECK(plb::admission_decide(q[1], busy) == Admit::kTake);     // 70 + 10 <= 100
    CHECK(plb::admission_decide(q[2], busy) == Admit::kWait);     // 70 + 40 > 100
    // a request larger than the cap runs when nothing else runs
    const AdmissionView wide = {0.0, 1.0, 500, 10};
    CHECK(plb::admission_decide(wide, st) == Admit::kTake);
    busy.active_cells = 1;
    CHECK(plb::admission_decide(wide, busy) == Admit::kWait);

    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
