"""The solve server: requests of mixed lattice, size, tau, storage, mask and
step count run together (continuous batching) and each result equals the
same request run alone; admission respects the memory budget."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def request_params(capi, rng, model, storage):
    from plbpd_gb300.workloads import porous_mask
    if model == "D2Q9":
        L = int(rng.integers(16, 80))
        nx, ny, nz = L + L % 2, 1, L
        faces = {"east": "periodic", "west": "periodic", "up": "noslip", "down": "noslip"}
        vel = {"up": (0.0, 0.0, 0.0), "down": (0.0, 0.0, 0.0)}
    else:
        L = int(rng.integers(8, 28))
        nx, ny, nz = L + L % 2, L, L
        faces = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
                 "down": "noslip"}
        vel = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}
    tau = float(rng.uniform(0.55, 1.5))
    p = capi.make_params(model, nx, ny, nz, (tau - 0.5) / 3.0, force=(float(rng.uniform(1e-6, 1e-5)), 0.0, 0.0),
                         face_type=faces, face_vel=vel, semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32,
                         storage=storage)
    mask = porous_mask(nx, ny, nz, float(rng.uniform(0.8, 1.0)), int(rng.integers(1 << 30)))
    steps = int(rng.integers(20, 300))
    return p, mask, steps


def run_alone(capi, p, mask, steps):
    with capi.Solve(p) as s:
        s.set_mask(mask)
        s.initialize()
        s.step(steps)
        return s.get(capi.FIELD_RHO), s.get(capi.FIELD_U)


def test_mixed_stream_equals_each_request_alone():
    from plbpd_gb300 import capi
    rng = np.random.default_rng(42)
    reqs = []
    for i in range(16):
        model = "D2Q9" if i % 5 < 3 else "D3Q19"
        storage = capi.STORAGE_FP16_DEV if i % 2 else capi.STORAGE_FP32
        reqs.append(request_params(capi, rng, model, storage))
    with capi.Server(budget_bytes=8 << 30, tick_steps=37) as srv:
        ids = []
        for p, m, n in reqs:             # arrivals while earlier requests run
            ids.append(srv.submit(p, n, m))
        results = []
        for rid in ids:
            srv.wait(rid, 300.0)
            results.append(srv.result(rid))
    for (p, m, n), (rho, u, t) in zip(reqs, results):
        rho_a, u_a = run_alone(capi, p, m, n)
        assert np.array_equal(rho.view(np.uint32), rho_a.view(np.uint32))
        assert np.array_equal(u.view(np.uint32), u_a.view(np.uint32))
        assert t[0] <= t[1] <= t[2]


def test_admission_respects_budget():
    from plbpd_gb300 import capi
    rng = np.random.default_rng(7)
    reqs = [request_params(capi, rng, "D3Q19", capi.STORAGE_FP32) for _ in range(6)]
    biggest = max(capi.lib().plb_solve_bytes(capi.C.byref(p)) for p, _, _ in reqs)
    budget = int(biggest * 1.5)          # at most one or two at a time
    with capi.Server(budget_bytes=budget, tick_steps=50) as srv:
        ids = [srv.submit(p, n, m) for p, m, n in reqs]
        for rid in ids:
            srv.wait(rid, 300.0)
        in_use, peak = srv.memory()
        times = [srv.result(rid)[2] for rid in ids]
    assert peak <= budget and in_use == 0
    assert all(t[2] >= t[1] for t in times)


def test_request_larger_than_budget_fails_cleanly():
    from plbpd_gb300 import capi
    rng = np.random.default_rng(3)
    p, m, n = request_params(capi, rng, "D3Q19", capi.STORAGE_FP32)
    with capi.Server(budget_bytes=1 << 20, tick_steps=50) as srv:
        rid = srv.submit(p, n, m)
        with pytest.raises(capi.PlbError):
            srv.wait(rid, 60.0)


def test_concurrent_submitters():
    from plbpd_gb300 import capi
    rng = np.random.default_rng(11)
    reqs = [request_params(capi, rng, "D2Q9", capi.STORAGE_FP32) for _ in range(8)]
    out = {}
    with capi.Server(budget_bytes=4 << 30, tick_steps=64) as srv:
        def client(k):
            p, m, n = reqs[k]
            rid = srv.submit(p, n, m)
            srv.wait(rid, 300.0)
            out[k] = srv.result(rid)[1]
        th = [threading.Thread(target=client, args=(k,)) for k in range(len(reqs))]
        for t in th:
            t.start()
        for t in th:
            t.join()
    for k, (p, m, n) in enumerate(reqs):
        _, u_a = run_alone(capi, p, m, n)
        assert np.array_equal(out[k].view(np.uint32), u_a.view(np.uint32))


def test_malformed_request_refused_at_submit():
    """A NaN viscosity is refused on the submitting thread; the requests
    around it are unaffected."""
    from plbpd_gb300 import capi
    rng = np.random.default_rng(5)
    good = [request_params(capi, rng, "D2Q9", capi.STORAGE_FP32) for _ in range(2)]
    bad, bm, bn = request_params(capi, rng, "D2Q9", capi.STORAGE_FP32)
    bad.nu = float("nan")
    with capi.Server(budget_bytes=2 << 30, tick_steps=40) as srv:
        r0 = srv.submit(good[0][0], good[0][2], good[0][1])
        with pytest.raises(capi.PlbError) as e:
            srv.submit(bad, bn, bm)
        assert e.value.code == capi.EINVAL
        r1 = srv.submit(good[1][0], good[1][2], good[1][1])
        out = []
        for rid in (r0, r1):
            srv.wait(rid, 300.0)
            out.append(srv.result(rid)[1])
    for (p, m, n), u in zip(good, out):
        assert np.array_equal(u.view(np.uint32), run_alone(capi, p, m, n)[1].view(np.uint32))


def test_cancel_queued_and_running_requests():
    """Cancelling a queued request drops it before admission; cancelling a
    running one ends it at the next tick and returns its memory; a request
    run beside them still equals its solo run."""
    from plbpd_gb300 import capi
    rng = np.random.default_rng(9)
    big_p, big_m, _ = request_params(capi, rng, "D3Q19", capi.STORAGE_FP32)
    small = request_params(capi, rng, "D2Q9", capi.STORAGE_FP32)
    budget = int(capi.lib().plb_solve_bytes(capi.C.byref(big_p)) * 1.2)
    with capi.Server(budget_bytes=budget, tick_steps=20) as srv:
        running = srv.submit(big_p, 2_000_000, big_m)      # holds the budget
        for _ in range(2000):
            if srv.status(running) == capi.REQ_RUNNING:
                break
            time.sleep(0.005)
        assert srv.status(running) == capi.REQ_RUNNING
        queued = srv.submit(big_p, 50, big_m)              # waits for it
        assert srv.status(queued) == capi.REQ_QUEUED
        srv.cancel(queued)
        assert srv.status(queued) == capi.REQ_CANCELLED
        srv.cancel(running)
        with pytest.raises(capi.PlbError) as e:
            srv.wait(running, 120.0)
        assert e.value.code == capi.ESTATE
        assert srv.status(running) == capi.REQ_CANCELLED
        with pytest.raises(capi.PlbError):
            srv.result(running)
        with pytest.raises(capi.PlbError):
            srv.result(queued)
        in_use, _ = srv.memory()
        assert in_use == 0
        p, m, n = small
        rid = srv.submit(p, n, m)
        srv.wait(rid, 300.0)
        u = srv.result(rid)[1]
    assert np.array_equal(u.view(np.uint32), run_alone(capi, p, m, n)[1].view(np.uint32))


def test_failing_client_does_not_disturb_others():
    """A client thread that raises after submitting (and never collects) leaves
    the other clients' results exact."""
    from plbpd_gb300 import capi
    rng = np.random.default_rng(13)
    reqs = [request_params(capi, rng, "D2Q9", capi.STORAGE_FP16_DEV) for _ in range(4)]
    out, errors = {}, []
    with capi.Server(budget_bytes=4 << 30, tick_steps=32) as srv:
        def client(k):
            p, m, n = reqs[k]
            rid = srv.submit(p, n, m)
            if k == 0:
                raise RuntimeError("client gave up")
            srv.wait(rid, 300.0)
            out[k] = srv.result(rid)[1]

        def guarded(k):
            try:
                client(k)
            except RuntimeError as ex:
                errors.append(str(ex))
        th = [threading.Thread(target=guarded, args=(k,)) for k in range(len(reqs))]
        for t in th:
            t.start()
        for t in th:
            t.join()
    assert errors == ["client gave up"]
    for k in range(1, len(reqs)):
        p, m, n = reqs[k]
        assert np.array_equal(out[k].view(np.uint32), run_alone(capi, p, m, n)[1].view(np.uint32))


def test_smaller_requests_are_admitted_first():
    """With the budget taken, the queued request with the least work is
    admitted first when room frees up (not the oldest)."""
    from plbpd_gb300 import capi
    rng = np.random.default_rng(21)
    p, m, _ = request_params(capi, rng, "D3Q19", capi.STORAGE_FP32)
    budget = int(capi.lib().plb_solve_bytes(capi.C.byref(p)) * 1.5)   # one at a time
    with capi.Server(budget_bytes=budget, tick_steps=20) as srv:
        first = srv.submit(p, 400, m)
        for _ in range(2000):
            if srv.status(first) == capi.REQ_RUNNING:
                break
            time.sleep(0.005)
        long_one = srv.submit(p, 300, m)     # older, more work
        short_one = srv.submit(p, 30, m)     # newer, less work
        for rid in (first, long_one, short_one):
            srv.wait(rid, 300.0)
        t_long = srv.result(long_one)[2]
        t_short = srv.result(short_one)[2]
        srv.result(first)
    assert t_short[1] <= t_long[1]           # admitted first
