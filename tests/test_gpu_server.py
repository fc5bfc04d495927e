"""The solve server: requests of mixed lattice, size, tau, storage, mask and
step count run together (continuous batching) and each result equals the
same request run alone; admission respects the memory budget."""
import threading

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
