"""Batches: many domains of different size, tau, force, walls and obstacles
advanced together by the tile-list kernel give, bit for bit, what each domain
gives advanced alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DUCT = {"east": "periodic", "west": "periodic", "north": "noslip", "south": "noslip", "up": "noslip",
        "down": "noslip"}
REST = {f: (0.0, 0.0, 0.0) for f in ("north", "south", "up", "down")}


def make_solves(capi, storage, seed=5, count=7, model="D3Q19", even_fp16=True):
    from plbpd_gb300.workloads import porous_mask
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        L = int(rng.integers(6, 30))
        nx, ny, nz = L + int(rng.integers(0, 5)), L, L + int(rng.integers(0, 3))
        if storage == capi.STORAGE_FP16_DEV and even_fp16:
            nx += nx % 2
        tau = float(rng.uniform(0.55, 1.2))
        vel = dict(REST)
        if i % 3 == 0:
            vel["up"] = (0.02, 0.0, 0.0)   # a moving lid on some domains
        s = capi.Solve.create(model, nx, ny, nz, (tau - 0.5) / 3.0, force=(float(rng.uniform(1e-6, 1e-4)), 0.0, 0.0),
                              u0=(0.005, 0.0, 0.0), face_type=DUCT, face_vel=vel,
                              semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32, storage=storage)
        if i % 2 == 0:
            s.set_mask(porous_mask(nx, ny, nz, float(rng.uniform(0.7, 0.9)), seed + i))
        s.initialize()
        out.append(s)
    return out


@pytest.mark.parametrize("multi", ["0", "1"])
@pytest.mark.parametrize("storage_name", ["fp32", "fp16", "fp16_odd", "fp32dev"])
@pytest.mark.parametrize("model", ["D3Q19", "D3Q27"])
def test_batch_equals_each_domain_alone(storage_name, model, multi, monkeypatch):
    """Domains with even nx run as pair tasks, the others as one-node tasks,
    in the same launch (fp16_odd: FP16 domains of both kinds); one launch a
    step in graph chunks, or a call's steps in one cooperative launch with
    grid barriers (PLB_BATCH_MULTI=1)."""
    monkeypatch.setenv("PLB_BATCH_MULTI", multi)
    from plbpd_gb300 import capi
    storage = {"fp32": capi.STORAGE_FP32, "fp16": capi.STORAGE_FP16_DEV, "fp16_odd": capi.STORAGE_FP16_DEV,
               "fp32dev": capi.STORAGE_FP32_DEV}[storage_name]
    even = storage_name != "fp16_odd"
    mix = make_solves(capi, storage, model=model, even_fp16=even)
    alone = make_solves(capi, storage, model=model, even_fp16=even)
    assert len({s.nx % 2 for s in mix}) == (1 if storage_name == "fp16" else 2)
    with capi.Batch(mix) as b:
        b.step(1)       # first collision from the initial state
        b.step(140)     # graph chunks plus a tail
        b.step(3)
    for s in alone:
        s.step(144)
    for a, m in zip(alone, mix):
        for w in (capi.FIELD_N, capi.FIELD_RHO, capi.FIELD_U):
            ga, gm = a.get(w), m.get(w)
            assert np.array_equal(ga.view(np.uint32), gm.view(np.uint32)), f"field {w} differs"
        np.testing.assert_array_equal(a.conservation(), m.conservation())


def test_batch_mixed_states():
    """Members that were stepped on their own before joining stay in step."""
    from plbpd_gb300 import capi
    mix = make_solves(capi, capi.STORAGE_FP32, seed=9, count=4)
    alone = make_solves(capi, capi.STORAGE_FP32, seed=9, count=4)
    mix[1].step(3)
    alone[1].step(3)
    with capi.Batch(mix) as b:
        b.step(10)
    for s in alone:
        s.step(10)
    for a, m in zip(alone, mix):
        assert np.array_equal(a.get(capi.FIELD_U).view(np.uint32), m.get(capi.FIELD_U).view(np.uint32))


def test_batch_rejects_mixed_lattices():
    from plbpd_gb300 import capi
    a = capi.Solve.create("D3Q19", 8, 8, 8, 0.1, face_type={f: "periodic" for f in capi.FACES},
                          semantics=capi.SEMANTICS_NATIVE)
    b = capi.Solve.create("D3Q27", 8, 8, 8, 0.1, face_type={f: "periodic" for f in capi.FACES},
                          semantics=capi.SEMANTICS_NATIVE)
    with pytest.raises(capi.PlbError):
        capi.Batch([a, b])


def test_batch_refuses_member_with_changed_collision():
    """The batch's kernel is fixed at creation: a member switched from BGK to
    TRT afterwards is refused, not run under the BGK kernel."""
    from plbpd_gb300 import capi
    mix = make_solves(capi, capi.STORAGE_FP32, seed=11, count=3)
    with capi.Batch(mix) as b:
        b.step(4)
        mix[1].set_collision(capi.COLLISION_TRT)
        with pytest.raises(capi.PlbError) as e:
            b.step(2)
        assert e.value.code == capi.ESTATE
        mix[1].set_collision(capi.COLLISION_BGK)
        b.step(2)   # back to the batch's operator: accepted


def test_member_calls_follow_batch_without_synchronize():
    """A member's own calls after plb_batch_step_async see the batch's result
    (its stream waits for the batch's work), with no plb_batch_synchronize."""
    from plbpd_gb300 import capi
    mix = make_solves(capi, capi.STORAGE_FP32, seed=13, count=3)
    alone = make_solves(capi, capi.STORAGE_FP32, seed=13, count=3)
    with capi.Batch(mix) as b:
        b.step_async(1)
        b.step_async(130)
        got = [m.get(capi.FIELD_U) for m in mix]
        cons = [m.conservation() for m in mix]
        b.synchronize()
    for s in alone:
        s.step(131)
    for a, g, c in zip(alone, got, cons):
        assert np.array_equal(a.get(capi.FIELD_U).view(np.uint32), g.view(np.uint32))
        np.testing.assert_array_equal(a.conservation(), c)


def test_batch_barrier_timeout_is_reported(monkeypatch):
    """A grid barrier of the multi-step kernel that cannot complete (fault
    injection: its arrival count starts past the grid) ends the launch after
    its bounded wait; plb_batch_synchronize reports PLB_ETIMEOUT and the
    context stays usable: a fresh batch of the same domains then matches
    the domains advanced alone."""
    import time
    from plbpd_gb300 import capi
    monkeypatch.setenv("PLB_BATCH_MULTI", "1")
    mix = make_solves(capi, capi.STORAGE_FP32, seed=21, count=3)
    with capi.Batch(mix) as b:
        b.step(2)
        b.fault_barrier()
        t0 = time.perf_counter()
        with pytest.raises(capi.PlbError) as e:
            b.step(5)
        assert e.value.code == capi.ETIMEOUT
        assert time.perf_counter() - t0 < 60.0
    fresh = make_solves(capi, capi.STORAGE_FP32, seed=23, count=3)
    alone = make_solves(capi, capi.STORAGE_FP32, seed=23, count=3)
    with capi.Batch(fresh) as b:
        b.step(9)
    for s in alone:
        s.step(9)
    for a, m in zip(alone, fresh):
        assert np.array_equal(a.get(capi.FIELD_U).view(np.uint32), m.get(capi.FIELD_U).view(np.uint32))
