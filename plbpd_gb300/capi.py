"""ctypes binding of the C ABI in include/plb.h (libplb_gb300.so).

The library is the only compute path: if it has not been built, importing the
binding raises, and there is no CPU fallback.  Arrays crossing the boundary
use plbpd's Field layout, shape (nz+2, ny+2, nx+2, V) in float32.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libplb_gb300.so")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ESTATE, EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6
FACE_NONE, FACE_PERIODIC, FACE_NOSLIP = 0, 1, 2
FACES = ("east", "west", "north", "south", "up", "down")
SEMANTICS_REFERENCE, SEMANTICS_NATIVE = 0, 1
ARITH_REFERENCE, ARITH_FP32 = 0, 1
COLLISION_BGK, COLLISION_TRT = 0, 1
STREAMING_AB, STREAMING_AA = 0, 1
STORAGE_FP32, STORAGE_FP16_DEV, STORAGE_FP64, STORAGE_FP32_DEV = 0, 1, 2, 3
FIELD_N, FIELD_NTMP, FIELD_RHO, FIELD_U = 0, 1, 2, 3
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4
Q_OF = {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27}


class PlbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"plb error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("q", C.c_int32), ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("nu", C.c_float), ("rho0", C.c_float), ("u0", C.c_float * 3), ("force", C.c_float * 3),
                ("rho_solid", C.c_float), ("face_type", C.c_int32 * 6), ("face_has_vel", C.c_int32 * 6),
                ("face_vel", (C.c_float * 3) * 6), ("semantics", C.c_int32), ("arith", C.c_int32),
                ("storage", C.c_int32), ("device", C.c_int32), ("collision", C.c_int32), ("trt_magic", C.c_float),
                ("streaming", C.c_int32)]


# (name, restype, argtypes) of every entry point declared in include/plb.h
_SIGS = [
    ("plb_last_error", C.c_char_p, []),
    ("plb_version", C.c_int, []),
    ("plb_model_tables", C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("plb_equilibrium", C.c_int, [C.c_int32, C.c_float, C.c_void_p, C.c_void_p]),
    ("plb_relaxation", C.c_int, [C.c_float, C.c_void_p, C.c_void_p]),
    ("plb_solve_create", C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    ("plb_solve_destroy", C.c_int, [C.c_void_p]),
    ("plb_set_relaxation", C.c_int, [C.c_void_p, C.c_float, C.c_void_p]),
    ("plb_set_collision", C.c_int, [C.c_void_p, C.c_int32, C.c_float]),
    ("plb_set_boundary", C.c_int, [C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("plb_set_mask", C.c_int, [C.c_void_p, C.c_void_p]),
    ("plb_initialize", C.c_int, [C.c_void_p]),
    ("plb_step", C.c_int, [C.c_void_p, C.c_int64]),
    ("plb_step_async", C.c_int, [C.c_void_p, C.c_int64]),
    ("plb_synchronize", C.c_int, [C.c_void_p]),
    ("plb_stream_handle", C.c_void_p, [C.c_void_p]),
    ("plb_tune_variants", C.c_int, []),
    ("plb_tune_force", C.c_int, [C.c_int32]),
    ("plb_tune_variant", C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    ("plb_tune", C.c_int, [C.c_void_p]),
    ("plb_collide", C.c_int, [C.c_void_p]),
    ("plb_stream_push", C.c_int, [C.c_void_p]),
    ("plb_apply_noslip", C.c_int, [C.c_void_p]),
    ("plb_apply_periodicity", C.c_int, [C.c_void_p]),
    ("plb_calc_moments", C.c_int, [C.c_void_p]),
    ("plb_reset", C.c_int, [C.c_void_p]),
    ("plb_reset_velocity", C.c_int, [C.c_void_p]),
    ("plb_reset_density", C.c_int, [C.c_void_p]),
    ("plb_field_len", C.c_size_t, [C.c_void_p, C.c_int32]),
    ("plb_get_field", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    ("plb_set_field", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    ("plb_conservation", C.c_int, [C.c_void_p, C.c_void_p]),
    ("plb_conservation_static", C.c_int, [C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    ("plb_batch_create", C.c_int, [C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("plb_batch_step", C.c_int, [C.c_void_p, C.c_int64]),
    ("plb_batch_step_async", C.c_int, [C.c_void_p, C.c_int64]),
    ("plb_batch_synchronize", C.c_int, [C.c_void_p]),
    ("plb_batch_destroy", C.c_int, [C.c_void_p]),
    ("plb_batch_cells", C.c_int64, [C.c_void_p]),
    ("plb_batch_fault_barrier", C.c_int, [C.c_void_p]),
    ("plb_batch_stream_handle", C.c_void_p, [C.c_void_p]),
    ("plb_solve_bytes", C.c_int64, [C.POINTER(Params)]),
    ("plb_server_start", C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_void_p)]),
    ("plb_server_submit", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    ("plb_server_status", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    ("plb_server_cancel", C.c_int, [C.c_void_p, C.c_int64]),
    ("plb_server_wait", C.c_int, [C.c_void_p, C.c_int64, C.c_double]),
    ("plb_server_result", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("plb_server_memory", C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("plb_server_stop", C.c_int, [C.c_void_p]),
    ("plb_host_alloc", C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    ("plb_host_free", C.c_int, [C.c_void_p]),
    ("plb_device_bytes", C.c_int64, [C.c_void_p]),
]

_LIB = None


def lib() -> C.CDLL:
    """The loaded native library; raises if it was not built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with plbpd_gb300.build.build() "
                              "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in _SIGS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(rc: int) -> int:
    if rc < 0:
        raise PlbError(rc, lib().plb_last_error().decode(errors="replace"))
    return rc


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def model_tables(name: str):
    q = Q_OF.get(name, 27)
    c = np.zeros((q, 3), np.int32)
    w = np.zeros(q, np.float32)
    rev = np.zeros(q, np.uint32)
    cs2 = np.zeros(1, np.float32)
    q = check(lib().plb_model_tables(name.encode(), _ptr(c), _ptr(w), _ptr(rev), _ptr(cs2)))
    return c[:q], w[:q], rev[:q], np.float32(cs2[0])


def equilibrium(q: int, rho: float, u) -> np.ndarray:
    uu = np.asarray(u, np.float32)
    out = np.zeros(q, np.float32)
    check(lib().plb_equilibrium(q, rho, _ptr(uu), _ptr(out)))
    return out


def relaxation(nu: float):
    t = np.zeros(1, np.float32)
    o = np.zeros(1, np.float32)
    check(lib().plb_relaxation(nu, _ptr(t), _ptr(o)))
    return float(t[0]), float(o[0])


def make_params(model: str, nx: int, ny: int, nz: int, nu: float, rho0: float = 1.0, u0=(0, 0, 0),
                force=(0, 0, 0), rho_solid: float = 1.0, face_type: dict | None = None,
                face_vel: dict | None = None, semantics: int = SEMANTICS_REFERENCE,
                arith: int = ARITH_REFERENCE, storage: int = STORAGE_FP32, device: int = 0,
                collision: int = COLLISION_BGK, trt_magic: float = 0.0, streaming: int = STREAMING_AB) -> Params:
    face_type = face_type or {}
    face_vel = face_vel or {}
    p = Params()
    p.q = Q_OF[model]
    p.nx, p.ny, p.nz = int(nx), int(ny), int(nz)
    p.nu, p.rho0, p.rho_solid = float(nu), float(rho0), float(rho_solid)
    for i in range(3):
        p.u0[i] = float(u0[i])
        p.force[i] = float(force[i])
    for f, name in enumerate(FACES):
        t = face_type.get(name)
        p.face_type[f] = {"periodic": FACE_PERIODIC, "noslip": FACE_NOSLIP}.get(t, FACE_NONE)
        if name in face_vel:
            p.face_has_vel[f] = 1
            for i in range(3):
                p.face_vel[f][i] = float(face_vel[name][i])
    p.semantics, p.arith, p.storage, p.device = int(semantics), int(arith), int(storage), int(device)
    p.collision, p.trt_magic, p.streaming = int(collision), float(trt_magic), int(streaming)
    return p


class Solve:
    """One device-resident solve (plb_solve)."""

    def __init__(self, params: Params):
        self.params = params
        self.q = int(params.q)
        self.nx, self.ny, self.nz = int(params.nx), int(params.ny), int(params.nz)
        h = C.c_void_p()
        check(lib().plb_solve_create(C.byref(params), C.byref(h)))
        self.h = h

    @classmethod
    def create(cls, *args, **kw) -> "Solve":
        return cls(make_params(*args, **kw))

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().plb_solve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def shape(self, which: int):
        v = {FIELD_N: self.q, FIELD_NTMP: self.q, FIELD_RHO: 1, FIELD_U: 3}[which]
        return (self.nz + 2, self.ny + 2, self.nx + 2, v)

    def set_mask(self, mask) -> None:
        if mask is None:
            check(lib().plb_set_mask(self.h, None))
            return
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        assert m.shape == (self.nz, self.ny, self.nx)
        check(lib().plb_set_mask(self.h, _ptr(m)))

    def set_collision(self, collision: int, trt_magic: float = 0.0) -> None:
        check(lib().plb_set_collision(self.h, int(collision), float(trt_magic)))

    def initialize(self) -> None: check(lib().plb_initialize(self.h))
    def step(self, n: int = 1) -> None: check(lib().plb_step(self.h, int(n)))
    def step_async(self, n: int = 1) -> None: check(lib().plb_step_async(self.h, int(n)))
    def synchronize(self) -> None: check(lib().plb_synchronize(self.h))
    def stream(self) -> int: return lib().plb_stream_handle(self.h) or 0

    def variant(self) -> int:
        """The fused-step kernel variant the autotuner chose (-1 before the
        first fused step)."""
        v = C.c_int32()
        check(lib().plb_tune_variant(self.h, C.byref(v)))
        return v.value

    def tune(self) -> int:
        """Times the fused-step variants on the current state now, keeps the
        fastest (no later trial) and returns it."""
        check(lib().plb_tune(self.h))
        return self.variant()
    def collide(self) -> None: check(lib().plb_collide(self.h))
    def stream_push(self) -> None: check(lib().plb_stream_push(self.h))
    def apply_noslip(self) -> None: check(lib().plb_apply_noslip(self.h))
    def apply_periodicity(self) -> None: check(lib().plb_apply_periodicity(self.h))
    def calc_moments(self) -> None: check(lib().plb_calc_moments(self.h))
    def reset(self) -> None: check(lib().plb_reset(self.h))
    def reset_velocity(self) -> None: check(lib().plb_reset_velocity(self.h))
    def reset_density(self) -> None: check(lib().plb_reset_density(self.h))

    def get(self, which: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape(which), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == lib().plb_field_len(self.h, which)
        check(lib().plb_get_field(self.h, which, _ptr(out)))
        return out

    def set(self, which: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32)
        assert a.size == lib().plb_field_len(self.h, which)
        check(lib().plb_set_field(self.h, which, _ptr(a)))

    def conservation(self) -> np.ndarray:
        out = np.zeros(4, np.float64)
        check(lib().plb_conservation(self.h, _ptr(out)))
        return out

    def device_bytes(self) -> int:
        return int(lib().plb_device_bytes(self.h))


class PinnedBuffer:
    """Page-locked host memory (plb_host_alloc) viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        check(lib().plb_host_alloc(self.nbytes, C.byref(p)))
        self._p = p
        buf = (C.c_char * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self) -> None:
        if self._p:
            self.array = None
            lib().plb_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many NATIVE solves advanced together (plb_batch); the solves stay
    usable on their own between batch calls."""

    def __init__(self, solves):
        self.solves = list(solves)
        arr = (C.c_void_p * len(self.solves))(*[s.h.value for s in self.solves])
        h = C.c_void_p()
        check(lib().plb_batch_create(len(self.solves), C.cast(arr, C.c_void_p), C.byref(h)))
        self.h = h

    def step(self, n: int = 1) -> None: check(lib().plb_batch_step(self.h, int(n)))
    def step_async(self, n: int = 1) -> None: check(lib().plb_batch_step_async(self.h, int(n)))
    def synchronize(self) -> None: check(lib().plb_batch_synchronize(self.h))
    def cells(self) -> int: return int(lib().plb_batch_cells(self.h))
    def fault_barrier(self) -> None: check(lib().plb_batch_fault_barrier(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().plb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Request(C.Structure):
    """plb_request: one solve for the server."""
    _fields_ = [("params", Params), ("mask", C.c_void_p), ("steps", C.c_int64)]


def tune_variants() -> int:
    """Number of compiled variants of the fused-step kernel."""
    return lib().plb_tune_variants()


def tune_force(variant: int) -> None:
    """Fixes the kernel variant of solves that have not chosen yet (-1: tune)."""
    check(lib().plb_tune_force(int(variant)))


class Server:
    """The solve server (plb_server_*): submit requests as they arrive, wait,
    collect rho/u.  Requests use NATIVE semantics."""

    def __init__(self, budget_bytes: int, tick_steps: int = 256, device: int = 0):
        h = C.c_void_p()
        check(lib().plb_server_start(int(device), int(budget_bytes), int(tick_steps), C.byref(h)))
        self.h = h
        self._dims = {}

    def submit(self, params: Params, steps: int, mask=None) -> int:
        req = Request()
        req.params = params
        req.steps = int(steps)
        m = None
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
            assert m.shape == (int(params.nz), int(params.ny), int(params.nx))
            req.mask = m.ctypes.data
        rid = C.c_int64()
        check(lib().plb_server_submit(self.h, C.byref(req), C.byref(rid)))   # copies the mask
        self._dims[rid.value] = (int(params.nz) + 2, int(params.ny) + 2, int(params.nx) + 2)
        return rid.value

    def status(self, rid: int) -> int:
        st = C.c_int32()
        check(lib().plb_server_status(self.h, int(rid), C.byref(st)))
        return st.value

    def cancel(self, rid: int) -> None:
        check(lib().plb_server_cancel(self.h, int(rid)))

    def wait(self, rid: int, timeout_s: float = 600.0) -> None:
        check(lib().plb_server_wait(self.h, int(rid), float(timeout_s)))

    def result(self, rid: int):
        """(rho, u, (t_submit, t_admit, t_done)) of a finished request."""
        shape = self._dims.pop(int(rid))
        rho = np.empty(shape + (1,), np.float32)
        u = np.empty(shape + (3,), np.float32)
        t = np.zeros(3, np.float64)
        check(lib().plb_server_result(self.h, int(rid), _ptr(rho), _ptr(u), _ptr(t)))
        return rho, u, tuple(float(x) for x in t)

    def memory(self):
        a, b = C.c_int64(), C.c_int64()
        check(lib().plb_server_memory(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def stop(self) -> None:
        if getattr(self, "h", None):
            lib().plb_server_stop(self.h)
            self.h = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()
