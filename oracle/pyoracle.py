"""ctypes views of the oracle libraries.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, always as the checker; the product package never does.

* :class:`Port` drives the C restatement (``oracle/_build/liblbm_oracle.so``,
  built from ``oracle/lbm_oracle.c``), which runs everywhere.
* :class:`RefSim` drives the reference's own sources compiled with
  ``oracle/ref_harness.cpp`` (``oracle/_ref/libplbpd_ref_*.so``), which exist
  only where the reference was compiled (x86-64, with its sources present).

Both keep state in the reference's layout: AoS with one halo layer,
shape (nz+2, ny+2, nx+2, V).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liblbm_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

FACES = ("east", "west", "north", "south", "up", "down")
FACE_NONE, FACE_PERIODIC, FACE_NOSLIP = 0, 1, 2
MODE_REFERENCE, MODE_NATIVE = 0, 1
ARITH_AVX2, ARITH_SCALAR, ARITH_FP32, ARITH_FP16DEV, ARITH_FP32DEV = 0, 1, 2, 3, 4
N, NTMP, RHO, U = 0, 1, 2, 3
Q_OF = {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27}

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_port() -> str:
    """Compile the C restatement (gcc, OpenMP) and return the library path."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def _load_port() -> C.CDLL:
    if not os.path.exists(PORT_LIB):
        build_port()
    lib = C.CDLL(PORT_LIB)
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.c_int, C.c_long, C.c_long, C.c_long, C.c_float, C.c_float,
                               _fp, _fp, C.c_float, _ip, _ip, _fp, C.c_int, C.c_int, C.c_int]
    for name in ("orc_destroy", "orc_initialize", "orc_collide", "orc_stream", "orc_noslip",
                 "orc_periodic", "orc_moments", "orc_reset"):
        getattr(lib, name).argtypes = [C.c_void_p]
        getattr(lib, name).restype = None
    lib.orc_step.argtypes = [C.c_void_p, C.c_long]
    lib.orc_field_len.argtypes = [C.c_void_p, C.c_int]
    lib.orc_field_len.restype = C.c_size_t
    lib.orc_get_field.argtypes = [C.c_void_p, C.c_int, _fp]
    lib.orc_set_field.argtypes = [C.c_void_p, C.c_int, _fp]
    lib.orc_get_field_f64.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.orc_set_field_f64.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.orc_set_mask.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
    lib.orc_set_mask.restype = C.c_int
    lib.orc_set_trt.argtypes = [C.c_void_p, C.c_float]
    lib.orc_set_trt.restype = C.c_int
    lib.orc_relaxation.argtypes = [C.c_void_p, _fp, _fp]
    lib.orc_conservation.argtypes = [C.c_void_p, _dp]
    lib.orc_eqlb.argtypes = [C.c_int, C.c_float, _fp, _fp]
    lib.orc_model_tables.argtypes = [C.c_int, _ip, _fp, C.POINTER(C.c_uint32), _fp]
    lib.orc_model_tables.restype = C.c_int
    lib.orc_set_threads.argtypes = [C.c_int]
    lib.orc_round_half.argtypes = [C.c_float]
    lib.orc_round_half.restype = C.c_float
    lib.orc_store_half.argtypes = [C.c_float]
    lib.orc_store_half.restype = C.c_float
    lib.orc_max_threads.restype = C.c_int
    return lib


_PORT = None


def port_lib() -> C.CDLL:
    global _PORT
    if _PORT is None:
        _PORT = _load_port()
    return _PORT


def _faces(face_type: dict, face_vel: dict):
    ft = (C.c_int * 6)(*[{"periodic": FACE_PERIODIC, "noslip": FACE_NOSLIP}.get(face_type.get(f), FACE_NONE)
                         for f in FACES])
    hv = (C.c_int * 6)(*[1 if f in face_vel else 0 for f in FACES])
    fv = (C.c_float * 18)(*[float(v) for f in FACES for v in face_vel.get(f, (0.0, 0.0, 0.0))])
    return ft, hv, fv


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class _Sim:
    q: int
    nx: int
    ny: int
    nz: int

    def shape(self, which: int):
        v = {N: self.q, NTMP: self.q, RHO: 1, U: 3}[which]
        return (self.nz + 2, self.ny + 2, self.nx + 2, v)


class Port(_Sim):
    """The C restatement.  mode: MODE_REFERENCE | MODE_NATIVE; arith:
    ARITH_AVX2 | ARITH_SCALAR | ARITH_FP32 | ARITH_FP16DEV; precision 0 =
    float, 1 = double; trt: None (BGK) or the TRT magic parameter."""

    def __init__(self, model, nx, ny, nz, nu, rho0, u0, force, rho_solid, face_type, face_vel,
                 mode=MODE_REFERENCE, arith=ARITH_AVX2, precision=0, mask=None, threads=None, trt=None):
        self.lib = port_lib()
        self.q = Q_OF[model]
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        ft, hv, fv = _faces(face_type, face_vel)
        self.h = self.lib.orc_create(self.q, self.nx, self.ny, self.nz, float(nu), float(rho0), _f3(u0),
                                     _f3(force), float(rho_solid), ft, hv, fv, mode, arith, precision)
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        if threads is not None:
            self.lib.orc_set_threads(int(threads))
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
            assert m.shape == (self.nz, self.ny, self.nx)
            if self.lib.orc_set_mask(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8))) != 0:
                raise ValueError("mask needs MODE_NATIVE")
        if trt is not None:   # the TRT magic parameter (0 selects 3/16)
            if self.lib.orc_set_trt(self.h, float(trt)) != 0:
                raise ValueError("TRT needs FP32/FP16DEV arithmetic or double, and tau > 1/2")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.orc_destroy(h)
            self.h = None

    def initialize(self):
        self.lib.orc_initialize(self.h)

    def step(self, n=1):
        self.lib.orc_step(self.h, int(n))

    def collide(self): self.lib.orc_collide(self.h)
    def stream(self): self.lib.orc_stream(self.h)
    def noslip(self): self.lib.orc_noslip(self.h)
    def periodic(self): self.lib.orc_periodic(self.h)
    def moments(self): self.lib.orc_moments(self.h)
    def reset(self): self.lib.orc_reset(self.h)

    def get(self, which: int) -> np.ndarray:
        out = np.empty(self.shape(which), dtype=np.float32)
        self.lib.orc_get_field(self.h, which, out.ctypes.data_as(_fp))
        return out

    def get64(self, which: int) -> np.ndarray:
        out = np.empty(self.shape(which), dtype=np.float64)
        self.lib.orc_get_field_f64(self.h, which, out.ctypes.data_as(_dp))
        return out

    def set(self, which: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(self.shape(which))
        self.lib.orc_set_field(self.h, which, a.ctypes.data_as(_fp))

    def set64(self, which: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape(which))
        self.lib.orc_set_field_f64(self.h, which, a.ctypes.data_as(_dp))

    def relaxation(self):
        t, o = C.c_float(), C.c_float()
        self.lib.orc_relaxation(self.h, C.byref(t), C.byref(o))
        return t.value, o.value

    def conservation(self) -> np.ndarray:
        out = (C.c_double * 4)()
        self.lib.orc_conservation(self.h, out)
        return np.array(out[:])


def eqlb(model: str, rho: float, u) -> np.ndarray:
    q = Q_OF[model]
    out = (C.c_float * q)()
    port_lib().orc_eqlb(q, float(rho), _f3(u), out)
    return np.array(out[:], dtype=np.float32)


def model_tables(model: str):
    q = Q_OF[model]
    c = (C.c_int * (3 * q))()
    w = (C.c_float * q)()
    rev = (C.c_uint32 * q)()
    cs2 = C.c_float()
    port_lib().orc_model_tables(q, c, w, rev, C.byref(cs2))
    return (np.array(c[:], dtype=np.int32).reshape(q, 3), np.array(w[:], dtype=np.float32),
            np.array(rev[:], dtype=np.uint32), np.float32(cs2.value))


# ----------------------------------------------------------------------------
# the reference itself
# ----------------------------------------------------------------------------
REF_VARIANTS = {"avx2": "libplbpd_ref_avx2.so", "scalar": "libplbpd_ref_scalar.so",
                "omp": "libplbpd_ref_omp.so"}
_REF = {}


def ref_available(variant: str = "avx2") -> bool:
    return os.path.exists(os.path.join(REF_DIR, REF_VARIANTS[variant]))


def ref_lib(variant: str = "avx2") -> C.CDLL:
    if variant not in _REF:
        lib = C.CDLL(os.path.join(REF_DIR, REF_VARIANTS[variant]))
        lib.refh_create.restype = C.c_void_p
        lib.refh_create.argtypes = [C.c_char_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_float, C.c_float,
                                    _fp, _fp, C.c_float, _ip, _ip, _fp]
        for name in ("refh_destroy", "refh_initialize", "refh_noslip", "refh_periodic", "refh_moments",
                     "refh_reset"):
            getattr(lib, name).argtypes = [C.c_void_p]
            getattr(lib, name).restype = None
        lib.refh_collide.argtypes = [C.c_void_p, C.c_int]
        lib.refh_stream.argtypes = [C.c_void_p, C.c_int]
        lib.refh_march.argtypes = [C.c_void_p, C.c_size_t]
        lib.refh_get_field.argtypes = [C.c_void_p, C.c_int, _fp]
        lib.refh_set_field.argtypes = [C.c_void_p, C.c_int, _fp]
        lib.refh_eqlb.argtypes = [C.c_char_p, C.c_float, _fp, _fp]
        lib.refh_model_tables.argtypes = [C.c_char_p, _ip, _fp, C.POINTER(C.c_uint), _fp]
        lib.refh_model_tables.restype = C.c_int
        lib.refh_set_threads.argtypes = [C.c_int]
        lib.refh_max_threads.restype = C.c_int
        _REF[variant] = lib
    return _REF[variant]


class RefSim(_Sim):
    """The reference's own classes (LBModel, Domain, Boundary, SimData, PLBPD)."""

    def __init__(self, model, nx, ny, nz, nu, rho0, u0, force, rho_solid, face_type, face_vel,
                 variant="avx2", threads=1):
        self.lib = ref_lib(variant)
        self.q = Q_OF[model]
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        ft, hv, fv = _faces(face_type, face_vel)
        self.lib.refh_set_threads(int(threads))
        self.h = self.lib.refh_create(model.encode(), self.nx, self.ny, self.nz, float(nu), float(rho0),
                                      _f3(u0), _f3(force), float(rho_solid), ft, hv, fv)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.refh_destroy(h)
            self.h = None

    def initialize(self): self.lib.refh_initialize(self.h)
    def march(self, n): self.lib.refh_march(self.h, int(n))

    def step(self, n=1):
        """PLBPD::march_in_time's phases, called one by one (no timing print)."""
        for _ in range(int(n)):
            self.lib.refh_collide(self.h, 0)
            self.lib.refh_stream(self.h, 0)
            self.lib.refh_noslip(self.h)
            self.lib.refh_periodic(self.h)
            self.lib.refh_moments(self.h)
            self.lib.refh_reset(self.h)

    def collide(self, reference=False): self.lib.refh_collide(self.h, int(reference))
    def stream(self, reference=False): self.lib.refh_stream(self.h, int(reference))
    def noslip(self): self.lib.refh_noslip(self.h)
    def periodic(self): self.lib.refh_periodic(self.h)
    def moments(self): self.lib.refh_moments(self.h)
    def reset(self): self.lib.refh_reset(self.h)

    def get(self, which: int) -> np.ndarray:
        out = np.empty(self.shape(which), dtype=np.float32)
        self.lib.refh_get_field(self.h, which, out.ctypes.data_as(_fp))
        return out

    def set(self, which: int, arr) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(self.shape(which))
        self.lib.refh_set_field(self.h, which, a.ctypes.data_as(_fp))
