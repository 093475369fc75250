"""ctypes front end of the CPU restatement (oracle/mpm_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline leg.  The product path never imports
it.

``advance(state, steps, contact)`` runs the one-thread build (particle index
order, the order the golden states were produced in) in place on a
``code_mpm_gb300.snapshot.State`` (contact 2: the non-contact loop with the
large-strain pass 2, which keeps the elastic deformation gradient in
``state["F_elastic"]``); ``advance(..., threads=N, omp=True)`` runs
the OpenMP build that mirrors the reference's per-node-lock parallel loop,
which is only ever timed.  ``advance_work`` is ``advance`` that also sums the
boundary work (displacement control, friction) the engine's monitors report.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_lock = threading.Lock()
_libs = {}


def build() -> None:
    """Compile the restatement with make (a second or two)."""
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)


def _lib(omp: bool):
    name = "libmpm_oracle_omp.so" if omp else "libmpm_oracle.so"
    with _lock:
        if name not in _libs:
            path = os.path.join(BUILD, name)
            if not os.path.exists(path):
                build()
            lib = C.CDLL(path)
            lib.oracle_advance.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
            lib.oracle_advance.restype = C.c_int
            lib.oracle_threads_available.restype = C.c_int
            lib.oracle_advance_work.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
            lib.oracle_advance_work.restype = C.c_int
            _libs[name] = lib
        return _libs[name]


class _Header(C.Structure):
    _fields_ = [("magic", C.c_char * 8), ("version", C.c_uint32), ("contact", C.c_uint32),
                ("length", C.c_double * 3), ("cells", C.c_int32 * 3), ("pad0", C.c_int32),
                ("time", C.c_double), ("dt_max", C.c_double), ("mass_min", C.c_double),
                ("damping", C.c_double), ("step", C.c_int64), ("n_particles", C.c_uint64),
                ("n_nodes", C.c_uint64), ("n_materials", C.c_uint32), ("n_timeline", C.c_uint32),
                ("n_dc", C.c_uint32), ("flags", C.c_uint32)]


_PTRS = ("materials", "tl_time", "tl_vel", "pos", "vel", "fext", "mass", "vol", "vol0", "F", "stress", "strain",
         "eps_p", "e_strain", "e_strain_max", "e_strain_ti", "e_plastic", "backstress", "mp_mass_gradient",
         "strain_rate", "material", "pflags", "dc_mult", "dc_list", "fixed", "friction", "g_mass", "g_mom", "g_vel",
         "g_force", "g_force_temp", "g_mass_gradient", "g_state")


class _Snap(C.Structure):
    _fields_ = [("h", _Header)] + [(n, C.c_void_p) for n in _PTRS] + [("F_elastic", C.c_void_p)]


def _make_snap(st):
    for k in _PTRS:
        a = st.arrays[k]
        if not a.flags["C_CONTIGUOUS"]:
            st.arrays[k] = np.ascontiguousarray(a)
    s = _Snap()
    h = s.h
    h.magic = b"MPMSNAP1"
    h.version = 1
    h.contact = int(st.contact)
    for a in range(3):
        h.length[a] = float(st.length[a])
        h.cells[a] = int(st.cells[a])
    h.time, h.dt_max, h.mass_min, h.damping = float(st.time), float(st.dt_max), float(st.mass_min), float(st.damping)
    h.step = int(st.step)
    h.n_particles = st.n_particles
    h.n_nodes = st.n_nodes
    h.n_materials = len(st.arrays["materials"])
    h.n_timeline = len(st.arrays["tl_time"])
    h.n_dc = len(st.arrays["dc_list"])
    for k in _PTRS:
        setattr(s, k, st.arrays[k].ctypes.data)
    if "F_elastic" not in st.arrays:
        from code_mpm_gb300 import snapshot

        st.arrays["F_elastic"] = snapshot.identity_f(st.n_particles)
    st.arrays["F_elastic"] = np.ascontiguousarray(st.arrays["F_elastic"], dtype=np.float64)
    s.F_elastic = st.arrays["F_elastic"].ctypes.data
    h.flags = 1
    return s


def advance(st, steps: int, contact: int, floor_friction: int = 0, threads: int = 0, omp: bool = False) -> float:
    """Advance ``st`` in place by ``steps`` steps of ``st.dt_max``; returns loop seconds (OpenMP build only)."""
    lib = _lib(omp)
    if len(st.arrays["g_mass"]) != st.n_nodes:
        raise ValueError("the oracle needs every node array (this State holds only the nodes' boundary conditions)")
    s = _make_snap(st)
    sec = C.c_double(0.0)
    rc = lib.oracle_advance(C.byref(s), int(steps), int(contact), int(floor_friction), int(threads), C.byref(sec))
    if rc != 0:
        raise RuntimeError(f"oracle_advance failed ({rc})")
    st.time = s.h.time
    st.step = s.h.step
    st.contact = s.h.contact
    return sec.value


def advance_work(st, steps: int, contact: int, floor_friction: int = 0, work=None):
    """As advance() (one-thread build), also summing the boundary work of the steps: returns
    [displacement-control work, friction work] added to `work` (a 2-list, zeros if None)."""
    lib = _lib(False)
    if len(st.arrays["g_mass"]) != st.n_nodes:
        raise ValueError("the oracle needs every node array (this State holds only the nodes' boundary conditions)")
    s = _make_snap(st)
    w = (C.c_double * 2)(*(work or (0.0, 0.0)))
    rc = lib.oracle_advance_work(C.byref(s), int(steps), int(contact), int(floor_friction), w)
    if rc != 0:
        raise RuntimeError(f"oracle_advance_work failed ({rc})")
    st.time = s.h.time
    st.step = s.h.step
    st.contact = s.h.contact
    return [w[0], w[1]]


def threads_available() -> int:
    return int(_lib(True).oracle_threads_available())
