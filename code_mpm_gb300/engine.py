"""Host-side mirror of the reference's PhysicsEngine solver interface over the C ABI.

``Engine`` owns one ``mpm_ctx`` (include/mpm_gb300.h) and exposes the
reference's entry points with their meaning and return values:

    runSimulation_Classic_DoublePass_MPLocks(dTimeIncrement_Total)          PhysicsEngine.h:54
    runSimulation_Classic_DoublePass_MPLocks_Contact(dTimeIncrement_Total)  PhysicsEngine.h:55
        advance by dTimeIncrement_Total in steps of d_TimeIncrement_Maximum,
        the last one shortened (…MPLocks.cpp:449-458); return 1 once
        d_Time >= d_TimeEnd, else 0 (:806-814)
    getTime_Current / getTime_End / getTime_Increment                       PhysicsEngine.h:66-71
    getCount_MaterialPoint / getCount_GridPoint                             PhysicsEngine.h:73-75

plus state transfer as ``code_mpm_gb300.snapshot.State``.  Every call goes
through libmpm_gb300.so; there is no CPU path, and a missing library or
device raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional

import numpy as np

from . import snapshot
from .snapshot import State

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmpm_gb300.so")
_lib = None

FORM_FP64 = 0
FORM_FP32 = 1
OPT_FLOOR_FRICTION = 1
OPT_PROFILE = 2


class MPMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mpm error {code}: {msg}")
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [("length", C.c_double * 3), ("cells", C.c_int32 * 3), ("pad", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("pad", C.c_int32), ("density", C.c_double), ("E", C.c_double),
                ("nu", C.c_double), ("yield_", C.c_double), ("C0", C.c_double), ("C1", C.c_double)]


class Sim(C.Structure):
    _fields_ = [("time", C.c_double), ("dt_max", C.c_double), ("mass_min", C.c_double), ("damping", C.c_double),
                ("time_end", C.c_double), ("step", C.c_int64)]


_PFIELDS = ("pos", "vel", "fext", "mass", "vol", "vol0", "F", "stress", "strain", "eps_p", "e_strain", "e_strain_max",
            "e_strain_ti", "e_plastic", "backstress", "mp_mass_gradient", "strain_rate")


class Particles(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in _PFIELDS] + [("material", C.c_void_p), ("pflags", C.c_void_p),
                                                      ("dc_mult", C.c_void_p), ("specimen", C.c_void_p),
                                                      ("F_elastic", C.c_void_p)]


_NMAP = (("fixed", "fixed"), ("friction", "friction"), ("mass", "g_mass"), ("mom", "g_mom"), ("vel", "g_vel"),
         ("force", "g_force"), ("force_temp", "g_force_temp"), ("mass_gradient", "g_mass_gradient"),
         ("state", "g_state"))


class Nodes(C.Structure):
    _fields_ = [(k, C.c_void_p) for k, _ in _NMAP]


class NetConfig(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("yield_", C.c_double), ("C0", C.c_double),
                ("C1", C.c_double), ("n_samples", C.c_int64), ("batch", C.c_int32), ("epochs", C.c_int32),
                ("lr", C.c_double), ("stress_range", C.c_double), ("epbar_max", C.c_double),
                ("deps_sigma", C.c_double), ("seed", C.c_uint64), ("sampling", C.c_int32), ("pad", C.c_int32)]


class NetReport(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("val_rms_dsig", C.c_double),
                ("val_rms_dsig_outside", C.c_double), ("val_max_dsig", C.c_double), ("val_rms_dR", C.c_double),
                ("seconds_generate", C.c_double), ("seconds_train", C.c_double), ("steps", C.c_int64),
                ("n_val", C.c_int64), ("out_scale", C.c_double * 8), ("out_shift", C.c_double * 8)]


class SurrogateStats(C.Structure):
    _fields_ = [("queued", C.c_int64), ("band", C.c_int64), ("rechecked", C.c_int64), ("recheck_rms", C.c_double),
                ("recheck_max", C.c_double), ("rejected", C.c_int64)]


class HoneycombDesc(C.Structure):  # mpm_honeycomb_desc (include/mpm_scene.h)
    _fields_ = [("wall", C.c_double), ("pitch", C.c_double), ("h", C.c_double), ("origin", C.c_double * 3),
                ("ncell", C.c_int32), ("layers", C.c_int32)]


class FoamDesc(C.Structure):  # mpm_foam_desc (include/mpm_scene.h)
    _fields_ = [("pitch", C.c_double), ("t0", C.c_double), ("t1", C.c_double), ("h", C.c_double),
                ("height", C.c_double), ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
                ("ncell", C.c_int32), ("width", C.c_int32), ("layers", C.c_int32), ("pad", C.c_int32),
                ("fx", C.c_void_p), ("fy", C.c_void_p)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("total_ms", C.c_double)]


class TuneResult(C.Structure):
    _fields_ = [("p2g_reduce", C.c_int32), ("p2g_block", C.c_int32), ("pass_block", C.c_int32),
                ("candidates", C.c_int32), ("best_ms_per_step", C.c_double), ("worst_ms_per_step", C.c_double),
                ("gather_batch", C.c_int32), ("pass1_corners", C.c_int32), ("pass1_block", C.c_int32)]


class Monitors(C.Structure):
    _fields_ = [("time", C.c_double), ("position_mean", C.c_double * 3), ("force_sum", C.c_double * 3),
                ("momentum", C.c_double * 3), ("strain_p_max", C.c_double), ("stress_p_max", C.c_double),
                ("stress_mean", C.c_double * 3), ("strain_mean", C.c_double * 3), ("kinetic", C.c_double),
                ("strain_energy", C.c_double), ("plastic_energy", C.c_double), ("count", C.c_int64 * 5),
                ("platen_work", C.c_double), ("friction_work", C.c_double)]


MON_DISPLACEMENT, MON_MOMENTUM, MON_PRINCIPAL, MON_STRESS, MON_ENERGY = 1, 2, 4, 8, 16

OPT_P2G_REDUCE = 3
OPT_P2G_BLOCK = 4
OPT_PASS_BLOCK = 5
OPT_GATHER = 6
OPT_GRAPH = 7
OPT_REORDER = 8
OPT_CELL_SORT = 9
OPT_PASS1_CORNERS = 10
OPT_PASS1_BLOCK = 11
OPT_LARGE_STRAIN = 12
OPT_FP64_FALLBACK = 13
OPT_SURROGATE_GUARD = 14


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load libmpm_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: build it with `python -m code_mpm_gb300.build`")
        L = C.CDLL(_LIB_PATH)
        vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        sig = {
            "mpm_create": ([C.POINTER(GridDesc), C.c_int, C.POINTER(vp)], C.c_int),
            "mpm_create_batch": ([C.POINTER(GridDesc), i32, C.c_int, C.POINTER(vp)], C.c_int),
            "mpm_batch_info": ([vp, C.POINTER(i64), C.POINTER(i32)], C.c_int),
            "mpm_destroy": ([vp], None),
            "mpm_last_error": ([vp], C.c_char_p),
            "mpm_device_info": ([C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
                                C.c_int),
            "mpm_set_stream": ([vp, vp], C.c_int),
            "mpm_set_option": ([vp, C.c_int, dbl], C.c_int),
            "mpm_upload_materials": ([vp, C.POINTER(Material), i32], C.c_int),
            "mpm_upload_particles": ([vp, C.POINTER(Particles), i64], C.c_int),
            "mpm_upload_dc_list": ([vp, vp, i64], C.c_int),
            "mpm_upload_nodes": ([vp, C.POINTER(Nodes)], C.c_int),
            "mpm_set_timeline": ([vp, vp, vp, i32], C.c_int),
            "mpm_set_sim": ([vp, C.POINTER(Sim)], C.c_int),
            "mpm_get_sim": ([vp, C.POINTER(Sim)], C.c_int),
            "mpm_download_particles": ([vp, C.POINTER(Particles)], C.c_int),
            "mpm_download_nodes": ([vp, C.POINTER(Nodes)], C.c_int),
            "mpm_advance": ([vp, i32, dbl, C.c_int], C.c_int),
            "mpm_run": ([vp, dbl, C.c_int, C.POINTER(C.c_int)], C.c_int),
            "mpm_synchronize": ([vp], C.c_int),
            "mpm_advance_timed": ([vp, i32, dbl, C.c_int, C.POINTER(C.c_float)], C.c_int),
            "mpm_profile_read": ([vp, C.POINTER(KernelStat), i32, C.POINTER(i32)], C.c_int),
            "mpm_profile_reset": ([vp], C.c_int),
            "mpm_launch_count": ([vp, C.POINTER(i64)], C.c_int),
            "mpm_cell_order": ([vp, vp, vp, i64], C.c_int),
            "mpm_cell_order_noalloc": ([C.POINTER(GridDesc), vp, i64, vp, vp, vp], C.c_int),
            "mpm_autotune": ([vp, i32, dbl, C.c_int, C.POINTER(TuneResult)], C.c_int),
            "mpm_upload_monitor_mask": ([vp, vp, i64], C.c_int),
            "mpm_monitors_read": ([vp, C.POINTER(Monitors)], C.c_int),
            "mpm_net_create": ([C.POINTER(NetConfig), C.POINTER(vp)], C.c_int),
            "mpm_net_destroy": ([vp], None),
            "mpm_net_train": ([vp, C.POINTER(NetReport)], C.c_int),
            "mpm_net_param_count": ([], i64),
            "mpm_net_get_params": ([vp, vp, i64], C.c_int),
            "mpm_net_set_params": ([vp, vp, i64], C.c_int),
            "mpm_net_loss_grad": ([vp, vp, vp, i64, vp, C.POINTER(dbl)], C.c_int),
            "mpm_net_infer": ([vp, vp, vp, i64, C.c_int, vp], C.c_int),
            "mpm_net_scales": ([vp, vp, vp, vp], C.c_int),
            "mpm_attach_surrogate": ([vp, vp, dbl, dbl], C.c_int),
            "mpm_surrogate_stats_read": ([vp, C.POINTER(SurrogateStats), C.c_int], C.c_int),
            "mpm_net_train_rows": ([vp, vp, i64, C.POINTER(NetReport)], C.c_int),
            "mpm_harvest_begin": ([vp, vp, i64, C.c_uint32, dbl], C.c_int),
            "mpm_harvest_end": ([vp, C.POINTER(i64)], C.c_int),
            "mpm_scene_honeycomb": ([C.POINTER(HoneycombDesc), vp, vp, C.c_uint64, C.POINTER(C.c_uint64), vp],
                                    C.c_int),
            "mpm_scene_graded_foam": ([C.POINTER(FoamDesc), vp, vp, C.c_uint64, C.POINTER(C.c_uint64), vp],
                                      C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def device_info() -> Dict[str, object]:
    name = C.create_string_buffer(256)
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    rc = lib().mpm_device_info(name, 256, C.byref(sm), C.byref(ma), C.byref(mi))
    if rc != 0:
        raise MPMError(rc, "no CUDA device")
    return {"name": name.value.decode(), "sm_count": sm.value, "cc": (ma.value, mi.value)}


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


NOALLOC_MAX_PARTICLES = 1 << 20


def cell_order_noalloc(length, cells, d_pos: int, n: int, d_keys: int, d_order: int, stream: int = 0) -> int:
    """mpm_cell_order_noalloc on caller-owned device buffers (addresses as ints); returns the status code.

    For callers that cannot allocate device memory: the library works in a
    fixed static scratch array and allocates nothing.  Calls share that
    scratch, so calls that overlap on the GPU race; at most
    NOALLOC_MAX_PARTICLES particles (larger n returns -6).
    """
    g = GridDesc()
    for a in range(3):
        g.length[a] = float(length[a])
        g.cells[a] = int(cells[a])
    return int(lib().mpm_cell_order_noalloc(C.byref(g), C.c_void_p(d_pos), int(n), C.c_void_p(d_keys),
                                            C.c_void_p(d_order), C.c_void_p(stream or None)))


class Engine:
    """One GPU engine instance (an ``mpm_ctx``)."""

    def __init__(self, length, cells, form: int = FORM_FP64, grids=None):
        """One grid (length, cells), or a batch of specimen grids [(length, cells), ...]."""
        self._L = lib()
        if grids is None:
            grids = [(length, cells)]
        tab = (GridDesc * len(grids))()
        for i, (ln, cl) in enumerate(grids):
            for a in range(3):
                tab[i].length[a] = float(ln[a])
                tab[i].cells[a] = int(cl[a])
        h = C.c_void_p()
        rc = self._L.mpm_create_batch(tab, len(grids), int(form), C.byref(h))
        if rc != 0 or not h.value:
            raise MPMError(rc, "mpm_create failed (no usable CUDA device or bad grid)")
        self._h = h
        self.form = int(form)
        self.length = np.asarray(grids[0][0], dtype=np.float64)
        self.cells = np.asarray(grids[0][1], dtype=np.int32)
        self.n_spec = len(grids)
        self.n_particles = 0
        self.n_nodes = int(sum(np.prod(np.asarray(cl, dtype=np.int64) + 1) for _, cl in grids))
        self._keep = []

    @classmethod
    def from_batch(cls, states, form: int = FORM_FP64, time_end: float = 1.0e300):
        """An engine advancing every specimen of `states` together (see code_mpm_gb300.batch)."""
        from . import batch

        pk = batch.pack(states)
        e = cls(None, None, form, grids=pk.grids)
        e.upload_state(pk.state, time_end=time_end)
        e.packed = pk
        return e

    def download_batch(self, states):
        """Per-specimen states after the batch has advanced."""
        from . import batch

        full = self.download_state(self.packed.state)
        return batch.unpack(full, states, self.packed.particle_offsets, self.packed.node_offsets)

    # -- plumbing -------------------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = self._L.mpm_last_error(self._h)
            raise MPMError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.mpm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self) -> int:
        return self._h.value

    def set_option(self, key: int, value: float) -> None:
        self._check(self._L.mpm_set_option(self._h, int(key), float(value)))

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self._L.mpm_set_stream(self._h, C.c_void_p(stream_ptr)))

    # -- state ------------------------------------------------------------------------
    @classmethod
    def from_state(cls, st: State, form: int = FORM_FP64, time_end: float = 1.0e300) -> "Engine":
        e = cls(st.length, st.cells, form)
        e.upload_state(st, time_end=time_end)
        return e

    def upload_state(self, st: State, time_end: float = 1.0e300) -> None:
        mats = st["materials"]
        tab = (Material * max(1, len(mats)))()
        for i, m in enumerate(mats):
            tab[i].type = int(m["type"])
            tab[i].density, tab[i].E, tab[i].nu = float(m["density"]), float(m["E"]), float(m["nu"])
            tab[i].yield_, tab[i].C0, tab[i].C1 = float(m["yield_"]), float(m["C0"]), float(m["C1"])
        self._check(self._L.mpm_upload_materials(self._h, tab, len(mats)))
        arrs = {k: np.ascontiguousarray(st[k]) for k in _PFIELDS}
        arrs["material"] = np.ascontiguousarray(st["material"], dtype=np.int32)
        arrs["pflags"] = np.ascontiguousarray(st["pflags"], dtype=np.uint8)
        arrs["dc_mult"] = np.ascontiguousarray(st["dc_mult"], dtype=np.float32)
        if "specimen" in st.arrays:
            arrs["specimen"] = np.ascontiguousarray(st["specimen"], dtype=np.int32)
        if "F_elastic" in st.arrays:
            arrs["F_elastic"] = np.ascontiguousarray(st["F_elastic"], dtype=np.float64)
        p = Particles(**{k: _ptr(v) for k, v in arrs.items()})
        self._check(self._L.mpm_upload_particles(self._h, C.byref(p), st.n_particles))
        self.n_particles = st.n_particles
        dcl = np.ascontiguousarray(st["dc_list"], dtype=np.uint32)
        self._check(self._L.mpm_upload_dc_list(self._h, _ptr(dcl), len(dcl)))
        # empty node arrays (a State holding only boundary conditions) stay unset: zero on the device
        narr = {k: np.ascontiguousarray(st[src]) for k, src in _NMAP if len(st[src]) > 0}
        nd = Nodes(**{k: _ptr(v) for k, v in narr.items()})
        self._check(self._L.mpm_upload_nodes(self._h, C.byref(nd)))
        t = np.ascontiguousarray(st["tl_time"], dtype=np.float64)
        v = np.ascontiguousarray(st["tl_vel"], dtype=np.float64)
        self._check(self._L.mpm_set_timeline(self._h, _ptr(t), _ptr(v), len(t)))
        self.set_sim(time=st.time, dt_max=st.dt_max, mass_min=st.mass_min, damping=st.damping, step=st.step,
                     time_end=time_end)

    def download_state(self, template: State) -> State:
        """A copy of ``template`` with every particle and node field replaced by the engine's."""
        st = template.copy()
        arrs = {k: st[k] for k in _PFIELDS}
        arrs["material"] = st["material"]
        arrs["pflags"] = st["pflags"]
        arrs["dc_mult"] = st["dc_mult"]
        if "F_elastic" not in st.arrays:
            st.arrays["F_elastic"] = np.zeros((st.n_particles, 9))
        arrs["F_elastic"] = st["F_elastic"]
        p = Particles(**{k: _ptr(v) for k, v in arrs.items()})
        self._check(self._L.mpm_download_particles(self._h, C.byref(p)))
        nd = Nodes(**{k: _ptr(st[src]) for k, src in _NMAP if len(st[src]) > 0})
        self._check(self._L.mpm_download_nodes(self._h, C.byref(nd)))
        s = self.get_sim()
        st.time, st.step = s["time"], s["step"]
        return st

    def download_particles(self, fields: Dict[str, np.ndarray]) -> None:
        """Fill the given preallocated host arrays (names as in State) from the device."""
        p = Particles(**{k: _ptr(v) for k, v in fields.items()})
        self._check(self._L.mpm_download_particles(self._h, C.byref(p)))

    def upload_particles(self, fields: Dict[str, np.ndarray], n: int) -> None:
        p = Particles(**{k: _ptr(v) for k, v in fields.items()})
        self._check(self._L.mpm_upload_particles(self._h, C.byref(p), int(n)))

    def set_sim(self, time: float, dt_max: float, mass_min: float = 0.0, damping: float = 0.0, step: int = 0,
                time_end: float = 1.0e300) -> None:
        s = Sim(float(time), float(dt_max), float(mass_min), float(damping), float(time_end), int(step))
        self._check(self._L.mpm_set_sim(self._h, C.byref(s)))

    def batch_info(self) -> np.ndarray:
        """First node of each specimen, then the total node count."""
        offs = (C.c_int64 * (self.n_spec + 1))()
        ns = C.c_int32(0)
        self._check(self._L.mpm_batch_info(self._h, offs, C.byref(ns)))
        return np.array(list(offs), dtype=np.int64)

    def get_sim(self) -> Dict[str, float]:
        s = Sim()
        self._check(self._L.mpm_get_sim(self._h, C.byref(s)))
        return {"time": s.time, "dt_max": s.dt_max, "mass_min": s.mass_min, "damping": s.damping,
                "time_end": s.time_end, "step": s.step}

    # -- stepping ----------------------------------------------------------------------
    def advance(self, nsteps: int, dt: Optional[float] = None, contact: bool = False) -> None:
        if dt is None:
            dt = self.get_sim()["dt_max"]
        self._check(self._L.mpm_advance(self._h, int(nsteps), float(dt), 1 if contact else 0))

    def advance_timed(self, nsteps: int, dt: Optional[float] = None, contact: bool = False) -> float:
        if dt is None:
            dt = self.get_sim()["dt_max"]
        ms = C.c_float(0.0)
        self._check(self._L.mpm_advance_timed(self._h, int(nsteps), float(dt), 1 if contact else 0, C.byref(ms)))
        return float(ms.value)

    def synchronize(self) -> None:
        self._check(self._L.mpm_synchronize(self._h))

    def autotune(self, steps: int = 3, dt: Optional[float] = None, contact: bool = False) -> Dict[str, float]:
        """Pick the fastest launch configuration on the current state (which is restored afterwards)."""
        if dt is None:
            dt = self.get_sim()["dt_max"]
        r = TuneResult()
        self._check(self._L.mpm_autotune(self._h, int(steps), float(dt), 1 if contact else 0, C.byref(r)))
        return {"p2g_reduce": r.p2g_reduce, "p2g_block": r.p2g_block, "pass_block": r.pass_block,
                "gather_batch": r.gather_batch, "pass1_corners": r.pass1_corners, "pass1_block": r.pass1_block,
                "candidates": r.candidates, "best_ms_per_step": r.best_ms_per_step,
                "worst_ms_per_step": r.worst_ms_per_step}

    def runSimulation_Classic_DoublePass_MPLocks(self, dTimeIncrement_Total: float) -> int:
        done = C.c_int(0)
        self._check(self._L.mpm_run(self._h, float(dTimeIncrement_Total), 0, C.byref(done)))
        return int(done.value)

    def runSimulation_Classic_DoublePass_MPLocks_Contact(self, dTimeIncrement_Total: float) -> int:
        done = C.c_int(0)
        self._check(self._L.mpm_run(self._h, float(dTimeIncrement_Total), 1, C.byref(done)))
        return int(done.value)

    def getTime_Current(self) -> float:
        return self.get_sim()["time"]

    def getTime_End(self) -> float:
        return self.get_sim()["time_end"]

    def getTime_Increment(self) -> float:
        return self.get_sim()["dt_max"]

    def getCount_MaterialPoint(self) -> int:
        return self.n_particles

    def getCount_GridPoint(self) -> int:
        return self.n_nodes

    def upload_monitor_mask(self, mask: np.ndarray) -> None:
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        self._check(self._L.mpm_upload_monitor_mask(self._h, _ptr(m), len(m)))

    def monitors(self) -> Dict[str, object]:
        """The reportConsole quantities (PhysicsEngine.cpp:40-183), reduced on the GPU."""
        r = Monitors()
        self._check(self._L.mpm_monitors_read(self._h, C.byref(r)))
        return {"time": r.time, "position_mean": list(r.position_mean), "force_sum": list(r.force_sum),
                "momentum": list(r.momentum), "strain_p_max": r.strain_p_max, "stress_p_max": r.stress_p_max,
                "stress_mean": list(r.stress_mean), "strain_mean": list(r.strain_mean), "kinetic": r.kinetic,
                "strain_energy": r.strain_energy, "plastic_energy": r.plastic_energy, "count": list(r.count),
                "platen_work": r.platen_work, "friction_work": r.friction_work}

    def cell_order(self):
        """(cell key per particle, particle order sorted by key) of the last step."""
        keys = np.zeros(self.n_particles, dtype=np.uint32)
        perm = np.zeros(self.n_particles, dtype=np.uint32)
        self._check(self._L.mpm_cell_order(self._h, _ptr(keys), _ptr(perm), self.n_particles))
        return keys, perm

    # -- profiling ----------------------------------------------------------------------
    def profile(self) -> Dict[str, Dict[str, float]]:
        arr = (KernelStat * 128)()
        cnt = C.c_int32(0)
        self._check(self._L.mpm_profile_read(self._h, arr, 128, C.byref(cnt)))
        return {arr[i].name.decode(): {"launches": int(arr[i].launches), "ms": float(arr[i].total_ms)}
                for i in range(min(cnt.value, 128))}

    def profile_reset(self) -> None:
        self._check(self._L.mpm_profile_reset(self._h))

    def launch_count(self) -> int:
        c = C.c_int64(0)
        self._check(self._L.mpm_launch_count(self._h, C.byref(c)))
        return int(c.value)

    # -- return-map network ------------------------------------------------------------
    def attach_surrogate(self, net: Optional["Net"], band: float = 0.02, recheck: float = 0.01) -> None:
        """Let the network compute the return map of clearly plastic von Mises hardening particles (FP32 form)."""
        self._check(self._L.mpm_attach_surrogate(self._h, net.handle if net else None, float(band), float(recheck)))
        self._keep.append(net)

    def harvest_begin(self, d_rows: int, cap: int, mat_mask: int = 1, band: float = 0.02) -> None:
        """Record return-map inputs of clearly plastic particles into device rows (n x 13 floats) while stepping."""
        self._check(self._L.mpm_harvest_begin(self._h, C.c_void_p(d_rows), int(cap), int(mat_mask), float(band)))

    def harvest_end(self) -> int:
        r = C.c_int64(0)
        self._check(self._L.mpm_harvest_end(self._h, C.byref(r)))
        return int(r.value)

    def surrogate_stats(self, reset: bool = False) -> Dict[str, float]:
        r = SurrogateStats()
        self._check(self._L.mpm_surrogate_stats_read(self._h, C.byref(r), 1 if reset else 0))
        return {"queued": r.queued, "band": r.band, "rechecked": r.rechecked, "recheck_rms": r.recheck_rms,
                "recheck_max": r.recheck_max, "rejected": r.rejected}


INFER_TC, INFER_FP32, INFER_EXACT, INFER_EXACT_FP64 = 0, 1, 2, 3


class Net:
    """The learned von Mises hardening return map (include/mpm_surrogate.h)."""

    def __init__(self, E=200.0e9, nu=0.3, yield_=250.0e6, C0=2.0e-3, C1=1.0e12, n_samples=20_000_000,
                 batch=65536, epochs=20, lr=4.0e-3, stress_range=1.5, epbar_max=0.2, deps_sigma=2.0e-4, seed=7,
                 sampling=0):
        self._L = lib()
        self.cfg = NetConfig(float(E), float(nu), float(yield_), float(C0), float(C1), int(n_samples), int(batch),
                             int(epochs), float(lr), float(stress_range), float(epbar_max), float(deps_sigma),
                             int(seed), int(sampling), 0)
        h = C.c_void_p()
        rc = self._L.mpm_net_create(C.byref(self.cfg), C.byref(h))
        if rc != 0 or not h.value:
            raise MPMError(rc, "mpm_net_create failed")
        self._h = h
        self.report = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.mpm_net_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise MPMError(rc, "mpm_net call failed")

    def train(self) -> Dict[str, float]:
        r = NetReport()
        self._check(self._L.mpm_net_train(self._h, C.byref(r)))
        self.report = {k: getattr(r, k) for k, _ in NetReport._fields_ if k not in ("out_scale", "out_shift")}
        self.report["out_scale"] = list(r.out_scale)[:7]
        self.report["out_shift"] = list(r.out_shift)[:7]
        return self.report

    def train_rows(self, d_rows: int, n: int) -> Dict[str, float]:
        """Train on device input rows (n x 13 physical), labelled by the exact FP64 map."""
        r = NetReport()
        self._check(self._L.mpm_net_train_rows(self._h, C.c_void_p(d_rows), int(n), C.byref(r)))
        self.report = {k: getattr(r, k) for k, _ in NetReport._fields_ if k not in ("out_scale", "out_shift")}
        return self.report

    def params(self) -> np.ndarray:
        n = int(self._L.mpm_net_param_count())
        a = np.zeros(n, dtype=np.float32)
        self._check(self._L.mpm_net_get_params(self._h, _ptr(a), n))
        return a

    def set_params(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float32)
        self._check(self._L.mpm_net_set_params(self._h, _ptr(a), a.size))

    def loss_grad(self, x: np.ndarray, t: np.ndarray):
        """(loss, gradient) of the training kernels on normalised rows x (n x 16), t (n x 8)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(int(self._L.mpm_net_param_count()), dtype=np.float32)
        loss = C.c_double(0.0)
        self._check(self._L.mpm_net_loss_grad(self._h, _ptr(x), _ptr(t), x.shape[0], _ptr(g), C.byref(loss)))
        return loss.value, g

    def scales(self):
        i = (C.c_double * 13)()
        s = (C.c_double * 7)()
        h = (C.c_double * 7)()
        self._check(self._L.mpm_net_scales(self._h, i, s, h))
        return np.array(list(i)), np.array(list(s)), np.array(list(h))

    def infer_device(self, d_in: int, d_out: int, n: int, kernel: int = INFER_TC, stream: int = 0) -> None:
        """Inference on device rows (pointers): inputs n x 13, outputs n x 7, physical units."""
        self._check(self._L.mpm_net_infer(self._h, C.c_void_p(d_in), C.c_void_p(d_out), int(n), int(kernel),
                                          C.c_void_p(stream)))
