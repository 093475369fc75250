"""Binary structure-of-arrays MPM state ("MPMSNAP1") and the in-memory State.

The reference keeps its state as heap objects (``MaterialPoint_BC``,
``GridPoint``, ``Material_BC``; MaterialPoint_BC.h:25-85, GridPoint.h:6-45,
Material_BC.h:13-35) and has no checkpoint format.  ``State`` holds the same
field set as flat numpy arrays (per-particle vectors n x k, row-major), which
is exactly what the C-ABI uploads and downloads.  ``save``/``load`` write the
little-endian layout that the oracle's C header ``oracle/mpm_snapshot.h``
reads, so a state can be handed between the reference, the CPU restatement
and the CUDA engine without loss (step-k exchange, resume).
"""
from __future__ import annotations

import dataclasses
import struct
from typing import Dict, Tuple

import numpy as np

MAGIC = b"MPMSNAP1"
HEADER_FMT = "<8sII3d3ii4dqQQIIII"
HEADER_SIZE = struct.calcsize(HEADER_FMT)
assert HEADER_SIZE == 128

# particle flag bits (MaterialPoint_BC.h:32-43)
PF_DC_X, PF_DC_Y, PF_DC_Z, PF_DC_SKIP, PF_SURFACE = 1, 2, 4, 8, 16
# node fixed bits (GridPoint.h:20) and node state bits (GridPoint.h:12-18)
NF_FIX_X, NF_FIX_Y, NF_FIX_Z = 1, 2, 4
NS_ACTIVE, NS_CONTACT, NS_POSITIVE, NS_NEGATIVE = 1, 2, 4, 8

# material type ids (Material_BC.h:6-11)
ELASTIC, PLASTIC, VONMISESHARDENING = 0, 3, 4

MATERIAL_DTYPE = np.dtype([("type", "<i4"), ("pad", "<i4"), ("density", "<f8"), ("E", "<f8"),
                           ("nu", "<f8"), ("yield_", "<f8"), ("C0", "<f8"), ("C1", "<f8")])

# (name, dtype, components, count): count 'p' particles, 'n' nodes, 'm' materials, 't' timeline, 'd' dc list.
FIELDS: Tuple[Tuple[str, str, int, str], ...] = (
    ("materials", "mat", 1, "m"),
    ("tl_time", "<f8", 1, "t"),
    ("tl_vel", "<f8", 3, "t"),
    ("pos", "<f8", 3, "p"),
    ("vel", "<f8", 3, "p"),
    ("fext", "<f8", 3, "p"),
    ("mass", "<f8", 1, "p"),
    ("vol", "<f8", 1, "p"),
    ("vol0", "<f8", 1, "p"),
    ("F", "<f8", 9, "p"),
    ("stress", "<f8", 6, "p"),
    ("strain", "<f8", 6, "p"),
    ("eps_p", "<f8", 6, "p"),
    ("e_strain", "<f8", 1, "p"),
    ("e_strain_max", "<f8", 1, "p"),
    ("e_strain_ti", "<f8", 1, "p"),
    ("e_plastic", "<f8", 1, "p"),
    ("backstress", "<f8", 1, "p"),
    ("mp_mass_gradient", "<f8", 3, "p"),
    ("strain_rate", "<f8", 6, "p"),
    ("material", "<i4", 1, "p"),
    ("pflags", "u1", 1, "p"),
    ("dc_mult", "<f4", 1, "p"),
    ("dc_list", "<u4", 1, "d"),
    ("fixed", "u1", 1, "n"),
    ("friction", "<f8", 1, "n"),
    ("g_mass", "<f8", 1, "n"),
    ("g_mom", "<f8", 3, "n"),
    ("g_vel", "<f8", 3, "n"),
    ("g_force", "<f8", 3, "n"),
    ("g_force_temp", "<f8", 3, "n"),
    ("g_mass_gradient", "<f8", 3, "n"),
    ("g_state", "u1", 1, "n"),
)

# Header flag: the elastic deformation gradient (MaterialPoint_BC.h:65, state of the large-strain pass 2)
# follows the fields as one more n x 9 array; without it, it is the identity.
HAS_FE = 1
FE_FIELD = "F_elastic"

PARTICLE_FIELDS = tuple(f[0] for f in FIELDS if f[3] == "p")
NODE_FIELDS = tuple(f[0] for f in FIELDS if f[3] == "n")


@dataclasses.dataclass
class State:
    """One MPM state: grid geometry, time, materials, timeline, particles, nodes."""

    length: np.ndarray  # (3,) grid extent [m]
    cells: np.ndarray  # (3,) int cells per axis; nodes = cells + 1
    time: float
    dt_max: float
    mass_min: float = 0.0
    damping: float = 0.0
    step: int = 0
    contact: int = 0
    arrays: Dict[str, np.ndarray] = dataclasses.field(default_factory=dict)

    # -- sizes ---------------------------------------------------------------
    @property
    def n_particles(self) -> int:
        return int(self.arrays["pos"].shape[0])

    @property
    def node_counts(self) -> np.ndarray:
        return np.asarray(self.cells, dtype=np.int64) + 1

    @property
    def n_nodes(self) -> int:
        return int(np.prod(self.node_counts))

    def __getitem__(self, k: str) -> np.ndarray:
        return self.arrays[k]

    def __setitem__(self, k: str, v: np.ndarray) -> None:
        self.arrays[k] = v

    def copy(self) -> "State":
        return dataclasses.replace(self, length=self.length.copy(), cells=self.cells.copy(),
                                   arrays={k: v.copy() for k, v in self.arrays.items()})

    def _count(self, sel: str) -> int:
        return {"p": self.n_particles, "n": self.n_nodes, "m": len(self.arrays["materials"]),
                "t": len(self.arrays["tl_time"]), "d": len(self.arrays["dc_list"])}[sel]


def empty_state(length, cells, n_particles: int, dt_max: float, n_materials: int = 1,
                n_timeline: int = 0, n_dc: int = 0, time: float = 0.0, node_fields: str = "all") -> State:
    """A State with every array allocated and zero-filled, F set to identity.  node_fields="bc" allocates only
    the nodes' boundary conditions (fixed, friction): the other node arrays are empty, an engine leaves those
    fields zero, and downloads skip them (for grids of hundreds of millions of nodes)."""
    st = State(length=np.asarray(length, dtype=np.float64), cells=np.asarray(cells, dtype=np.int32),
               time=float(time), dt_max=float(dt_max))
    counts = {"p": n_particles, "n": int(np.prod(np.asarray(cells, dtype=np.int64) + 1)),
              "m": n_materials, "t": n_timeline, "d": n_dc}
    for name, dt, comp, sel in FIELDS:
        n = counts[sel]
        if sel == "n" and node_fields == "bc" and name not in ("fixed", "friction"):
            n = 0
        if dt == "mat":
            st.arrays[name] = np.zeros(n, dtype=MATERIAL_DTYPE)
        else:
            shape = (n,) if comp == 1 else (n, comp)
            st.arrays[name] = np.zeros(shape, dtype=np.dtype(dt))
    st.arrays["F"][:, 0] = 1.0
    st.arrays["F"][:, 4] = 1.0
    st.arrays["F"][:, 8] = 1.0
    st.arrays["dc_mult"][:] = 1.0
    return st


def identity_f(n: int) -> np.ndarray:
    a = np.zeros((n, 9))
    a[:, 0] = a[:, 4] = a[:, 8] = 1.0
    return a


def save(path: str, st: State) -> None:
    nm, nt, nd = (len(st.arrays[k]) for k in ("materials", "tl_time", "dc_list"))
    fe = st.arrays.get(FE_FIELD)
    hdr = struct.pack(HEADER_FMT, MAGIC, 1, int(st.contact), *map(float, st.length),
                      *map(int, st.cells), 0, float(st.time), float(st.dt_max), float(st.mass_min),
                      float(st.damping), int(st.step), st.n_particles, st.n_nodes, nm, nt, nd,
                      HAS_FE if fe is not None else 0)
    with open(path, "wb") as f:
        f.write(hdr)
        for name, dt, comp, sel in FIELDS:
            a = st.arrays[name]
            want = MATERIAL_DTYPE if dt == "mat" else np.dtype(dt)
            n = st._count(sel)
            a = np.ascontiguousarray(a, dtype=want).reshape(-1)
            if a.size != n * comp:
                raise ValueError(f"field {name}: {a.size} elements, expected {n * comp}")
            f.write(a.tobytes())
        if fe is not None:
            a = np.ascontiguousarray(fe, dtype="<f8").reshape(-1)
            if a.size != st.n_particles * 9:
                raise ValueError(f"field {FE_FIELD}: {a.size} elements, expected {st.n_particles * 9}")
            f.write(a.tobytes())


def load(path: str) -> State:
    with open(path, "rb") as f:
        raw = f.read()
    vals = struct.unpack_from(HEADER_FMT, raw, 0)
    if vals[0] != MAGIC or vals[1] != 1:
        raise ValueError(f"{path}: not an MPMSNAP1 file")
    contact = vals[2]
    length = np.array(vals[3:6])
    cells = np.array(vals[6:9], dtype=np.int32)
    time, dt_max, mass_min, damping = vals[10:14]
    step, npart, nnodes, nm, nt, nd, flags = vals[14:21]
    st = State(length=length, cells=cells, time=time, dt_max=dt_max, mass_min=mass_min,
               damping=damping, step=step, contact=contact)
    counts = {"p": npart, "n": nnodes, "m": nm, "t": nt, "d": nd}
    off = HEADER_SIZE
    for name, dt, comp, sel in FIELDS:
        want = MATERIAL_DTYPE if dt == "mat" else np.dtype(dt)
        n = counts[sel] * comp
        a = np.frombuffer(raw, dtype=want, count=n, offset=off).copy()
        off += n * want.itemsize
        st.arrays[name] = a if comp == 1 else a.reshape(-1, comp)
    if flags & HAS_FE:
        n = npart * 9
        st.arrays[FE_FIELD] = np.frombuffer(raw, dtype="<f8", count=n, offset=off).copy().reshape(-1, 9)
        off += n * 8
    if off != len(raw):
        raise ValueError(f"{path}: {len(raw) - off} trailing bytes")
    return st
