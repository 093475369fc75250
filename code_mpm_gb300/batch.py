"""Batches of independent specimens advanced together by one engine.

The reference runs one scene per PhysicsEngine.  A batch packs many scenes,
each with its own grid, into one context (mpm_create_batch): particles are
concatenated with a specimen id per particle, nodes are concatenated in
specimen order, material tables are concatenated (each specimen's indices
offset), and displacement-control lists are offset into the concatenated
particle numbering.  All specimens share one time step and one timeline; a
per-specimen platen speed goes in the particles' displacement-control
multiplier.
"""
from __future__ import annotations

import dataclasses
from typing import List, Sequence, Tuple

import numpy as np

from .snapshot import FIELDS, State


@dataclasses.dataclass
class Packed:
    grids: List[Tuple[np.ndarray, np.ndarray]]  # (length, cells) per specimen
    state: State                               # concatenated arrays (length/cells of specimen 0)
    particle_offsets: np.ndarray                # n_spec + 1
    node_offsets: np.ndarray                    # n_spec + 1


def pack(states: Sequence[State]) -> Packed:
    if not states:
        raise ValueError("empty batch")
    s0 = states[0]
    for st in states[1:]:
        if st.dt_max != s0.dt_max or st.time != s0.time:
            raise ValueError("a batch advances with one time step and one clock")
        if not (np.array_equal(st["tl_time"], s0["tl_time"]) and np.array_equal(st["tl_vel"], s0["tl_vel"])):
            raise ValueError("a batch shares one timeline (put per-specimen speeds in dc_mult)")
    poff = np.cumsum([0] + [st.n_particles for st in states]).astype(np.int64)
    noff = np.cumsum([0] + [st.n_nodes for st in states]).astype(np.int64)
    moff = np.cumsum([0] + [len(st["materials"]) for st in states]).astype(np.int64)
    arrays = {}
    for name, _dt, _comp, sel in FIELDS:
        if sel in ("p", "n", "m"):
            arrays[name] = np.concatenate([st[name] for st in states])
    arrays["material"] = np.concatenate([np.where(st["material"] >= 0, st["material"] + moff[i], -1)
                                         for i, st in enumerate(states)]).astype(np.int32)
    arrays["dc_list"] = np.concatenate([st["dc_list"].astype(np.int64) + poff[i]
                                        for i, st in enumerate(states)]).astype(np.uint32)
    arrays["tl_time"] = s0["tl_time"].copy()
    arrays["tl_vel"] = s0["tl_vel"].copy()
    arrays["specimen"] = np.concatenate([np.full(st.n_particles, i, dtype=np.int32)
                                         for i, st in enumerate(states)])
    packed = State(length=s0.length.copy(), cells=s0.cells.copy(), time=s0.time, dt_max=s0.dt_max,
                   mass_min=s0.mass_min, damping=s0.damping, step=s0.step, arrays=arrays)
    return Packed(grids=[(st.length.copy(), st.cells.copy()) for st in states], state=packed,
                  particle_offsets=poff, node_offsets=noff)


def unpack(packed_state: State, templates: Sequence[State], poff: np.ndarray, noff: np.ndarray) -> List[State]:
    """Split a downloaded batch state back into per-specimen states."""
    out = []
    for i, t in enumerate(templates):
        st = t.copy()
        for name, _dt, _comp, sel in FIELDS:
            if sel == "p" and name != "material":
                st[name] = packed_state[name][poff[i]:poff[i + 1]].copy()
            elif sel == "n":
                st[name] = packed_state[name][noff[i]:noff[i + 1]].copy()
        st.time, st.step = packed_state.time, packed_state.step
        out.append(st)
    return out
