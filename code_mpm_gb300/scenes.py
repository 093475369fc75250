"""Synthetic scenes for the explicit-MPM hot path.

The reference builds its scenes in hard-coded ``initializeWorld_*`` methods
(e.g. PhysicsEngine_initializeWorld_Classic_Bar.cpp:4-256,
PhysicsEngine_initializeWorld_Classic_Cellular_Shim_Square.cpp:4-371); those
are scene preparation, not the solver path.  The generators here produce the
same kinds of state (regular grid, fixed node planes, materials, particle
lattices, a displacement-controlled platen and its timeline) directly as a
``State``.  Particle lattices follow
``MaterialPoint_Factory_Classic_CC::createDomain_Cuboid``
(MaterialPoint_Factory_Classic_createDomain_Cuboid.cpp:4-57): quarter-point
spacing, mirrored octants, offsets accumulated by repeated addition.
"""
from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .snapshot import (ELASTIC, NF_FIX_X, NF_FIX_Y, NF_FIX_Z, PF_DC_SKIP, PF_DC_X, PF_DC_Y, PF_DC_Z,
                       PF_SURFACE, PLASTIC, VONMISESHARDENING, State, empty_state)


def _axis_offsets(start: float, half: float, step: float) -> List[float]:
    out = []
    d = start
    while d <= half:
        out.append(d)
        d += step
    return out


def cuboid_lattice(center: Sequence[float], dim: Sequence[float], offset: float) -> np.ndarray:
    """Particle positions of createDomain_Cuboid (…createDomain_Cuboid.cpp:4-57), in its order."""
    single = dim[2] <= offset
    xs = _axis_offsets(0.5 * offset, 0.5 * dim[0], offset)
    ys = _axis_offsets(0.5 * offset, 0.5 * dim[1], offset)
    zs = _axis_offsets(0.0 if single else 0.5 * offset, 0.5 * dim[2], offset)
    signs = [(1, 1, 1), (-1, 1, 1), (-1, -1, 1), (1, -1, 1)]
    if not single:
        signs += [(1, 1, -1), (-1, 1, -1), (-1, -1, -1), (1, -1, -1)]
    X, Y, Z = np.meshgrid(np.array(xs), np.array(ys), np.array(zs), indexing="ij")
    base = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)  # dx outer, dz inner
    sg = np.array(signs, dtype=np.float64)  # (m, 3)
    pts = center[None, None, :] + base[:, None, :] * sg[None, :, :]
    return pts.reshape(-1, 3)


def block_lattice(lo: Sequence[float], hi: Sequence[float], h: float, ppc: int = 2) -> np.ndarray:
    """ppc^3 particles per cell at the cell's regular sub-cell centres, cell-major order (x fastest)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    n = np.rint((hi - lo) / h).astype(np.int64)
    sub = (np.arange(ppc) + 0.5) / ppc
    ci = [np.arange(k) for k in n]
    # cell-major: for cz, cy, cx, then sub-cell (sz, sy, sx)
    cz, cy, cx, sz, sy, sx = np.meshgrid(ci[2], ci[1], ci[0], sub, sub, sub, indexing="ij")
    x = lo[0] + (cx + sx) * h
    y = lo[1] + (cy + sy) * h
    z = lo[2] + (cz + sz) * h
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def node_positions(st: State) -> np.ndarray:
    """Node coordinates as GridPoint_Factory::createGrid computes them: (i*L)/n (GridPoint_Factory.h:53-55)."""
    nn = st.node_counts
    ax = [np.arange(nn[a], dtype=np.float64) * st.length[a] / st.cells[a] for a in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")  # x fastest: index = ix + iy*nx + iz*nx*ny
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def _material(st: State, i: int, type_: int, density: float, E: float, nu: float,
              yield_: float = 0.0, C0: float = 0.0, C1: float = 0.0) -> None:
    m = st["materials"]
    m[i]["type"] = type_
    m[i]["density"] = density
    m[i]["E"] = E
    m[i]["nu"] = nu
    m[i]["yield_"] = yield_
    m[i]["C0"] = C0
    m[i]["C1"] = C1


def _finish_particles(st: State, pos: np.ndarray, volume: float, mat_of: np.ndarray) -> None:
    n = pos.shape[0]
    st["pos"][:] = pos
    st["vol0"][:] = volume
    st["vol"][:] = volume
    st["material"][:] = mat_of
    dens = st["materials"]["density"][mat_of]
    st["mass"][:] = dens * volume
    assert st["pos"].shape == (n, 3)


def _alloc(length, cells, n, dt, nm, nt, nd) -> State:
    return empty_state(length, cells, n, dt, n_materials=nm, n_timeline=nt, n_dc=nd)


# ---------------------------------------------------------------------------
# Elastic bar (classic fixed-free vibrating bar)
# ---------------------------------------------------------------------------
def bar(cells_len: int = 50, cells_w: int = 10, h: float = 1.0e-3, E: float = 70.0e9, nu: float = 0.3,
        rho: float = 2700.0, v0: float = 1.0, seed: int = 0, jitter: float = 1.0e-6) -> State:
    """Elastic cuboid bar, fixed at one end, first-mode velocity v_x = v0 sin(pi x / 2L).

    The bar (cells_len x cells_w x cells_w cells) sits one cell in from the
    grid origin, with one padding cell on every side; the node plane at the
    bar's end x = h is fixed in x.  Particles: createDomain_Cuboid lattice at
    spacing h/2 (eight per cell), jittered by +-jitter*h.
    """
    L, W = cells_len * h, cells_w * h
    cells = np.array([cells_len + 2, cells_w + 2, cells_w + 2], dtype=np.int32)
    length = cells * h
    offset = 0.5 * h
    center = np.array([h + 0.5 * L, h + 0.5 * W, h + 0.5 * W])
    pos = cuboid_lattice(center, np.array([L, W, W]), offset)
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = pos + rng.uniform(-jitter * h, jitter * h, size=pos.shape)
    dt = 0.2 * h / math.sqrt(E / rho)
    st = _alloc(length, cells, pos.shape[0], dt, 1, 0, 0)
    _material(st, 0, ELASTIC, rho, E, nu)
    _finish_particles(st, pos, offset * offset * offset, np.zeros(pos.shape[0], dtype=np.int32))
    st["vel"][:, 0] = v0 * np.sin(math.pi * (pos[:, 0] - h) / (2.0 * L))
    xn = node_positions(st)
    st["fixed"][np.abs(xn[:, 0] - h) < 0.5 * h] |= NF_FIX_X
    return st


# ---------------------------------------------------------------------------
# J2 block compressed by a rigid platen (contact path)
# ---------------------------------------------------------------------------
def platen_block(size=(0.08, 0.08, 0.04), h: float = 1.0e-3, ppc: int = 2, E: float = 200.0e9,
                 nu: float = 0.3, rho: float = 7850.0, yield_: float = 250.0e6, H: float = 2.0e9,
                 C1: float = 1.0e12, speed: float = 5.0, friction: float = 0.1, pad: int = 2,
                 headroom: int = 4, surface: bool = True) -> State:
    """J2 block on a fixed floor, crushed in -z by a displacement-controlled platen.

    Linear hardening modulus H is mapped onto the reference's saturating law
    dR = C0 (sqrt(2/3) C1 - R) de_p (…VonMisesHardening.cpp:87-90) with a
    large C1 and C0 = H / C1, so the initial slope d(sigma_eq)/d(e_p) equals
    C0*C1 = H.  The platen is one layer of particles one cell above the
    block, flagged displacement-controlled on all axes and skipped by G2P
    (b_DisplacementControl), multiplier -1 on a +speed timeline.  The floor
    nodes (z = pad*h) are fixed in z and carry Coulomb friction `friction`
    on their x/y tangents.
    """
    size = np.asarray(size, dtype=np.float64)
    nb = np.rint(size / h).astype(np.int64)
    cells = np.array([nb[0] + 2 * pad, nb[1] + 2 * pad, nb[2] + pad + headroom], dtype=np.int32)
    length = cells * h
    lo = np.array([pad * h, pad * h, pad * h])
    hi = lo + nb * h
    body = block_lattice(lo, hi, h, ppc)
    off = h / ppc
    ztop = hi[2] + 0.5 * h
    plo = np.array([lo[0] - h, lo[1] - h, ztop])
    phi = np.array([hi[0] + h, hi[1] + h, ztop + h])
    platen = block_lattice(plo, phi, h, ppc)
    platen = platen[platen[:, 2] < ztop + off]  # one particle layer
    pos = np.concatenate([body, platen], axis=0)
    nbody = body.shape[0]
    dt = 0.2 * h / math.sqrt(E / rho)
    st = _alloc(length, cells, pos.shape[0], dt, 2, 2, platen.shape[0])
    _material(st, 0, VONMISESHARDENING, rho, E, nu, yield_, H / C1, C1)
    _material(st, 1, ELASTIC, rho, E, nu)
    mat = np.zeros(pos.shape[0], dtype=np.int32)
    mat[nbody:] = 1
    _finish_particles(st, pos, off * off * off, mat)
    st["pflags"][nbody:] = PF_DC_X | PF_DC_Y | PF_DC_Z | PF_DC_SKIP | PF_SURFACE
    st["dc_mult"][nbody:] = -1.0
    st["vel"][nbody:, 2] = -speed
    st["dc_list"][:] = np.arange(nbody, pos.shape[0], dtype=np.uint32)
    if surface:
        eps = 0.51 * off
        b = body
        on = ((b[:, 0] - lo[0] < eps) | (hi[0] - b[:, 0] < eps) | (b[:, 1] - lo[1] < eps) |
              (hi[1] - b[:, 1] < eps) | (b[:, 2] - lo[2] < eps) | (hi[2] - b[:, 2] < eps))
        st["pflags"][:nbody][on] |= PF_SURFACE
    st["tl_time"][:] = [0.0, 10.0]
    st["tl_vel"][:] = [[0.0, 0.0, speed], [0.0, 0.0, speed]]
    xn = node_positions(st)
    floor = np.abs(xn[:, 2] - lo[2]) < 0.5 * h
    st["fixed"][floor] |= NF_FIX_Z
    st["friction"][floor] = friction
    return st


# ---------------------------------------------------------------------------
# Small mixed scene exercising every branch of the non-contact step
# ---------------------------------------------------------------------------
def mixed_small(seed: int = 1, h: float = 1.0e-3, ncell=(8, 10, 6), vscale: float = 40.0) -> State:
    """A few thousand particles covering every branch of the double-pass step.

    Three materials (elastic, perfectly plastic, von Mises hardening), an
    x-fixed wall carrying friction (the reference's friction branch,
    …MPLocks.cpp:106-124), a y-fixed floor (reaction-force accumulation
    :125-131), a z-fixed plane, a platen controlled on a subset of axes with
    a multi-point timeline, random velocities large enough to yield, and a
    few particles that sit outside the grid on one side.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cells = np.array(ncell, dtype=np.int32)
    length = cells * h
    lo = np.array([1.0 * h, 1.0 * h, 1.0 * h])
    hi = np.array([(ncell[0] - 2) * h, (ncell[1] - 3) * h, (ncell[2] - 1) * h])
    body = block_lattice(lo, hi, h, 2)
    body = body + rng.uniform(-0.2 * h, 0.2 * h, size=body.shape)
    pl = block_lattice(np.array([lo[0], hi[1] + 0.5 * h, lo[2]]),
                       np.array([hi[0], hi[1] + 1.5 * h, hi[2]]), h, 2)
    pl = pl[pl[:, 1] < hi[1] + 1.0 * h]
    stray = np.array([[-0.3 * h, 2.0 * h, 2.0 * h], [length[0] + 0.2 * h, 3.0 * h, 2.5 * h],
                      [2.0 * h, -1.5 * h, 2.0 * h]])
    pos = np.concatenate([body, pl, stray], axis=0)
    n = pos.shape[0]
    nb, npl = body.shape[0], pl.shape[0]
    c = math.sqrt(70.0e9 / 2700.0)
    dt = 0.2 * h / c
    st = _alloc(length, cells, n, dt, 3, 4, npl)
    _material(st, 0, ELASTIC, 2700.0, 70.0e9, 0.3)
    _material(st, 1, PLASTIC, 7800.0, 210.0e9, 0.3, 310.0e6)
    _material(st, 2, VONMISESHARDENING, 2700.0, 70.0e9, 0.33, 70.0e6, 35.0, 55.0e6)
    mat = rng.integers(0, 3, size=n).astype(np.int32)
    mat[nb:nb + npl] = 0
    off = 0.5 * h
    _finish_particles(st, pos, off * off * off, mat)
    st["vel"][:nb] = rng.normal(0.0, vscale, size=(nb, 3))
    st["stress"][:nb] = rng.normal(0.0, 20.0e6, size=(nb, 6))
    st["backstress"][:nb] = rng.uniform(0.0, 5.0e6, size=nb)
    st["fext"][:nb] = rng.normal(0.0, 1.0e-3, size=(nb, 3))
    st["pflags"][nb:nb + npl] = PF_DC_Y | PF_DC_Z
    st["dc_mult"][nb:nb + npl] = -1.0
    st["dc_list"][:] = np.arange(nb, nb + npl, dtype=np.uint32)
    st["tl_time"][:] = [0.0, 5.0 * dt, 12.0 * dt, 1.0]
    st["tl_vel"][:] = [[0.0, 0.0, 0.0], [0.0, 8.0, 1.0], [0.0, 15.0, -2.0], [0.0, 15.0, -2.0]]
    xn = node_positions(st)
    wall = np.abs(xn[:, 0] - (ncell[0] - 1) * h) < 0.5 * h
    st["fixed"][wall] |= NF_FIX_X
    st["friction"][wall] = 0.3
    st["fixed"][np.abs(xn[:, 0]) < 0.5 * h] |= NF_FIX_X
    st["fixed"][np.abs(xn[:, 1] - 1.0 * h) < 0.5 * h] |= NF_FIX_Y
    st["fixed"][np.abs(xn[:, 2]) < 0.5 * h] |= NF_FIX_Z
    return st


# ---------------------------------------------------------------------------
# Body particles of the cellular scenes on the GPU (include/mpm_scene.h): the
# same lattice, order and surface flags as the numpy code below, bit for bit.
# ---------------------------------------------------------------------------
def _scene_call(fn, desc):
    import ctypes as C

    from . import engine

    n = C.c_uint64(0)
    rc = fn(C.byref(desc), None, None, 0, C.byref(n), None)
    if rc != 0:
        raise engine.MPMError(rc, "scene generation failed")
    pos = np.empty((n.value, 3), dtype=np.float64)
    surf = np.empty(n.value, dtype=np.uint8)
    rc = fn(C.byref(desc), pos.ctypes.data_as(C.c_void_p), surf.ctypes.data_as(C.c_void_p), n.value, C.byref(n),
            None)
    if rc != 0:
        raise engine.MPMError(rc, "scene generation failed")
    return pos, surf.astype(bool)


def honeycomb_body_gpu(wall: float, pitch: float, ncell: int, h: float, layers: int,
                       origin) -> Tuple[np.ndarray, np.ndarray]:
    """Body particles and surface flags of honeycomb() generated on the GPU (mpm_scene_honeycomb)."""
    from . import engine

    L = engine.lib()
    d = engine.HoneycombDesc()
    d.wall, d.pitch, d.h = float(wall), float(pitch), float(h)
    for a in range(3):
        d.origin[a] = float(origin[a])
    d.ncell, d.layers = int(ncell), int(layers)
    return _scene_call(L.mpm_scene_honeycomb, d)


def foam_body_gpu(pitch: float, t0: float, t1: float, h: float, height: float, x0: float, y0: float, z0: float,
                  ncell: int, width: int, layers: int, fx: np.ndarray,
                  fy: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Body particles and surface flags of graded_foam() generated on the GPU (mpm_scene_graded_foam)."""
    import ctypes as C

    from . import engine

    L = engine.lib()
    fx = np.ascontiguousarray(fx, dtype=np.float64)
    fy = np.ascontiguousarray(fy, dtype=np.float64)
    d = engine.FoamDesc()
    d.pitch, d.t0, d.t1, d.h, d.height = float(pitch), float(t0), float(t1), float(h), float(height)
    d.x0, d.y0, d.z0 = float(x0), float(y0), float(z0)
    d.ncell, d.width, d.layers = int(ncell), int(width), int(layers)
    d.fx, d.fy = fx.ctypes.data_as(C.c_void_p), fy.ctypes.data_as(C.c_void_p)
    return _scene_call(L.mpm_scene_graded_foam, d)


def honeycomb(wall: float, pitch: float, ncell: int, target: int, speed: float, h: float = 0.25e-3,
              E: float = 200.0e9, nu: float = 0.3, rho: float = 7850.0, yield_: float = 250.0e6,
              H: float = 2.0e9, C1: float = 1.0e12, friction: float = 0.1, pad: int = 2,
              headroom: int = 3, device: bool = False) -> State:
    """A square honeycomb crushed in-plane by a rigid platen (contact path).

    Cross-section in the x-z plane: ncell x ncell square cells of pitch
    `pitch` with walls `wall` thick, (ncell*pitch + wall) wide; extruded
    along y by as many particle layers as bring the count near `target`.
    Particles sit at the centres of an h/2 lattice (8 per grid cell) inside
    the walls; those with an empty lattice neighbour in x or z are surface
    particles.  A one-layer platen above the top moves down at `speed`
    (multiplier -speed on a unit timeline, so a batch can give each specimen
    its own speed); the floor nodes are fixed in z with Coulomb friction.
    device: the body particles are generated on the GPU (honeycomb_body_gpu), bit for bit the same.
    """
    s = 0.5 * h
    W = ncell * pitch + wall
    n1 = int(np.ceil(W / s))
    c = (np.arange(n1) + 0.5) * s
    per_layer = honeycomb_layer_count(wall, pitch, ncell, h)
    ny = max(2, int(round(target / max(per_layer, 1))))
    nbx = n1 // 2 + 1
    cells = np.array([nbx + 2 * pad, ny // 2 + 1 + 2 * pad, nbx + pad + headroom], dtype=np.int32)
    length = cells * h
    org = np.array([pad * h, pad * h, pad * h])
    if device:
        body, bsurf = honeycomb_body_gpu(wall, pitch, ncell, h, ny, org)
    else:
        inx = (np.mod(c, pitch) < wall) & (c < W)
        X, Z = np.meshgrid(c, c, indexing="ij")
        wall_xz = (inx[:, None] | inx[None, :]) & (X < W) & (Z < W)
        ix, iz = np.nonzero(wall_xz)
        # surface: a wall lattice site with an empty neighbour in x or z
        padm = np.pad(wall_xz, 1)
        surf2 = ~(padm[2:, 1:-1] & padm[:-2, 1:-1] & padm[1:-1, 2:] & padm[1:-1, :-2])[ix, iz]
        yy = (np.arange(ny) + 0.5) * s
        body = np.stack([np.repeat(org[0] + c[ix], ny), np.tile(org[1] + yy, len(ix)),
                         np.repeat(org[2] + c[iz], ny)], axis=1)
        bsurf = np.repeat(surf2, ny)
    ztop = org[2] + W + 0.5 * h
    px = org[0] + np.arange(-h + 0.5 * s, W + h, s)
    py = org[1] + np.arange(-h + 0.5 * s, ny * s + h, s)
    PX, PY = np.meshgrid(px, py, indexing="ij")
    platen = np.stack([PX.ravel(), PY.ravel(), np.full(PX.size, ztop)], axis=1)
    pos = np.concatenate([body, platen], axis=0)
    nbody = body.shape[0]
    dt = 0.2 * h / math.sqrt(E / rho)
    st = _alloc(length, cells, pos.shape[0], dt, 2, 2, platen.shape[0])
    _material(st, 0, VONMISESHARDENING, rho, E, nu, yield_, H / C1, C1)
    _material(st, 1, ELASTIC, rho, E, nu)
    mat = np.zeros(pos.shape[0], dtype=np.int32)
    mat[nbody:] = 1
    _finish_particles(st, pos, s * s * s, mat)
    st["pflags"][:nbody][bsurf] |= PF_SURFACE
    st["pflags"][nbody:] = PF_DC_X | PF_DC_Y | PF_DC_Z | PF_DC_SKIP | PF_SURFACE
    st["dc_mult"][nbody:] = -float(speed)
    st["vel"][nbody:, 2] = -float(speed)
    st["dc_list"][:] = np.arange(nbody, pos.shape[0], dtype=np.uint32)
    st["tl_time"][:] = [0.0, 10.0]
    st["tl_vel"][:] = [[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]]
    xn = node_positions(st)
    floor = np.abs(xn[:, 2] - org[2]) < 0.5 * h
    st["fixed"][floor] |= NF_FIX_Z
    st["friction"][floor] = friction
    return st


def honeycomb_batch(n: int = 256, seed: int = 4, total: float = 40.0e6, nmin: int = 10_000, nmax: int = 500_000,
                    h: float = 0.25e-3, device: bool = False):
    """The batched cellular workload: n honeycombs with walls U(0.4, 1.2) mm, pitch U(4, 8) mm,
    4-10 cells per side, particle counts log-uniform in [nmin, nmax] scaled so the batch holds
    about `total` particles, platen speed U(1, 10) m/s per specimen."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(nmin), np.log(nmax), n))
    counts = np.clip(counts * total / counts.sum(), nmin, nmax)
    speed = rng.uniform(1.0, 10.0, n)
    out = []
    for i in range(n):
        # A cross-section whose two thinnest extrusion layers already exceed the count cannot meet it: draw the
        # geometry again (the smallest one, 4 cells of 4 mm with 0.4 mm walls, holds about 6,600 particles).
        for _ in range(10_000):
            wall, pitch, ncell = rng.uniform(0.4e-3, 1.2e-3), rng.uniform(4.0e-3, 8.0e-3), int(rng.integers(4, 11))
            if 2 * honeycomb_layer_count(wall, pitch, ncell, h) <= counts[i]:
                break
        else:
            wall, pitch, ncell = 0.4e-3, 4.0e-3, 4
        out.append(honeycomb(wall, pitch, ncell, int(counts[i]), speed[i], h=h, device=device))
    return out


def honeycomb_layer_count(wall: float, pitch: float, ncell: int, h: float) -> int:
    """Particles in one y-layer of honeycomb()'s cross-section."""
    s = 0.5 * h
    W = ncell * pitch + wall
    c = (np.arange(int(np.ceil(W / s))) + 0.5) * s
    m = int((c < W).sum())
    k = int(((np.mod(c, pitch) < wall) & (c < W)).sum())
    return m * m - (m - k) * (m - k)


def graded_foam(ncell: int = 8, pitch: float = 5.0e-3, t0: float = 0.3e-3, t1: float = 1.0e-3,
                block=(0.2, 0.2, 0.1), h: float = 0.25e-3, perturb: float = 0.1, seed: int = 5,
                E: float = 70.0e9, nu: float = 0.33, rho: float = 2700.0, yield_: float = 120.0e6, H: float = 700.0e6,
                C1: float = 1.0e12, speed: float = 20.0, friction: float = 0.2, pad: int = 2, headroom: int = 4,
                height: Optional[float] = None, device: bool = False) -> State:
    """Density-graded square-cell foam crushed out of plane by a rigid platen (contact path).

    The grid covers the whole block (block / h cells, 800 x 800 x 400 by default) while the foam occupies
    ncell x ncell square cells of pitch `pitch` centred in x-y: walls are the planes x, y = x0 + k pitch (k = 0 ..
    ncell) extruded along z, their thickness growing linearly from t0 at the floor to t1 at the top, each wall's
    thickness scaled by 1 + U(-perturb, perturb) (seeded).  Particles sit at the centres of an h/2 lattice inside
    the walls (8 per cell); those with an empty lattice neighbour in x or y are surface particles.  A one-layer
    platen above the top moves down at `speed`; the floor node plane is fixed in z with Coulomb friction.  Grids
    above 50M nodes hold only the nodes' boundary conditions on the host (node_fields="bc").
    device: the body particles are generated on the GPU (foam_body_gpu), bit for bit the same.
    """
    cells = np.array([int(round(block[a] / h)) for a in range(3)], dtype=np.int32)
    length = cells * h
    s = 0.5 * h
    z0 = pad * h
    if height is None:
        height = length[2] - (pad + headroom) * h
    W = ncell * pitch + t1 * (1.0 + perturb)
    x0 = round(0.5 * (length[0] - W) / h) * h
    y0 = round(0.5 * (length[1] - W) / h) * h
    m = int(np.ceil(W / s))
    c = (np.arange(m) + 0.5) * s
    nz = int(round(height / s))
    rng = np.random.Generator(np.random.PCG64(seed))
    fx = 1.0 + rng.uniform(-perturb, perturb, ncell + 1)
    fy = 1.0 + rng.uniform(-perturb, perturb, ncell + 1)
    if device:
        body, bsurf = foam_body_gpu(pitch, t0, t1, h, height, x0, y0, z0, ncell, m, nz, fx, fy)
    else:
        kx = np.minimum((c // pitch).astype(np.int64), ncell)
        rel = c - kx * pitch
        layers, surf_layers = [], []
        for k in range(nz):
            zc = (k + 0.5) * s
            t = t0 + (t1 - t0) * zc / height
            inx = rel < t * fx[kx]
            iny = rel < t * fy[kx]
            wall = inx[:, None] | iny[None, :]
            ix, iy = np.nonzero(wall)
            padm = np.pad(wall, 1)
            surf = ~(padm[2:, 1:-1] & padm[:-2, 1:-1] & padm[1:-1, 2:] & padm[1:-1, :-2])[ix, iy]
            layers.append(np.stack([x0 + c[ix], y0 + c[iy], np.full(ix.size, z0 + zc)], axis=1))
            surf_layers.append(surf)
        body = np.concatenate(layers)
        bsurf = np.concatenate(surf_layers)
    ztop = z0 + height + 0.5 * h
    px = x0 + np.arange(-h + 0.5 * s, W + h, s)
    py = y0 + np.arange(-h + 0.5 * s, W + h, s)
    PX, PY = np.meshgrid(px, py, indexing="ij")
    platen = np.stack([PX.ravel(), PY.ravel(), np.full(PX.size, ztop)], axis=1)
    pos = np.concatenate([body, platen])
    nbody = body.shape[0]
    dt = 0.2 * h / math.sqrt(E / rho)
    n_nodes = int(np.prod(cells.astype(np.int64) + 1))
    st = empty_state(length, cells, pos.shape[0], dt, n_materials=2, n_timeline=2, n_dc=platen.shape[0],
                     node_fields="bc" if n_nodes > 50_000_000 else "all")
    _material(st, 0, VONMISESHARDENING, rho, E, nu, yield_, H / C1, C1)
    _material(st, 1, ELASTIC, rho, E, nu)
    mat = np.zeros(pos.shape[0], dtype=np.int32)
    mat[nbody:] = 1
    _finish_particles(st, pos, s * s * s, mat)
    st["pflags"][:nbody][bsurf] |= PF_SURFACE
    st["pflags"][nbody:] = PF_DC_X | PF_DC_Y | PF_DC_Z | PF_DC_SKIP | PF_SURFACE
    st["dc_mult"][nbody:] = -float(speed)
    st["vel"][nbody:, 2] = -float(speed)
    st["dc_list"][:] = np.arange(nbody, pos.shape[0], dtype=np.uint32)
    st["tl_time"][:] = [0.0, 10.0]
    st["tl_vel"][:] = [[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]]
    nn = cells + 1
    floor = pad * nn[0] * nn[1] + np.arange(nn[0] * nn[1], dtype=np.int64)  # node plane iz = pad
    st["fixed"][floor] |= NF_FIX_Z
    st["friction"][floor] = friction
    return st


def contact_small(seed: int = 2, h: float = 1.0e-3, nb=(6, 5, 4), speed: float = 30.0) -> State:
    """Small platen_block variant with jittered particles, for contact-path parity."""
    st = platen_block(size=(nb[0] * h, nb[1] * h, nb[2] * h), h=h, ppc=2, yield_=150.0e6, H=2.0e9,
                      speed=speed, friction=0.0, pad=2, headroom=3)
    rng = np.random.Generator(np.random.PCG64(seed))
    n = st.n_particles
    body = (st["pflags"] & PF_DC_SKIP) == 0
    st["pos"][body] += rng.uniform(-0.15 * h, 0.15 * h, size=(int(body.sum()), 3))
    st["vel"][body] = rng.normal(0.0, 5.0, size=(int(body.sum()), 3))
    assert st.n_particles == n
    return st
