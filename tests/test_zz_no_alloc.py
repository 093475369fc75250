"""The cell-order entry point that allocates nothing (mpm_cell_order_noalloc).

It serves callers that cannot allocate device memory when they need the
cell order (code inside a memory pool that owns the whole device heap,
plug-ins whose host framework forbids cudaMalloc on its thread, loops that
cannot afford an allocation).  Its result must equal what the allocating
path, mpm_cell_order(), reports for the same positions; for this integer
work the tolerance is zero (bit-exact), on two calls in a row because the
calls share one scratch array.

The file name sorts last so that a run that stops at the first failure has
run every other test first.
"""
import numpy as np
import pytest

from code_mpm_gb300 import engine, scenes

pytestmark = pytest.mark.gpu


def _reference_order(st):
    """The allocating path: an engine holding the state reports the cell order of its first step."""
    with engine.Engine.from_state(st) as e:
        e.advance(1, st.dt_max, False)
        return e.cell_order()


def _noalloc_order(torch, st):
    n = st.n_particles
    pos = torch.from_numpy(np.ascontiguousarray(st["pos"].T)).cuda()  # x[n], y[n], z[n]
    keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    order = torch.zeros(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = engine.cell_order_noalloc(st.length, st.cells, pos.data_ptr(), n, keys.data_ptr(), order.data_ptr(),
                                   stream)
    assert rc == 0
    torch.cuda.synchronize()
    return keys.cpu().numpy().view(np.uint32), order.cpu().numpy().view(np.uint32)


def test_noalloc_cell_order_matches_allocating_path_twice():
    torch = pytest.importorskip("torch")
    from code_mpm_gb300 import build

    build.build()
    first = scenes.mixed_small(seed=21)
    second = scenes.platen_block(size=(0.03, 0.03, 0.02), h=1.0e-3)  # ~150k particles, reuses the scratch
    for st in (first, second):
        want_keys, want_order = _reference_order(st)
        keys, order = _noalloc_order(torch, st)
        assert np.array_equal(keys, want_keys)
        assert np.array_equal(order, want_order)


def test_noalloc_cell_order_at_exactly_its_capacity():
    """n = MPM_NOALLOC_MAX_PARTICLES: the whole scratch layout is in use, the digit counts of the last tiles
    included; twice in a row, against the allocating path."""
    torch = pytest.importorskip("torch")
    st = scenes.bar(cells_len=128, cells_w=32)  # 128 x 32 x 32 cells at 8 particles per cell
    assert st.n_particles == engine.NOALLOC_MAX_PARTICLES
    want_keys, want_order = _reference_order(st)
    for _ in range(2):
        keys, order = _noalloc_order(torch, st)
        assert np.array_equal(keys, want_keys)
        assert np.array_equal(order, want_order)


def test_noalloc_rejects_more_than_its_capacity():
    torch = pytest.importorskip("torch")
    st = scenes.mixed_small(seed=22)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = engine.cell_order_noalloc(st.length, st.cells, buf.data_ptr(), engine.NOALLOC_MAX_PARTICLES + 1,
                                   buf.data_ptr(), buf.data_ptr(), 0)
    assert rc == -6
