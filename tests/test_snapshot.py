import numpy as np

from code_mpm_gb300 import scenes, snapshot


def test_roundtrip(tmp_path):
    st = scenes.mixed_small(seed=5)
    p = tmp_path / "a.snap"
    snapshot.save(str(p), st)
    r = snapshot.load(str(p))
    assert r.n_particles == st.n_particles and r.n_nodes == st.n_nodes
    for k in st.arrays:
        assert np.array_equal(np.asarray(r[k]).view(np.uint8), np.asarray(st[k]).view(np.uint8)), k


def test_bar_matches_config_counts():
    st = scenes.bar()
    assert st.n_particles == 40000
    assert tuple(st.cells) == (52, 12, 12)
    # createDomain_Cuboid lattice: quarter points (spacing h/2)
    assert np.isclose(st["vol0"][0], (0.5e-3) ** 3)


def test_platen_block_count():
    st = scenes.platen_block(size=(0.01, 0.01, 0.005))
    body = (st["pflags"] & snapshot.PF_DC_SKIP) == 0
    assert body.sum() == 10 * 10 * 5 * 8
    assert len(st["dc_list"]) == (~body).sum()
