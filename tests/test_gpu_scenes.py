"""The cellular scenes' body particles generated on the GPU (include/mpm_scene.h) against the numpy generator
of code_mpm_gb300/scenes.py: every array of the resulting State bit for bit (positions, order, surface flags),
for honeycombs over the batch's parameter range and for graded foams (the reduced one and a taller one whose
walls span several perturbed thicknesses).  The setup times are printed."""
import json
import time

import numpy as np
import pytest

from code_mpm_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from code_mpm_gb300 import build, engine

    build.build()
    engine.lib()


def _same(a, b):
    assert a.n_particles == b.n_particles and a.n_nodes == b.n_nodes
    for k in a.arrays:
        assert np.array_equal(a[k], b[k]), k


def test_honeycombs_match_host_generator():
    rng = np.random.Generator(np.random.PCG64(3))
    for _ in range(12):
        wall, pitch, ncell = rng.uniform(0.4e-3, 1.2e-3), rng.uniform(4.0e-3, 8.0e-3), int(rng.integers(4, 11))
        target = int(rng.uniform(2, 30) * scenes.honeycomb_layer_count(wall, pitch, ncell, 0.25e-3))
        speed = rng.uniform(1.0, 10.0)
        _same(scenes.honeycomb(wall, pitch, ncell, target, speed, device=True),
              scenes.honeycomb(wall, pitch, ncell, target, speed))


@pytest.mark.parametrize("kw", [dict(ncell=2, block=(0.02, 0.02, 0.012), seed=5),
                                dict(ncell=3, block=(0.03, 0.03, 0.03), seed=9, perturb=0.1)])
def test_graded_foams_match_host_generator(kw):
    _same(scenes.graded_foam(device=True, **kw), scenes.graded_foam(**kw))


def test_setup_time_of_the_batch():
    t0 = time.perf_counter()
    dev = scenes.honeycomb_batch(n=32, total=5.0e6, device=True)
    t1 = time.perf_counter()
    host = scenes.honeycomb_batch(n=32, total=5.0e6)
    t2 = time.perf_counter()
    for a, b in zip(dev, host):
        _same(a, b)
    print(json.dumps({"specimens": len(dev), "particles": int(sum(s.n_particles for s in dev)),
                      "seconds_gpu_body": t1 - t0, "seconds_host": t2 - t1}))
