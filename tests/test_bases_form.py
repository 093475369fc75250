"""The FP32 linear bases from the stored cell-local coordinate u (axis_bases_u, code_mpm_gb300/csrc/physics.cuh):
the reduced form the kernels use against the general per-offset form (r = u - o, N = 1 - |r| with 0 outside
[0, 1], gradient sign(r)/h where 1e-12 < |r| < 1 -- the FP32 image of calculateBases_Classic's shape functions),
in float32 on the CPU, value for value over u in [0, 1]: every float near 0, 1/2 and 1, and a seeded sample of
the rest (the kernels store u only in [0, 1])."""
import numpy as np

F = np.float32


def general(u, ih):
    N, G = [], []
    for o in (0, 1):
        r = (u - F(o)).astype(F)
        ar = np.abs(r)
        nv = (F(1) - ar).astype(F)
        nv = np.where((nv < 0) | (nv > 1), F(0), nv)
        s = np.sign(r).astype(F)
        N.append(nv)
        G.append(np.where((ar > F(1e-12)) & (ar < F(1.0 - 1e-12)), (s * ih).astype(F), F(0)))
    return N, G


def reduced(u, ih):
    a1 = np.abs((u - F(1)).astype(F))
    N = [(F(1) - u).astype(F), (F(1) - a1).astype(F)]
    G = [np.where((u > F(1e-12)) & (u < F(1)), ih, F(0)), np.where((a1 > F(1e-12)) & (a1 < F(1)), -ih, F(0))]
    return N, G


def _bits(lo, hi):
    return np.arange(lo, hi, dtype=np.uint32).view(F)


def test_reduced_bases_equal_the_general_form():
    one = int(np.array(1.0, F).view(np.uint32))
    half = int(np.array(0.5, F).view(np.uint32))
    rng = np.random.Generator(np.random.PCG64(11))
    u = np.concatenate([_bits(0, 1 << 22), _bits(half - (1 << 21), half + (1 << 21)), _bits(one - (1 << 22), one + 1),
                        rng.integers(0, one + 1, 1 << 23, dtype=np.uint32).view(F),
                        rng.random(1 << 22, dtype=F)])
    assert u.min() >= 0 and u.max() <= 1
    for ih in (F(4000.0), F(1000.0), F(1.0 / 3.0e-4)):
        Ng, Gg = general(u, ih)
        Nr, Gr = reduced(u, ih)
        for a, b in zip(Ng + Gg, Nr + Gr):
            assert np.array_equal(a.view(np.uint32), b.astype(F).view(np.uint32))
