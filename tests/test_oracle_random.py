"""CLCG random numbers of the oracle (src/auxilliary/test_random.hh:27-110)."""
import numpy as np
from math import erf, log, sqrt

import oracle as O


def _clcg_python(n):
    """Independent restatement of L'Ecuyer's combined LCG (CACM 31(6), 1988)
    with the reference's parameters and seeds (parallel_random.cc:35-71)."""
    a1, m1, a2, m2 = 40014, 2147483563, 40692, 2147483399
    y1 = y2 = 1
    out = []
    for _ in range(n):
        x = y1 - y2
        if x < 1:
            x += m1 - 1
        y1 = (a1 * y1) % m1
        y2 = (a2 * y2) % m2
        out.append(x)
    return np.array(out, dtype=np.int64)


def test_integer_stream_matches_independent_restatement():
    assert np.array_equal(O.CLCG().draw_int(1000).astype(np.int64), _clcg_python(1000))


def test_parallel_leapfrog_equals_serial():
    # TestParallelConsistent: thread t of 4 draws elements t, t+4, ...
    n = 64
    seq = O.CLCG().draw_int(n)
    par = np.zeros(n, np.int32)
    for t in range(4):
        par[t::4] = O.CLCG(4, t).draw_int(len(range(t, n, 4)))
    assert np.array_equal(seq, par)


def test_uniform_cdf():
    n, nbins = 1 << 24, 32
    u = O.CLCG().draw_uniform(n)
    assert u.min() > 0.0 and u.max() < 1.0
    x = 1.1 + u * (3.4 - 1.1)
    idx = np.maximum(np.floor((x - 1.1) / (3.4 - 1.1) * nbins).astype(int), 0)
    cdf = np.cumsum(np.bincount(idx, minlength=nbins)[:nbins] / n)
    assert np.max(np.abs(cdf - (np.arange(nbins) + 1) / nbins)) < 2e-4


def test_normal_cdf():
    n, nbins = 1 << 24, 64
    z = O.CLCG().draw_normal(n)
    idx = np.maximum(np.floor((z + 10.0) / 20.0 * nbins).astype(int), 0)
    cdf = np.cumsum(np.bincount(idx, minlength=nbins)[:nbins] / n)
    xs = -10.0 + (np.arange(nbins) + 1) / nbins * 20.0
    true = np.array([0.5 * (1 + erf(x / sqrt(2.0))) for x in xs])
    assert np.max(np.abs(cdf - true)) < 2e-4


def test_polar_method_pairs():
    """draw_normal returns z_1 then the cached z_2 of one polar-method draw."""
    u = O.CLCG().draw_uniform(400)
    z = O.CLCG().draw_normal(100)
    k = 0
    for p in range(50):  # Marsaglia polar method with rejection
        while True:
            u1, u2 = 2.0 * u[k] - 1.0, 2.0 * u[k + 1] - 1.0
            k += 2
            s = u1 * u1 + u2 * u2
            if 0 < s < 1:
                break
        L = sqrt(-2 * log(s) / s)
        assert z[2 * p] == L * u1 and z[2 * p + 1] == L * u2


def _reference_rng():
    """The reference's own CLCGenerator, compiled from its sources by
    oracle/build_ref.py (present only where the reference sources are)."""
    import ctypes as C
    import os
    import pytest
    from oracle import build_ref
    path = build_ref.build()
    if path is None or not os.path.exists(path):
        pytest.skip("reference sources not available: reference RNG not built")
    L = C.CDLL(path)
    L.ref_clcg_create.restype = C.c_void_p
    L.ref_clcg_destroy.argtypes = [C.c_void_p]
    L.ref_clcg_draw_int.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]
    L.ref_clcg_draw_uniform.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]
    L.ref_clcg_draw_normal.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]
    L.ref_clcg_leapfrog_ints.argtypes = [C.c_int, C.c_int64, C.POINTER(C.c_int32)]
    L.ref_clcg_leapfrog_ints.restype = C.c_int
    return L, C


def test_oracle_rng_equals_reference_build():
    """Draw-by-draw equality with the reference's own generator: integers,
    uniforms and polar-method normals (bitwise), serial and leapfrog."""
    L, C = _reference_rng()
    n = 200000
    for kind, ctype, dtype in (("int", C.c_int32, np.int32), ("uniform", C.c_double, np.float64),
                               ("normal", C.c_double, np.float64)):
        h = L.ref_clcg_create()
        ref = np.zeros(n, dtype=dtype)
        getattr(L, f"ref_clcg_draw_{kind}")(h, n, ref.ctypes.data_as(C.POINTER(ctype)))
        L.ref_clcg_destroy(h)
        mine = getattr(O.CLCG(), f"draw_{kind}")(n)
        assert np.array_equal(np.asarray(mine), ref), kind
    nthreads, m = 4, 1000
    ref = np.zeros(nthreads * m, dtype=np.int32)
    got = L.ref_clcg_leapfrog_ints(nthreads, m, ref.ctypes.data_as(C.POINTER(C.c_int32)))
    for t in range(got):
        assert np.array_equal(O.CLCG(got, t).draw_int(m), ref[t * m:(t + 1) * m]), f"thread {t} of {got}"
