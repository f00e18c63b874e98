"""The shared arithmetic of the step (spatial_cell_gb300/csrc/scmath.h) on the
host: Philox known answers, accuracy of the elementary functions against
double-precision libm, binary16 rounding against numpy, the draws'
distribution, and the exactness of the single-precision forms of the
reference's double-precision comparisons.  The same header is compiled into
the sm_103a step; tests/test_gpu_parity.py shows the device gives the same
bits."""
import ctypes

import numpy as np
import pytest

from oracle import engine

F = ctypes.POINTER(ctypes.c_float)


@pytest.fixture(scope="module")
def lib():
    L, _ = engine.load("port")
    L.scp_math_eval.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.scp_philox.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    L.scp_f2h.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.scp_draws.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32,
                            ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p]
    L.scp_compare_forms.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    return L


def _eval(lib, fn, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, np.float32)
    out = np.empty_like(x)
    lib.scp_math_eval(fn, x.ctypes.data, y.ctypes.data, out.ctypes.data, len(x))
    return out


def _ulps(got, ref):
    r32 = ref.astype(np.float32)
    spacing = np.abs(np.spacing(r32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref) / spacing


def test_philox_known_answers(lib):
    # Random123 known-answer vectors of philox4x32-10
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        c = np.array(ctr, np.uint32)
        out = np.zeros(4, np.uint32)
        lib.scp_philox(c.ctypes.data, key[0], key[1], out.ctypes.data)
        assert tuple(int(v) for v in out) == want


@pytest.mark.parametrize("fn,lo,hi,tol", [(0, -10, 10, 2.0), (1, -10, 10, 2.0), (2, -1, 1, 1.5),
                                          (3, 1e-7, 1, 2.0), (4, -80, 80, 1.0)])
def test_elementary_accuracy(lib, fn, lo, hi, tol):
    rng = np.random.default_rng(fn)
    x = rng.uniform(lo, hi, 400000).astype(np.float32)
    ref = [np.sin, np.cos, np.arccos, np.log, np.exp][fn](x.astype(np.float64))
    got = _eval(lib, fn, x)
    assert _ulps(got, ref).max() <= tol


def test_pow_accuracy_in_step_range(lib):
    rng = np.random.default_rng(7)
    x = rng.uniform(0.0, 1.0, 400000).astype(np.float32)
    got = _eval(lib, 5, x, np.full_like(x, 0.2))
    ref = np.power(x.astype(np.float64), np.float64(np.float32(0.2)))
    # exp(y * log(x)) carries log's relative error times |y log x| into the result
    assert _ulps(got[x > 1e-30], ref[x > 1e-30]).max() <= 3.0
    mid = x > 0.05
    assert _ulps(got[mid], ref[mid]).max() <= 2.0
    special = np.array([0.0, 1.0, np.inf], np.float32)
    assert list(_eval(lib, 5, special, np.full(3, 0.2, np.float32))) == [0.0, 1.0, np.inf]


def test_special_values(lib):
    assert np.isnan(_eval(lib, 0, [np.inf, np.nan])).all()
    assert _eval(lib, 2, [1.0])[0] == 0.0
    assert np.isnan(_eval(lib, 2, [1.0000001, -1.5])).all()
    assert np.signbit(_eval(lib, 0, [-0.0])[0])


def test_half_rounding_matches_numpy(lib):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(0, 1, 200000), rng.normal(0, 3e4, 20000), rng.normal(0, 1e-5, 20000),
                        [65504, 65519.99, 65520, -65520, 6.1e-5, 5.96e-8, 2.98e-8, 0.0, -0.0, np.inf]]).astype(np.float32)
    out = np.zeros(len(x), np.uint16)
    lib.scp_f2h(x.ctypes.data, out.ctypes.data, len(x))
    assert np.array_equal(out, x.astype(np.float16).view(np.uint16))
    nan = np.array([np.nan], np.float32)
    lib.scp_f2h(nan.ctypes.data, out.ctypes.data, 1)
    assert out[0] == 0x7FFF


def test_draw_distributions(lib):
    n = 200000
    u = np.zeros(n, np.float32)
    g = np.zeros(n, np.float32)
    lib.scp_draws(42, 0, 0, n, 3, 2, 0, u.ctypes.data)
    lib.scp_draws(42, 1, 0, n, 3, 0, 1, g.ctypes.data)
    assert 0.0 < u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.005 and abs(u.var() - 1 / 12) < 0.002
    assert abs(g.mean()) < 0.01 and abs(g.var() - 1.0) < 0.02
    # different ids / steps / draws give independent values
    u2 = np.zeros(n, np.float32)
    lib.scp_draws(42, 0, 0, n, 4, 2, 0, u2.ctypes.data)
    assert abs(np.corrcoef(u, u2)[0, 1]) < 0.01


def test_single_precision_forms_are_exact(lib):
    rng = np.random.default_rng(11)
    s = np.concatenate([rng.uniform(0, 6, 500000), [0.0, 1e-40, 2.0, 5.0, 2.5, 4.5]]).astype(np.float32)
    bound = (s.astype(np.float64) * 1.4)
    # distances scattered around the bound, including adversarial neighbours
    d = (bound * (1 + rng.normal(0, 3e-7, len(s)))).astype(np.float32)
    d2 = np.nextafter(bound.astype(np.float32), np.float32(np.inf))
    d3 = np.nextafter(bound.astype(np.float32), np.float32(0))
    bad = np.zeros(len(s), np.uint8)
    for dd in (d, d2, d3, bound.astype(np.float32)):
        lib.scp_compare_forms(0, np.ascontiguousarray(dd).ctypes.data, s.ctypes.data, bad.ctypes.data, len(s))
        assert not bad.any()
    x = np.concatenate([rng.uniform(-0.002, 0.002, 500000),
                        np.nextafter(np.float32(0.001), np.float32([0, 1])), [0.001, -0.001]]).astype(np.float32)
    bad = np.zeros(len(x), np.uint8)
    lib.scp_compare_forms(1, x.ctypes.data, x.ctypes.data, bad.ctypes.data, len(x))
    assert not bad.any()


def _forms_bad(lib, kind, a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    bad = np.zeros(len(a), np.uint8)
    lib.scp_compare_forms(kind, a.ctypes.data, b.ctypes.data, bad.ctypes.data, len(a))
    return bad


def test_collision_distance_single_precision_form(lib):
    """(float)((double)(rp + rt) + 0.8 * (double)rp) evaluated as a rounded
    float-float value equals the double expression bit for bit."""
    rng = np.random.default_rng(11)
    nice = np.arange(1, 1025, dtype=np.float32) / np.float32(64)     # radii on a fine grid, all pairs
    ga, gb = np.meshgrid(nice, nice)
    cases = [
        (ga.ravel(), gb.ravel()),
        (rng.uniform(0, 10, 1_000_000), rng.uniform(0, 10, 1_000_000)),
        (np.exp(rng.uniform(-80, 80, 300_000)), np.exp(rng.uniform(-80, 80, 300_000))),
        (rng.uniform(-5, 5, 200_000), rng.uniform(-5, 5, 200_000)),
        (np.array([0, -0.0, 1, np.inf, -np.inf, np.nan, 1e-45, 3e38, 1.0], np.float32),
         np.array([0, 0, -1, 1, 1, 1, 1e-45, 3e38, np.nan], np.float32)),
    ]
    for a, b in cases:
        a32 = a.astype(np.float32)
        # neighbours of each value too: nudges that move the sum across float midpoints
        for da in (0, 1, -1):
            aa = a32.view(np.uint32).astype(np.int64) + da
            aa = np.clip(aa, 0, 0xFFFFFFFF).astype(np.uint32).view(np.float32)
            assert not _forms_bad(lib, 2, aa, b).any()


def test_polar_attraction_single_precision_form(lib):
    rng = np.random.default_rng(12)
    edge = np.array([1e-6, 2.0, 0.0, -0.0, -1.0, np.inf, -np.inf, np.nan, 1e-45, 3e38], np.float32)
    around = np.concatenate([np.nextafter(edge, np.float32(np.inf)), np.nextafter(edge, np.float32(-np.inf)), edge])
    x = np.concatenate([around, rng.uniform(0, 3, 500_000), np.exp(rng.uniform(-20, 2, 300_000)),
                        rng.uniform(-1, 1, 10_000)]).astype(np.float32)
    assert not _forms_bad(lib, 3, x, x).any()


def test_brownian_scalings_single_precision_forms(lib):
    rng = np.random.default_rng(13)
    radii = np.concatenate([np.arange(1, 1025, dtype=np.float32) / np.float32(64), rng.uniform(0, 20, 400_000),
                            np.exp(rng.uniform(-60, 60, 200_000)),
                            np.array([2.5, 0, -1, np.inf, -np.inf, np.nan, 1e-45, 3e38], np.float32)]).astype(np.float32)
    radii = np.concatenate([radii, np.nextafter(radii, np.float32(np.inf)), np.nextafter(radii, np.float32(-np.inf))])
    for scale in (rng.uniform(0, 3, len(radii)), np.exp(rng.uniform(-60, 60, len(radii))),
                  np.full(len(radii), 0.05), np.full(len(radii), 0.7)):
        x = scale.astype(np.float32)
        assert not _forms_bad(lib, 4, x, radii).any()
        assert not _forms_bad(lib, 5, x, radii).any()
