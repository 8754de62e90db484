"""The guarded FP32 bin indices of the Dr16 histogram kernel
(picca_gb300/csrc/pg_continuum.cu: bin_certain and the bin coordinates of
cont_stacks_kernel), checked on the CPU. The kernel forms the bin coordinate
t from the two-float log10(lambda) in FP32 and takes trunc(t) only when t is
farther than the guard (1e-3 on the log grid, 5e-3 on the linear grid) from
an integer; otherwise the FP64 find_bins decides. Emulating that FP32
arithmetic (single-rounding FMAs; exp10f as the correctly rounded value
moved by up to 2 units in the last place, its documented error), every
certain index must equal find_bins_log / find_bins_lin
(py/picca/delta_extraction/utils.py:139-186) on random wavelengths."""

import numpy as np

f32 = np.float32
LN10 = f32(2.302585093)


def _fma32(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) +
            np.asarray(c, np.float64)).astype(f32)


def _split(v):
    # v = hi + lo with hi in FP32 and lo the FP32 remainder (to 2^-48 of v)
    hi = v.astype(f32)
    lo = (v - hi.astype(np.float64)).astype(f32)
    return hi, lo


def _certain(t, guard):
    a = np.abs(t.astype(np.float64))
    fr = a - np.trunc(a)
    return (a < 1e6) & (fr > guard) & (fr < 1 - guard)


def _move_ulps(x, k):
    # a positive FP32 value moved by k units in the last place
    bits = x.view(np.int32).astype(np.int64) + k
    return bits.astype(np.int32).view(f32)


def test_log_grid_indices():
    rng = np.random.default_rng(11)
    for origin in (np.log10(3600.0), np.log10(1040.0)):
        step = 3e-4
        ll = origin + rng.uniform(-0.4, 2000.4, 400_000) * step
        L_hi, L_lo = _split(ll)
        o_hi, o_lo = _split(np.array([origin]))
        inv = f32(1.0 / step)
        diff = ((L_hi - o_hi[0]).astype(f32) + (L_lo - o_lo[0]).astype(f32)).astype(f32)
        t = _fma32(diff, inv, 0.5)
        ref = ((ll - origin) / step + 0.5).astype(np.int64)
        sure = _certain(t, 1e-3)
        assert sure.mean() > 0.99
        assert np.array_equal(np.trunc(t[sure]).astype(np.int64), ref[sure])


def test_rest_frame_log_grid_indices():
    rng = np.random.default_rng(12)
    origin, step = np.log10(1040.0), 3e-4
    z = rng.uniform(2.0, 4.0, 400_000)
    zp1 = np.log10(1 + z)
    ll = zp1 + origin + rng.uniform(-0.4, 500.4, z.size) * step
    L_hi, L_lo = _split(ll)
    zr_hi, zr_lo = _split(zp1 + origin)
    diff = ((L_hi - zr_hi).astype(f32) + (L_lo - zr_lo).astype(f32)).astype(f32)
    t = _fma32(diff, f32(1.0 / step), 0.5)
    ref = (((ll - zp1) - origin) / step + 0.5).astype(np.int64)
    sure = _certain(t, 1e-3)
    assert sure.mean() > 0.99
    assert np.array_equal(np.trunc(t[sure]).astype(np.int64), ref[sure])


def test_linear_grid_indices():
    rng = np.random.default_rng(13)
    lam0, dlam = 3600.0, 0.8
    lam = lam0 + rng.uniform(-0.4, 2375.4, 400_000) * dlam
    ll = np.log10(lam)
    L_hi, L_lo = _split(ll)
    e10 = _move_ulps((10.0 ** L_hi.astype(np.float64)).astype(f32), rng.integers(-2, 3, ll.size))
    lam32 = (e10.astype(np.float64) * _fma32(L_lo, LN10, 1.0).astype(np.float64)).astype(f32)
    t = _fma32((lam32 - f32(lam0)).astype(f32), f32(1.0 / dlam), 0.5)
    ref = ((10.0 ** ll - lam0) / dlam + 0.5).astype(np.int64)
    sure = _certain(t, 5e-3)
    assert sure.mean() > 0.98
    assert np.array_equal(np.trunc(t[sure]).astype(np.int64), ref[sure])
