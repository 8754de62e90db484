"""Error bounds that the neighbour search's FP32 shortcuts rely on
(picca_gb300/csrc/pg_neighbours.cu), checked on the CPU by emulating the
kernel's FP32 arithmetic (round-to-nearest FP32 products, fused
multiply-adds rounded once) against FP64 over random sky pairs:

* the FP32 cosine of two unit vectors given in FP32 is within 4e-7 of the
  FP64 cosine, so a cosine above cos(ang_max) + 1e-5 is inside ang_max and
  one below cos(ang_max) - 1e-5 is outside (the pre-filter and the accept
  shortcut);
* for (1 + cos ang) / 2 >= 1/4, the FP32 sqrt((1 + cos ang) / 2) is within
  1e-6 relative of the FP64 cos(ang / 2) (the r_comov pre-cut shortcut, whose
  decision margin is 4e-6 relative).
"""

import numpy as np

f32 = np.float32


def _fma32(a, b, c):
    # a*b of two FP32 values is exact in FP64; one rounding of a*b + c to
    # FP32 (the FP64 sum's own rounding is far below FP32's)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _unit(ra, dec):
    return np.stack([np.cos(ra) * np.cos(dec), np.sin(ra) * np.cos(dec), np.sin(dec)], axis=-1)


def _pairs(n, max_sep, seed):
    rng = np.random.default_rng(seed)
    ra1 = rng.uniform(0, 2 * np.pi, n)
    dec1 = np.arcsin(rng.uniform(-0.99, 0.99, n))
    # the second point at a random separation and position angle
    sep = max_sep * np.sqrt(rng.uniform(0, 1, n))
    sep[: n // 10] = rng.uniform(0, 1e-4, n // 10)  # a share of very close pairs
    pa = rng.uniform(0, 2 * np.pi, n)
    dec2 = np.arcsin(np.clip(np.sin(dec1) * np.cos(sep) + np.cos(dec1) * np.sin(sep) * np.cos(pa),
                             -1, 1))
    ra2 = ra1 + np.arctan2(np.sin(pa) * np.sin(sep) * np.cos(dec1),
                           np.cos(sep) - np.sin(dec1) * np.sin(dec2))
    return _unit(ra1, dec1), _unit(ra2, dec2)


def _dot32(v1, v2):
    a, b = v1.astype(f32), v2.astype(f32)
    prod = (a[:, 0].astype(np.float64) * b[:, 0].astype(np.float64)).astype(f32)
    return _fma32(a[:, 2], b[:, 2], _fma32(a[:, 1], b[:, 1], prod))


def test_fp32_cosine_within_bound():
    for max_sep, seed in ((0.06, 1), (0.5, 2), (np.pi, 3)):
        v1, v2 = _pairs(200_000, max_sep, seed)
        dot64 = np.einsum("ij,ij->i", v1, v2)
        err = np.abs(_dot32(v1, v2).astype(np.float64) - dot64)
        assert err.max() < 4e-7, err.max()


def test_fp32_half_angle_cosine_within_bound():
    v1, v2 = _pairs(200_000, 2 * np.pi / 3, 4)
    dot32 = _dot32(v1, v2)
    xh = (f32(0.5) * (f32(1.0) + dot32)).astype(f32)
    keep = xh >= f32(0.25)
    ch = np.sqrt(np.maximum(xh, f32(0))).astype(f32)
    ang = np.arccos(np.clip(np.einsum("ij,ij->i", v1, v2), -1, 1))
    exact = np.cos(ang / 2)
    rel = np.abs(ch.astype(np.float64) - exact) / exact
    assert keep.mean() > 0.9
    assert rel[keep].max() < 1e-6, rel[keep].max()
