"""The guard bands of the precision-form pair kernel
(picca_gb300/csrc/pg_pairs_fast.cu: make_fast_const, stage_forest1, the
chunk staging and the per-pair FMAs), checked on the CPU: the kernel's FP32
evaluation of the bin coordinates x' (r_par) and x_tr' (r_trans), emulated
with FP32 roundings and single-rounding FMAs, stays within the guard bands
of the exact (FP64) values for every pixel pair within one bin of the
accepted ranges. A pair outside its band is decided from FP32 alone, so this
is what makes the FP32 bins equal to the reference's FP64 bins."""

import numpy as np

from picca_gb300 import synthetic

f32 = np.float32
U = 2.0 ** -24


def _fma32(a, b, c):
    # products of FP32 values are exact in FP64; one rounding to FP32
    return (a.astype(np.float64) * b.astype(np.float64) + np.float64(c)).astype(f32)


def _guards(np_, nt, r_par_min, r_par_range, r_trans_max, max_rho):
    inv_p = np_ / r_par_range
    pmin = r_par_min * inv_p
    g_par = 16 * U * (np_ + abs(pmin) + 2) + 1e-6 + 8 * U * inv_p * max_rho
    g_tr = 16 * U * (nt + 2) + 1e-6
    return g_par, g_tr


def test_fp32_bin_coordinates_within_guards():
    np_, nt, r_par_max, r_trans_max = 50, 50, 200.0, 200.0
    fs = synthetic.make_forests(400, 17, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform")
    ang_max = synthetic.correlation_ang_max(r_trans_max, float(fs.z.min()))
    inv_p, inv_t = np_ / r_par_max, nt / r_trans_max
    pc = f32(0.5)
    v = np.stack([fs.x_cart, fs.y_cart, fs.z_cart], axis=1)
    rng = np.random.default_rng(3)
    checked = 0
    worst_par = worst_tr = 0.0
    for f1 in rng.choice(fs.num, size=60, replace=False):
        cosang = np.clip(v @ v[f1], -1, 1)
        nbrs = np.nonzero((np.arccos(cosang) < ang_max) & (np.arange(fs.num) != f1))[0][:20]
        a0, a1 = fs.pix_offset[f1], fs.pix_offset[f1 + 1]
        r1, d1 = fs.r_comov[a0:a1], fs.dist_m[a0:a1]
        r_ref = r1[(a1 - a0) // 2]
        rho1 = (r1 - r_ref).astype(f32)
        max_rho = float(np.abs(rho1).max())
        g_par, g_tr = _guards(np_, nt, 0.0, r_par_max, r_trans_max, max_rho)
        for g in nbrs:
            ang = float(np.arccos(cosang[g]))
            c, s = np.cos(ang / 2), np.sin(ang / 2)
            cp, st = f32(c * inv_p), f32(s * inv_t)
            b0, b1 = fs.pix_offset[g], fs.pix_offset[g + 1]
            r2, d2 = fs.r_comov[b0:b1], fs.dist_m[b0:b1]
            # chunk staging: nB = -(cp * rho2) rounded once, t = st d2 - 1/2 (FMA)
            nb = (-(cp.astype(np.float64) * (r2 - r_ref).astype(f32).astype(np.float64))).astype(f32)
            t = _fma32(np.full(b1 - b0, st), d2.astype(f32), -0.5)
            # per pair: p = cp rho1 + nB (FMA), x' = |p| - pc; x_tr' = st d1 + t (FMA)
            p = _fma32(np.full((a1 - a0, b1 - b0), cp), rho1[:, None], nb[None, :])
            xp = (np.abs(p) - pc).astype(f32)
            xt = _fma32(np.full((a1 - a0, b1 - b0), st), d1.astype(f32)[:, None], t[None, :])
            # the reference's FP64 values in the same units
            x_exact = np.abs((r1[:, None] - r2[None, :]) * c) * inv_p - 0.5
            xt_exact = (d1[:, None] + d2[None, :]) * s * inv_t - 0.5
            keep = (x_exact >= -1) & (x_exact <= np_ + 1) & (xt_exact >= -1) & (xt_exact <= nt + 1)
            err_par = np.abs(xp.astype(np.float64) - x_exact)[keep]
            err_tr = np.abs(xt.astype(np.float64) - xt_exact)[keep]
            if err_par.size:
                assert err_par.max() < g_par, (err_par.max(), g_par)
                assert err_tr.max() < g_tr, (err_tr.max(), g_tr)
                worst_par = max(worst_par, err_par.max() / g_par)
                worst_tr = max(worst_tr, err_tr.max() / g_tr)
                checked += err_par.size
    assert checked > 100_000
    # the bands are not vacuous: the errors use a sizeable part of them
    assert worst_par > 0.01 and worst_tr > 0.01


def test_fp32_cross_bin_coordinates_within_guards():
    """The delta x quasar form (xcf_xi_fast_kernel): signed r_par from -200
    to 200 in 100 bins, the quasar staged as nB = -cp rho_q and
    t = st d_q - 1/2, per pixel p = cp rho1 + nB and x_tr' = st d1 + t."""
    np_, nt, r_par_min, r_par_max, r_trans_max = 100, 50, -200.0, 200.0, 200.0
    fs = synthetic.make_forests(300, 21, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform")
    qs = synthetic.make_quasars(600, 22, (150.0, 156.0), (0.0, 6.0))
    ang_max = synthetic.correlation_ang_max(r_trans_max, float(fs.z.min()))
    inv_p, inv_t = np_ / (r_par_max - r_par_min), nt / r_trans_max
    pmin = r_par_min * inv_p
    pc = f32(pmin + 0.5)
    vq = np.stack([qs.x_cart, qs.y_cart, qs.z_cart], axis=1)
    rng = np.random.default_rng(4)
    checked = 0
    worst_par = worst_tr = 0.0
    for f1 in rng.choice(fs.num, size=80, replace=False):
        v1 = np.array([fs.x_cart[f1], fs.y_cart[f1], fs.z_cart[f1]])
        cosang = np.clip(vq @ v1, -1, 1)
        nbrs = np.nonzero(np.arccos(cosang) < ang_max)[0]
        a0, a1 = fs.pix_offset[f1], fs.pix_offset[f1 + 1]
        r1, d1 = fs.r_comov[a0:a1], fs.dist_m[a0:a1]
        r_ref = r1[(a1 - a0) // 2]
        rho1 = (r1 - r_ref).astype(f32)
        g_par, g_tr = _guards(np_, nt, r_par_min, r_par_max - r_par_min, r_trans_max,
                              float(np.abs(rho1).max()))
        if not nbrs.size:
            continue
        ang = np.arccos(cosang[nbrs])
        c, s = np.cos(ang / 2), np.sin(ang / 2)
        cp, st = (c * inv_p).astype(f32), (s * inv_t).astype(f32)
        rq, dq = qs.obj_r_comov[nbrs], qs.obj_dist_m[nbrs]
        nb = (-(cp.astype(np.float64) * (rq - r_ref).astype(f32).astype(np.float64))).astype(f32)
        t = _fma32(st, dq.astype(f32), -0.5)
        p = _fma32(cp[None, :], rho1[:, None], nb[None, :])
        xp = (p - pc).astype(f32)
        xt = _fma32(st[None, :], d1.astype(f32)[:, None], t[None, :])
        x_exact = (r1[:, None] - rq[None, :]) * c[None, :] * inv_p - pmin - 0.5
        xt_exact = (d1[:, None] + dq[None, :]) * s[None, :] * inv_t - 0.5
        keep = (x_exact >= -1) & (x_exact <= np_ + 1) & (xt_exact >= -1) & (xt_exact <= nt + 1)
        err_par = np.abs(xp.astype(np.float64) - x_exact)[keep]
        err_tr = np.abs(xt.astype(np.float64) - xt_exact)[keep]
        if err_par.size:
            assert err_par.max() < g_par, (err_par.max(), g_par)
            assert err_tr.max() < g_tr, (err_tr.max(), g_tr)
            worst_par = max(worst_par, err_par.max() / g_par)
            worst_tr = max(worst_tr, err_tr.max() / g_tr)
            checked += err_par.size
    assert checked > 20_000
    assert worst_par > 0.01 and worst_tr > 0.01


def _move_ulps(x, k):
    bits = x.view(np.int32).astype(np.int64) + k
    return bits.astype(np.int32).view(f32)


def _round_rem(x):
    # round to nearest even (the kernel's magic-number add) and the remainder
    r = np.rint(x.astype(np.float64))
    return r.astype(np.int64), (x.astype(np.float64) - r)


def test_fp32_rmu_bins_outside_guards_equal_fp64():
    """r-mu binning (auto, mu in [0, 1] in 50 bins, r in [0, 200] in 50): the
    kernel's FP32 r = r2 rsqrt(r2) and mu = |p| rsqrt(r2), with rsqrtf taken
    up to 2 units in the last place off (its documented error); every pair
    that the kernel does not queue for the FP64 re-decision gets the FP64
    bins and acceptance."""
    np_, nt, r_trans_max = 50, 50, 200.0
    fs = synthetic.make_forests(300, 23, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform")
    ang_max = synthetic.correlation_ang_max(r_trans_max, float(fs.z.min()))
    inv_t = nt / r_trans_max
    inv_mu, mu_off = f32(np_ / 1.0), f32(0.5)
    g_mu0 = 16 * U * (np_ + 2) + 1e-6
    g_tr = 32 * U * (nt + 2) + 1e-6
    v = np.stack([fs.x_cart, fs.y_cart, fs.z_cart], axis=1)
    rng = np.random.default_rng(5)
    checked = queued = 0
    for f1 in rng.choice(fs.num, size=40, replace=False):
        cosang = np.clip(v @ v[f1], -1, 1)
        nbrs = np.nonzero((np.arccos(cosang) < ang_max) & (np.arange(fs.num) != f1))[0][:12]
        a0, a1 = fs.pix_offset[f1], fs.pix_offset[f1 + 1]
        r1, d1 = fs.r_comov[a0:a1], fs.dist_m[a0:a1]
        r_ref = r1[(a1 - a0) // 2]
        rho1 = (r1 - r_ref).astype(f32)
        g = min(16 * U * (nt + 2) + 1e-6 + 8 * U * inv_t * float(np.abs(rho1).max()), 0.05)
        low_clamp = f32(-0.5 + 2 * g)
        h_r = f32(0.5 - g_tr - g)
        for k in nbrs:
            ang = float(np.arccos(cosang[k]))
            c, s = np.cos(ang / 2), np.sin(ang / 2)
            cp, st = f32(c * inv_t), f32(s * inv_t)
            b0, b1 = fs.pix_offset[k], fs.pix_offset[k + 1]
            r2, d2 = fs.r_comov[b0:b1], fs.dist_m[b0:b1]
            nb = (-(np.float64(cp) * (r2 - r_ref).astype(f32).astype(np.float64))).astype(f32)
            t2 = (np.float64(st) * d2.astype(f32).astype(np.float64)).astype(f32)
            shape = (a1 - a0, b1 - b0)
            pp = _fma32(np.full(shape, cp), rho1[:, None], nb[None, :])
            xt = _fma32(np.full(shape, st), d1.astype(f32)[:, None], t2[None, :])
            rr = _fma32(pp, pp, (xt.astype(np.float64) ** 2).astype(f32))
            sinv = _move_ulps((1.0 / np.sqrt(rr.astype(np.float64))).astype(f32),
                              rng.integers(-2, 3, shape))
            ru = (rr.astype(np.float64) * sinv).astype(f32)
            mu = (np.abs(pp).astype(np.float64) * sinv).astype(f32)
            xm = np.maximum(_fma32(mu, inv_mu, -mu_off), low_clamp)
            ip, fp = _round_rem(xm)
            it, ft = _round_rem((ru - f32(0.5)).astype(f32))
            gm = _fma32((f32(g) * sinv).astype(f32), inv_mu, g_mu0)
            near = ~(gm < 0.25) | (np.abs(fp) > 0.5 - gm) | (np.abs(ft) > h_r)
            acc32 = (ip >= 0) & (ip < np_) & (it >= 0) & (it < nt)
            # the reference: r and mu from the FP64 r_par, r_trans
            rp = (r1[:, None] - r2[None, :]) * c
            rt = (d1[:, None] + d2[None, :]) * s
            r = np.sqrt(rp ** 2 + rt ** 2)
            with np.errstate(invalid="ignore", divide="ignore"):
                mu64 = np.abs(rp) / r
            bmu, br = np.floor(mu64 * np_).astype(np.int64), np.floor(r * inv_t).astype(np.int64)
            acc64 = (r > 0) & (bmu < np_) & (br < nt)
            sure = ~near & (r > 0)
            assert np.array_equal(acc32[sure], acc64[sure])
            both = sure & acc64
            assert np.array_equal(ip[both], bmu[both]) and np.array_equal(it[both], br[both])
            checked += int(sure.sum())
            queued += int(near.sum())
    assert checked > 100_000
    assert queued < 0.01 * checked


def test_half_angle_identities_give_the_fp32_constants():
    """The cross-correlation kernel forms cos and sin of half the angle from
    the half-angle identities on the FP64 dot product above 1e-3 rad; the FP32
    constants cp and st it derives are those of the trigonometric form."""
    rng = np.random.default_rng(9)
    ang = np.concatenate([rng.uniform(1e-3, 0.3, 1_000_000), np.geomspace(1e-3, 3.0, 10_000)])
    cosang = np.cos(ang)
    trig = np.arccos(cosang) / 2
    for inv in (0.25, 0.5, 100.0 / 400.0):
        cp_trig = (np.cos(trig) * inv).astype(f32)
        st_trig = (np.sin(trig) * inv).astype(f32)
        cp_half = (np.sqrt(0.5 * (1.0 + cosang)) * inv).astype(f32)
        st_half = (np.sqrt(0.5 * (1.0 - cosang)) * inv).astype(f32)
        assert np.array_equal(cp_half, cp_trig)
        # sin: at most one unit in the last place apart, where the two FP64
        # values straddle an FP32 rounding boundary
        ulps = np.abs(st_half.view(np.int32).astype(np.int64) - st_trig.view(np.int32))
        assert ulps.max() <= 1 and (ulps > 0).mean() < 1e-4
