"""The algebra of the factored cross Wick terms (pg_xcf_wick_factored) on
the CPU: with U[i, P] = sum of the quasars' zw over the listed pairs of pixel
i in bin P and W[i, P] = sum of w1 w_q, U^T X1' U - T2 and
W^T diag(zw1 / w1) W - diag(sum c w12^2) equal the oracle's T4 and T3 (the
loop of xcf.compute_wickT1234_pairs, py/picca/xcf.py:1318-1350) for one
forest and its quasars; and the pixels a quasar keeps form one interval (the
direct T2 sum relies on it)."""

import numpy as np

from conftest import golden
from oracle import cpu
from oracle import wick as ow
from picca_gb300 import constants, synthetic, utils


def test_factored_terms_match_the_loop():
    fs = synthetic.make_forests(30, 17, (150.0, 151.5), (0.0, 1.5), max_pixels=160)
    qs = synthetic.make_quasars(500, 18, (150.0, 151.5), (0.0, 1.5), z_lo=2.0, z_hi=3.6)
    variance, xi = ow.interpolants(golden("cf1d.npz"))
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    rp, np_, nt = 100.0, 40, 20
    p = ow.make_params(-rp, rp, rp, np_, nt, x_correlation=True)
    ang_max = utils.compute_ang_max(cosmo, rp, 2.0, 2.0)
    offsets, index = cpu.neighbours(fs, qs, cpu.make_params(-rp, rp, rp, np_, nt), ang_max,
                                    auto_mode=0, xcf=True)
    f = int(np.argmax(np.diff(offsets)))
    nbrs = [int(index[k]) for k in range(int(offsets[f]), int(offsets[f + 1]))]
    assert len(nbrs) > 20
    po = np.asarray(fs.pix_offset)
    sl = slice(po[f], po[f + 1])
    w1, z1, r1 = fs.weights[sl], fs.z[sl], fs.r_comov[sl]
    x1 = ow.weighted_xi_1d(fs.log_lambda[sl], w1, variance, xi)
    zw1 = ((1 + z1) / 3.25) ** 1.9
    ang = np.array([cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                           fs.dec[f], fs.cos_dec[f], qs.x_cart[g],
                                           qs.y_cart[g], qs.z_cart[g], qs.ra[g], qs.dec[g])
                    for g in nbrs])
    rq, wq = qs.obj_r_comov[nbrs], qs.obj_weight[nbrs]
    zwq = ((1 + qs.z_qso[nbrs]) / 3.25) ** 0.44
    out = ow.new_outputs(p)
    out["t4"] = np.zeros_like(out["t1"])
    ow.xforest(p, r1, w1, zw1, x1, rq, wq, zwq, ang, out)

    r_par = (r1[:, None] - rq[None, :]) * np.cos(ang / 2)[None, :]
    r_trans = (r1[:, None] + rq[None, :]) * np.sin(ang / 2)[None, :]
    keep = (r_par < rp) & (r_trans < rp) & (r_par >= -rp)
    bins = ((r_trans / rp * nt).astype(int)
            + nt * ((r_par + rp) / (2 * rp) * np_).astype(int))
    used = np.unique(bins[keep])
    col = {b: k for k, b in enumerate(used)}
    nz, n1 = used.size, r1.size
    u, w, d, t2 = np.zeros((n1, nz)), np.zeros((n1, nz)), np.zeros(nz), np.zeros((nz, nz))
    c = zw1 / w1
    x1z = x1.copy()
    np.fill_diagonal(x1z, 0.0)
    for j in range(rq.size):
        kept = np.nonzero(keep[:, j])[0]
        if kept.size:
            assert kept[-1] - kept[0] + 1 == kept.size  # one interval per quasar
        cols = [col[bins[i, j]] for i in kept]
        for ci, i in zip(cols, kept):
            w12 = w1[i] * wq[j]
            u[i, ci] += zwq[j]
            w[i, ci] += w12
            d[ci] += c[i] * w12 * w12
            for ck, k in zip(cols, kept):
                t2[ci, ck] += x1z[i, k] * zwq[j] ** 2
    t24 = u.T @ (x1z @ u)
    t3 = w.T @ (c[:, None] * w) - np.diag(d)

    def embed(block):
        full = np.zeros((np_ * nt, np_ * nt))
        full[np.ix_(used, used)] = block
        return full

    for got, want in ((embed(t2), out["t2"]), (embed(t24 - t2), out["t4"]),
                      (embed(t3), out["t3"])):
        scale = np.abs(want).max()
        assert scale > 0
        assert np.all(np.abs(got - want) <= 1e-10 * np.abs(want) + 1e-12 * scale)
