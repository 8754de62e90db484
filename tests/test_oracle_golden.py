"""Pin the CPU oracle against picca's own outputs.

1. Function level: the C restatements of ``cf.compute_xi_forest_pairs_fast``
   and ``xcf.compute_xi_forest_pairs_fast`` against the reference functions
   themselves (run as plain Python when the fixtures were made), for every
   option branch: bit-identical counts and sums.
2. End to end: the oracle pipeline (neighbours + pair sums + aggregation) on
   picca's test deltas against picca's golden correlation files, with the
   reference test's comparison rule (exact, else allclose rtol 1e-5 / atol
   1e-8, py/picca/tests/test_helpers.py:45-108) and exact pair counts.
"""

import numpy as np
import pytest

from conftest import golden
from corr_cases import CASES, prepare
from oracle import cpu as oracle


def _cf_case_params(p):
    nan_none = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
    return oracle.make_params(
        p[0], p[1], p[2], int(p[3]), int(p[4]), z_min_pairs=nan_none(p[5]),
        z_max_pairs=nan_none(p[6]), zerr_cut_deg=nan_none(p[7]), zerr_cut_kms=nan_none(p[8]),
        x_correlation=bool(p[9]), rmu_binning=bool(p[10]), ang_correlation=bool(p[11]),
        remove_same_half_plate_close_pairs=bool(p[12]))


def test_cf_pair_function_matches_reference():
    f = golden("pair_cases.npz")
    for k in range(int(f["num_cf_cases"])):
        pre = f"cf{k}_"
        params = _cf_case_params(f[pre + "params"])
        nbins = params.num_bins_r_par * params.num_bins_r_trans
        outs = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
        zq1, zq2, ang, shp = f[pre + "scalars"]
        oracle.cf_forest_pair(params, f[pre + "z1"], f[pre + "r1"], f[pre + "m1"], f[pre + "w1"],
                              f[pre + "d1"], zq1, f[pre + "z2"], f[pre + "r2"], f[pre + "m2"],
                              f[pre + "w2"], f[pre + "d2"], zq2, ang, bool(shp), outs)
        for name, got in zip(("we", "xi", "rp", "rt", "z", "nb"), outs):
            want = f[pre + "out_" + name]
            assert np.array_equal(got, want), (k, str(f[pre + "name"]), name)


def test_xcf_pair_function_matches_reference():
    f = golden("pair_cases.npz")
    for k in range(int(f["num_xcf_cases"])):
        pre = f"xcf{k}_"
        p = f[pre + "params"]
        params = oracle.make_params(
            p[0], p[1], p[2], int(p[3]), int(p[4]),
            z_min_pairs=None if np.isnan(p[5]) else p[5],
            z_max_pairs=None if np.isnan(p[6]) else p[6], rmu_binning=bool(p[7]))
        nbins = params.num_bins_r_par * params.num_bins_r_trans
        outs = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
        oracle.xcf_forest(params, f[pre + "z1"], f[pre + "r1"], f[pre + "m1"], f[pre + "w1"],
                          f[pre + "d1"], f[pre + "zq"], f[pre + "rq"], f[pre + "mq"],
                          f[pre + "wq"], f[pre + "ang"], outs)
        for name, got in zip(("we", "xi", "rp", "rt", "z", "nb"), outs):
            want = f[pre + "out_" + name]
            assert np.array_equal(got, want), (k, str(f[pre + "name"]), name)


def compare_like_reference(got, want, names=("RP", "RT", "Z", "NB", "HEALPID", "WE", "DA")):
    """The reference test rule, plus exact equality for integer columns."""
    for name in names:
        a = np.asarray(want[name])
        b = np.asarray(got[name])
        assert a.shape == b.shape, name
        if a.dtype.kind in "iu":
            assert np.array_equal(a, b), name
        elif not np.array_equal(a, b):
            assert np.allclose(a, b, rtol=1e-5, atol=1e-8), (
                name, float(np.max(np.abs(a - b))))


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_pipeline_matches_golden(case, picca_inputs):
    set1, set2, params, ang_max, kind = prepare(case, picca_inputs)
    p = oracle.make_params(**params)
    if kind == "cf":
        got = oracle.cf_pipeline(set1, set2, p, ang_max)
    else:
        got = oracle.xcf_pipeline(set1, set2, p, ang_max)
    compare_like_reference(got, golden(f"cor_{case}.npz"))
