"""GPU tests of the pair kernels' launch-shape autotuner and of the CUDA-graph
replay of a step.

* Every candidate launch shape (warps per CTA, CTAs per SM) of the auto- and
  cross-correlation precision-form kernels gives pair counts identical to the
  default shape; the weight and xi sums (error-free in the block
  histograms) equal to 1e-12 and the r_par, r_trans and z sums (plain FP32
  block sums) to 2e-6, relative or of the column's largest value: only the
  order of the sums changes with the shape.
* ``tune_pairs`` picks one of the candidates, caches it, and a second call
  reads the cache without timing.
* A step captured in a CUDA graph and replayed gives the same rows as the
  eager launches.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import build_ext
    build_ext.build()
    return torch


def _workload(xcf):
    from picca_gb300 import pairs, synthetic
    fs = synthetic.make_forests(500, 17, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform")
    fs2 = (synthetic.make_quasars(800, 18, (150.0, 156.0), (0.0, 6.0)) if xcf else None)
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    if xcf:
        params = pairs.make_params(-200.0, 200.0, 200.0, 100, 50, ang_max, x_correlation=True)
    else:
        params = pairs.make_params(0.0, 200.0, 200.0, 50, 50, ang_max)
    eng = pairs.PairEngine()
    dev1 = pairs.DeviceForests(fs, eng.device)
    dev2 = pairs.DeviceForests(fs2, eng.device) if fs2 is not None else None
    offsets, index, total = eng.neighbours(params, dev1, dev2, xcf=xcf)
    order, num_work, _ = eng.work_order(dev1, dev2, offsets, index, total, xcf=xcf)
    return eng, params, dev1, dev2, offsets, index, order, num_work, len(fs.healpix_list)


def _run(eng, params, dev1, dev2, offsets, index, order, num_work, num_rows, xcf):
    from picca_gb300 import pairs
    nbins = int(params.num_bins_r_par) * int(params.num_bins_r_trans)
    rows = eng.alloc_rows(num_rows, nbins)
    eng.accumulate(params, dev1, dev2, offsets, index, order, num_work, rows,
                   pairs.MODE_FP32_GUARD, xcf=xcf)
    eng.stats()
    return [r.cpu().numpy() for r in rows]


@pytest.mark.parametrize("xcf", [False, True])
def test_every_launch_shape_gives_identical_pair_counts(cuda, xcf):
    from picca_gb300 import autotune
    work = _workload(xcf)
    eng = work[0]
    autotune.set_tuning(eng.plan)
    ref = _run(*work, xcf)
    assert ref[5].sum() > 0
    for cand in (autotune.XCF_CANDIDATES if xcf else autotune.CF_CANDIDATES):
        autotune.set_tuning(eng.plan, cf=(0, 0) if xcf else cand, xcf=cand if xcf else (0, 0))
        got = _run(*work, xcf)
        np.testing.assert_array_equal(got[5], ref[5], err_msg=str(cand))
        for k in range(5):
            # weights and xi are summed error-free in the block histograms;
            # r_par, r_trans and z sums are plain FP32 sums there
            rtol = 1e-12 if k < 2 else 2e-6
            np.testing.assert_allclose(got[k], ref[k], rtol=rtol,
                                       atol=rtol * np.abs(ref[k]).max(),
                                       err_msg=f"{cand} column {k}")


def test_tuner_picks_and_caches(cuda, tmp_path):
    from picca_gb300 import autotune, pairs
    eng, params, dev1, dev2, offsets, index, order, num_work, num_rows = _workload(False)
    path = str(tmp_path / "tune.json")
    first = autotune.tune_pairs(eng, params, dev1, dev2, offsets, index, order, num_work,
                                num_rows, pairs.MODE_FP32_GUARD, sample_items=200,
                                cache_path=path)
    assert not first["cached"]
    shapes = [(r["warps"], r["ctas_per_sm"]) for r in first["alternatives"]]
    assert tuple(first["choice"]) in shapes
    assert autotune.get_tuning(eng.plan)[0] == tuple(first["choice"])
    second = autotune.tune_pairs(eng, params, dev1, dev2, offsets, index, order, num_work,
                                 num_rows, pairs.MODE_FP32_GUARD, cache_path=path)
    assert second["cached"] and second["choice"] == first["choice"]


def test_graph_replay_matches_eager(cuda):
    from picca_gb300 import pairs
    eng, params, dev1, dev2, offsets, index, order, num_work, num_rows = _workload(False)
    eager = _run(eng, params, dev1, dev2, offsets, index, order, num_work, num_rows, False)
    nbins = int(params.num_bins_r_par) * int(params.num_bins_r_trans)
    rows = eng.alloc_rows(num_rows, nbins)
    step = pairs.GraphStep(eng, params, dev1, dev2, offsets, index, order, num_work, rows,
                           pairs.MODE_FP32_GUARD)
    for _ in range(2):
        step.replay()
        cuda.cuda.synchronize()
        eng.stats()
        got = [r.cpu().numpy() for r in rows]
        np.testing.assert_array_equal(got[5], eager[5])
        for k in range(5):
            rtol = 1e-12 if k < 2 else 2e-6
            np.testing.assert_allclose(got[k], eager[k], rtol=rtol,
                                       atol=rtol * np.abs(eager[k]).max())
