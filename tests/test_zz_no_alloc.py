"""The allocation-free pair accumulation (pg_cf_xi_static) gives the same
rows as the plan-based entry point (pg_cf_xi).

pg_cf_xi_static exists for callers that cannot call cudaMalloc (a framework
owns the device allocator, or every buffer is sized at start-up): its scratch
is a library-owned device array shared by all calls, so this test also
checks that a second call in a row, which finds the first call's contents in
that array, still gives the same result. Tolerances are those of the other
pair tests: identical pair counts, sums within 1e-12 (FP64 mode) or 2e-6
(precision form) relative. This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32_guard"])
def test_static_scratch_entry_matches_plan_entry(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import _native, build_ext, pairs, synthetic
    build_ext.build()
    lib = _native.lib()
    lib.pg_cf_xi_static.restype = ctypes.c_int
    lib.pg_cf_xi_static.argtypes = [
        ctypes.POINTER(_native.CorrParams), ctypes.POINTER(_native.ForestSetC),
        ctypes.POINTER(_native.ForestSetC), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(_native.XiRowsC),
        ctypes.c_void_p]
    fs = synthetic.make_forests(400, 17, (150.0, 155.0), (0.0, 5.0), 2.1, 3.5, "uniform")
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    params = pairs.make_params(0.0, 200.0, 200.0, 50, 50, ang_max)
    mode = pairs.MODE_FP64 if precision == "fp64" else pairs.MODE_FP32_GUARD
    engine = pairs.PairEngine()
    dev = pairs.DeviceForests(fs, engine.device)
    offsets, index, total = engine.neighbours(params, dev)
    order, num_work, _ = engine.work_order(dev, None, offsets, index, total)
    nrows, nbins = len(fs.healpix_list), 2500
    ref = engine.alloc_rows(nrows, nbins)
    engine.accumulate(params, dev, None, offsets, index, order, num_work, ref, mode)
    engine.stats()
    ref = [r.cpu().numpy() for r in ref]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rtol = 1e-12 if precision == "fp64" else 2e-6
    for _ in range(2):
        rows = engine.alloc_rows(nrows, nbins)
        out = _native.XiRowsC(*[r.data_ptr() for r in rows])
        status = lib.pg_cf_xi_static(ctypes.byref(params), ctypes.byref(dev.c), None,
                                     offsets.data_ptr(), index.data_ptr(), None,
                                     order.data_ptr(), num_work, mode, ctypes.byref(out), stream)
        assert status == 0, lib.pg_strerror(status)
        got = [r.cpu().numpy() for r in rows]
        assert np.array_equal(got[5], ref[5])
        for a, b in zip(got[:5], ref[:5]):
            scale = np.maximum(np.abs(b), np.sqrt(np.abs(ref[0])) * 0.1 + 1e-300)
            assert np.all(np.abs(a - b) <= rtol * scale)
