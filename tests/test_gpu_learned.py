"""GPU tests of the learned warm start.

* Kernels: the BF16 tensor-core forward (fused bias + GELU), backward (fused
  GELU derivative, column sums, MSE gradient) and Adam against the FP64
  oracle that applies the same BF16 storage rounding; tolerance 1e-2 in
  relative norm (FP32 accumulation and BF16 storage of the outputs), Adam
  to 1e-5 relative. The fused tcgen05 inference kernel against the GEMM
  forward (5e-3) and the oracle (1e-2), tails of 1 and 300 rows included.
* Method: after training on plain fits of one set of forests, the warm-started
  fit of another set reaches the plain fit's optimum ((a, b) within 1e-4,
  chi2 within 1e-6 relative) with fewer Newton iterations than the plain
  start, and falls back to the plain fit for a small fraction of forests.
* Certificate: started at the FP64 optimum, the certified fit accepts at
  least 90% of the forests in one iteration and stays there (the rest, whose
  FP32 gradient cannot certify a point, go to the plain fit); started 10%
  away with a single iteration allowed, it accepts none of the
  register-kernel forests.
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


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_backward_adam_match_oracle(cuda):
    torch = cuda
    from oracle import mlp as om
    from picca_gb300 import learned
    net = learned.WarmStartMLP(seed=3)
    rng = np.random.default_rng(1)
    m = 300
    x = np.zeros((m, learned.FEATURE_STRIDE), dtype=np.float32)
    x[:, :learned.NUM_FEATURES] = rng.normal(0, 0.5, (m, learned.NUM_FEATURES))
    t = rng.normal(0, 0.3, (m, 2)).astype(np.float32)
    x16 = torch.tensor(x, device="cuda").bfloat16()
    tt = torch.tensor(t, device="cuda")
    y, acts = net.forward(x16, keep=True)
    loss = net.backward(acts, y, tt)
    views = net._views(net.params.cpu().double())
    weights = [(w.numpy().reshape(a, b), bb.numpy()) for (w, bb), (a, b) in
               zip(views, learned.WarmStartMLP.SHAPES)]
    xin = x[:, :learned.NUM_FEATURES].astype(np.float64)
    y_ref, acts_ref = om.forward(xin, weights, quantize=True)
    assert _rel(y.cpu().numpy(), y_ref) < 1e-2
    grads_ref, loss_ref = om.backward(acts_ref, y_ref, t.astype(np.float64), weights,
                                      quantize=True)
    assert abs(float(loss.item()) - loss_ref) <= 2e-2 * loss_ref
    gviews = net._views(net.grads.cpu().double())
    for layer in range(4):
        gw, gb = gviews[layer]
        assert _rel(gw.numpy().reshape(grads_ref[layer][0].shape), grads_ref[layer][0]) < 2e-2
        assert _rel(gb.numpy(), grads_ref[layer][1]) < 2e-2
    # one Adam step
    p0 = net.params.cpu().double().numpy()
    g0 = net.grads.cpu().double().numpy()
    net.adam_step(lr=1e-3)
    p_ref, _, _ = om.adam(p0, g0, np.zeros_like(p0), np.zeros_like(p0), 1, lr=1e-3)
    assert np.allclose(net.params.cpu().double().numpy(), p_ref, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("m", [1, 300, 4096])
def test_fused_forward_matches_gemm_forward_and_oracle(cuda, m):
    """The fused tcgen05 inference kernel against the layer-by-layer GEMM
    forward (same BF16 roundings, FP32 sums in another order: 5e-3 in
    relative norm) and the FP64 oracle with BF16 storage rounding (1e-2)."""
    torch = cuda
    from oracle import mlp as om
    from picca_gb300 import learned
    net = learned.WarmStartMLP(seed=5)
    rng = np.random.default_rng(m)
    x = np.zeros((m, learned.FEATURE_STRIDE), dtype=np.float32)
    x[:, :learned.NUM_FEATURES] = rng.normal(0, 0.5, (m, learned.NUM_FEATURES))
    x16 = torch.tensor(x, device="cuda").bfloat16()
    fused = net.forward_fused(x16).cpu().numpy()
    gemm = net.forward(x16).cpu().numpy()
    assert _rel(fused, gemm) < 5e-3
    views = net._views(net.params.cpu().double())
    weights = [(w.numpy().reshape(a, b), bb.numpy()) for (w, bb), (a, b) in
               zip(views, learned.WarmStartMLP.SHAPES)]
    y_ref, _ = om.forward(x[:, :learned.NUM_FEATURES].astype(np.float64), weights,
                          quantize=True)
    assert _rel(fused, y_ref) < 1e-2
    # after an optimiser step the operand image is rebuilt
    net.grads.normal_(0, 1e-2)
    net.adam_step(lr=1e-2)
    assert _rel(net.forward_fused(x16).cpu().numpy(), net.forward(x16).cpu().numpy()) < 5e-3


def test_warm_start_reaches_plain_optimum_faster(cuda):
    torch = cuda
    from picca_gb300 import continuum, learned, synthetic_spectra
    train_raw = synthetic_spectra.make_raw_forests(3000, 101)
    eval_raw = synthetic_spectra.make_raw_forests(1000, 202)
    eng = continuum.Dr16Gpu(train_raw.grid, num_iterations=3, min_num_qso_in_fit=20)
    train = continuum.DeviceSpectra(train_raw, eng.device)
    feats, targs, _ = learned.collect_training(eng, train)
    net = learned.WarmStartMLP(seed=0)
    hist = net.train(feats, targs, epochs=8, batch=512, lr=2e-3)
    assert hist[-1] < hist[0]
    # evaluation: the same model state for both starts
    ev = continuum.DeviceSpectra(eval_raw, eng.device)
    plain = continuum.fit_results_to_host(eng.fit(ev))
    warm, _, fallback = learned.warm_fit(eng, ev, net)
    warm = continuum.fit_results_to_host(warm)
    ok = (plain["status"] == 0) & (warm["status"] == 0)
    assert ok.mean() > 0.95
    scale = np.maximum(1.0, np.maximum(np.abs(plain["zero_point"]), np.abs(plain["slope"])))
    assert np.all(np.abs(warm["zero_point"] - plain["zero_point"])[ok] <= 1e-4 * scale[ok])
    assert np.all(np.abs(warm["slope"] - plain["slope"])[ok] <= 1e-4 * scale[ok])
    # chi2 sums terms of both signs: relative to max(|chi2|, ndata)
    chi_scale = np.maximum(np.abs(plain["chi2"]), plain["ndata"])
    assert np.all(np.abs(warm["chi2"] - plain["chi2"])[ok] <= 1e-6 * chi_scale[ok])
    fallback = fallback.cpu().numpy()
    assert fallback.mean() < 0.2
    warm_iters = warm["iterations"][~fallback].mean()
    plain_iters = plain["iterations"][~fallback].mean()
    assert warm_iters < plain_iters, (warm_iters, plain_iters)


def test_certificate_accepts_optimum_rejects_far_start(cuda):
    torch = cuda
    from picca_gb300 import continuum, synthetic_spectra
    raw = synthetic_spectra.make_raw_forests(2000, 303)
    eng = continuum.Dr16Gpu(raw.grid, num_iterations=1)
    sp = continuum.DeviceSpectra(raw, eng.device)
    ref = eng.fit(sp)
    ok = (ref["status"] == 0).cpu().numpy()
    start = torch.stack([ref["zero_point"], ref["slope"]], 1).contiguous()
    start = torch.nan_to_num(start)
    cert = continuum.fit_results_to_host(eng.fit_warm(sp, start, max_iter=3))
    host = continuum.fit_results_to_host(ref)
    # forests whose FP32 gradient is too noisy to certify a point (those the
    # plain fit finishes in FP64) are left to the plain fit: a few percent
    acc = ok & (cert["status"] == 0)
    assert acc.sum() >= 0.9 * ok.sum(), (acc.sum(), ok.sum())
    assert np.all(cert["status"][ok & ~acc] == 1)
    # one Newton step from the optimum for all but the nearly degenerate
    # forests (an FP32 Hessian without a positive determinant takes gradient
    # steps first)
    assert np.mean(cert["iterations"][acc] <= 1) >= 0.95
    scale = np.maximum(1.0, np.maximum(np.abs(host["zero_point"]), np.abs(host["slope"])))
    assert np.all(np.abs(cert["zero_point"] - host["zero_point"])[acc] <= 1e-5 * scale[acc])
    assert np.all(np.abs(cert["slope"] - host["slope"])[acc] <= 1e-5 * scale[acc])
    chi_scale = np.maximum(np.abs(host["chi2"]), host["ndata"])
    assert np.all(np.abs(cert["chi2"] - host["chi2"])[acc] <= 1e-6 * chi_scale[acc])
    # 10% off, one iteration: the Newton step is too long to be taken uncertified
    far = start.clone()
    far[:, 0] *= 1.1
    far[:, 1] += 0.1 * far[:, 0]
    short = np.diff(raw.pix_offset) <= 224
    res = continuum.fit_results_to_host(eng.fit_warm(sp, far, max_iter=1))
    assert np.all(res["status"][ok & short] == 1)


def test_fused_warm_start_matches_features_then_network(cuda):
    """pg_mlp_warm_start (features formed inside the tensor-core kernel)
    gives the a0 of pg_mlp_features and the network output of
    pg_mlp_forward on its features (700 forests: a partial last tile)."""
    torch = cuda
    from picca_gb300 import continuum, learned, synthetic_spectra
    raw = synthetic_spectra.make_raw_forests(700, 404)
    eng = continuum.Dr16Gpu(raw.grid, num_iterations=1)
    sp = continuum.DeviceSpectra(raw, eng.device)
    net = learned.WarmStartMLP(seed=7)
    model_c, keep = eng._model()
    feat, a0 = learned.features(eng, sp, model_c)
    y_ref = net.forward_fused(feat)
    y, a0_f = net.warm_start(eng, sp, model_c)
    assert torch.equal(a0[:700], a0_f)
    assert float((y - y_ref).norm() / y_ref.norm()) < 1e-6
