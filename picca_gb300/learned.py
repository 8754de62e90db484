"""Learned warm start for the Dr16 continuum fit (no counterpart in picca).

A 66 -> 256 -> 256 -> 256 -> 2 MLP with GELU activations predicts, from a
forest's flux divided by the current mean continuum (64 rest-frame bins),
its redshift and signal-to-noise, the continuum parameters relative to the
reference starting point a0 (the ivar-weighted mean flux,
expected_fluxes/utils.py:92): targets (a/a0 - 1, b/a0). Training runs every
matrix product in the library's BF16 GEMM with FP32 accumulation (forward
with fused bias + GELU, backward with fused GELU derivative) and the
library's Adam kernel on FP32 master weights; inference (the warm start)
runs the whole network in one fused tcgen05 kernel (pg_mlp_forward).

The plain fit stays the reference: ``warm_fit`` starts the damped Newton
solver from the prediction with a small iteration budget and re-fits from
a0 (the plain start) every forest whose warm-started fit does not converge;
the fraction re-fitted is the fallback rate.
"""

import ctypes
import math

import numpy as np
import torch

from . import _native, continuum
from ._native import check

HIDDEN = 256
NUM_FEATURES = 66
FEATURE_STRIDE = 80
NUM_OUT = 2
EPI_NONE, EPI_GELU, EPI_GELU_GRAD = 0, 1, 2


def _bind():
    lib = _native.lib()
    if getattr(lib, "_mlp_bound", False):
        return lib
    vp, i64, i32, f32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_float
    lib.pg_mlp_gemm.argtypes = [vp, i64, i64, vp, i64, i64, i32, i32, i32, vp, i32, vp, vp, i64,
                                vp, vp, i64, f32, vp]
    lib.pg_mlp_colsum.argtypes = [vp, i32, i32, i64, vp, vp]
    lib.pg_mlp_mse_grad.argtypes = [vp, vp, i32, i32, vp, vp, vp]
    lib.pg_mlp_adam.argtypes = [vp, vp, vp, vp, vp, i64, f32, f32, f32, f32, i32, f32, vp]
    lib.pg_mlp_to_bf16.argtypes = [vp, vp, i64, vp]
    lib.pg_mlp_features.argtypes = [vp, ctypes.POINTER(continuum.SpectraC),
                                    ctypes.POINTER(continuum.ContModelC), vp, i32, vp, vp]
    lib.pg_mlp_packed_elems.argtypes = []
    lib.pg_mlp_packed_elems.restype = ctypes.c_int64
    lib.pg_mlp_pack.argtypes = [vp, vp, vp]
    lib.pg_mlp_forward.argtypes = [vp, vp, vp, vp, i64, i32, vp, vp]
    lib.pg_mlp_warm_start.argtypes = [vp, ctypes.POINTER(continuum.SpectraC),
                                      ctypes.POINTER(continuum.ContModelC), vp, vp, vp, vp, vp]
    for name in ("pg_mlp_gemm", "pg_mlp_colsum", "pg_mlp_mse_grad", "pg_mlp_adam",
                 "pg_mlp_to_bf16", "pg_mlp_features", "pg_mlp_pack", "pg_mlp_forward",
                 "pg_mlp_warm_start"):
        getattr(lib, name).restype = ctypes.c_int
    lib._mlp_bound = True
    return lib


def _ptr(t):
    return None if t is None else t.data_ptr()


class WarmStartMLP:
    """Parameters, Adam state and the forward/backward passes."""

    SHAPES = [(NUM_FEATURES, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, NUM_OUT)]

    def __init__(self, device=None, seed=0):
        from .pairs import require_cuda
        require_cuda()
        _bind()
        self.device = torch.device(device or "cuda")
        sizes = []
        for fan_in, fan_out in self.SHAPES:
            sizes += [fan_in * fan_out, fan_out]
        self.sizes = sizes
        total = sum(sizes)
        gen = torch.Generator().manual_seed(seed)
        flat = torch.zeros(total, dtype=torch.float32)
        off = 0
        for (fan_in, fan_out) in self.SHAPES:
            bound = math.sqrt(6.0 / (fan_in + fan_out))
            flat[off:off + fan_in * fan_out] = (torch.rand(fan_in * fan_out, generator=gen) * 2 - 1) * bound
            off += fan_in * fan_out + fan_out
        self.params = flat.to(self.device)
        self.grads = torch.zeros_like(self.params)
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.params16 = torch.empty(total, dtype=torch.bfloat16, device=self.device)
        # the tensor-core operand image of the weights, rebuilt when they change
        self.packed = torch.empty(int(_bind().pg_mlp_packed_elems()), dtype=torch.bfloat16,
                                  device=self.device)
        self._packed_step = -1
        self._plan = None
        self.step = 0
        self._sync16()

    # parameter views -------------------------------------------------------
    def _views(self, flat):
        out, off = [], 0
        for (fan_in, fan_out) in self.SHAPES:
            out.append((flat[off:off + fan_in * fan_out], flat[off + fan_in * fan_out:
                                                               off + fan_in * fan_out + fan_out]))
            off += fan_in * fan_out + fan_out
        return out

    def _sync16(self):
        self._packed_step = -1
        check(_bind().pg_mlp_to_bf16(self.params.data_ptr(), self.params16.data_ptr(),
                                     self.params.numel(), self._stream()), "to_bf16")

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def gemm(self, a, sam, sak, b, sbk, sbn, m, n, k, bias=None, epilogue=EPI_NONE, zin=None,
             zout=None, ldz=0, c=None, cf=None, ldc=0, beta=0.0):
        check(_bind().pg_mlp_gemm(a.data_ptr(), sam, sak, b.data_ptr(), sbk, sbn, m, n, k,
                                  _ptr(bias), epilogue, _ptr(zin), _ptr(zout), ldz, _ptr(c),
                                  _ptr(cf), ldc, beta, self._stream()), "mlp gemm")

    # forward ---------------------------------------------------------------
    def forward_fused(self, x16):
        """Inference forward pass in one tcgen05 kernel (pg_mlp_forward):
        x16 bf16 [m, FEATURE_STRIDE] -> FP32 [m, 2]."""
        lib = _bind()
        self._ensure_packed()
        m = x16.shape[0]
        y = torch.empty(m, NUM_OUT, dtype=torch.float32, device=self.device)
        check(lib.pg_mlp_forward(self._plan.handle, self.packed.data_ptr(), self.params.data_ptr(),
                                 x16.data_ptr(), m, x16.stride(0), y.data_ptr(), self._stream()),
              "mlp forward")
        return y

    def _ensure_packed(self):
        if self._packed_step != self.step:
            check(_bind().pg_mlp_pack(self.params16.data_ptr(), self.packed.data_ptr(),
                                      self._stream()), "mlp pack")
            self._packed_step = self.step
        if self._plan is None:
            from ._native import Plan
            self._plan = Plan()

    def warm_start(self, engine, spectra, model_c):
        """Features and network in one kernel (pg_mlp_warm_start): returns the
        FP32 output [num, 2] and a0 (FP64 [num])."""
        self._ensure_packed()
        n = spectra.num
        y = torch.empty(max(n, 1), NUM_OUT, dtype=torch.float32, device=self.device)
        a0 = torch.empty(max(n, 1), dtype=torch.float64, device=self.device)
        check(_bind().pg_mlp_warm_start(self._plan.handle, ctypes.byref(spectra.c),
                                        ctypes.byref(model_c), self.packed.data_ptr(),
                                        self.params.data_ptr(), y.data_ptr(), a0.data_ptr(),
                                        self._stream()), "mlp warm start")
        return y[:n], a0[:n]

    def forward(self, x16, keep=False):
        """x16: bf16 [m, FEATURE_STRIDE] (first 66 columns used). Returns
        the FP32 output [m, 2] and, with keep=True, the activations."""
        m = x16.shape[0]
        w16 = self._views(self.params16)
        w32 = self._views(self.params)
        acts = {"x": x16}
        h = x16
        ld_in, k_in = FEATURE_STRIDE, NUM_FEATURES
        for layer in range(3):
            z = torch.empty(m, HIDDEN, dtype=torch.float32, device=self.device) if keep else None
            out = torch.empty(m, HIDDEN, dtype=torch.bfloat16, device=self.device)
            self.gemm(h, ld_in, 1, w16[layer][0], HIDDEN, 1, m, HIDDEN, k_in,
                      bias=w32[layer][1], epilogue=EPI_GELU, zout=z, ldz=HIDDEN, c=out,
                      ldc=HIDDEN)
            acts[f"z{layer}"] = z
            acts[f"h{layer}"] = out
            h, ld_in, k_in = out, HIDDEN, HIDDEN
        y = torch.empty(m, NUM_OUT, dtype=torch.float32, device=self.device)
        self.gemm(h, HIDDEN, 1, w16[3][0], NUM_OUT, 1, m, NUM_OUT, HIDDEN, bias=w32[3][1],
                  cf=y, ldc=NUM_OUT)
        return (y, acts) if keep else y

    def backward(self, acts, y, target):
        """Gradients of the MSE loss into self.grads; returns the loss."""
        lib = _bind()
        m = y.shape[0]
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        dz = torch.empty(m, NUM_OUT, dtype=torch.bfloat16, device=self.device)
        check(lib.pg_mlp_mse_grad(y.data_ptr(), target.data_ptr(), m, NUM_OUT, dz.data_ptr(),
                                  loss.data_ptr(), self._stream()), "mse grad")
        w16 = self._views(self.params16)
        g32 = self._views(self.grads)
        width = NUM_OUT
        for layer in (3, 2, 1, 0):
            h_in = acts["x"] if layer == 0 else acts[f"h{layer - 1}"]
            ld_in = FEATURE_STRIDE if layer == 0 else HIDDEN
            fan_in = NUM_FEATURES if layer == 0 else HIDDEN
            # dW = h_in^T dz
            self.gemm(h_in, 1, ld_in, dz, width, 1, fan_in, width, m, cf=g32[layer][0],
                      ldc=width)
            check(lib.pg_mlp_colsum(dz.data_ptr(), m, width, width, g32[layer][1].data_ptr(),
                                    self._stream()), "colsum")
            if layer == 0:
                break
            # dz_prev = (dz W^T) * gelu'(z_prev)
            dprev = torch.empty(m, HIDDEN, dtype=torch.bfloat16, device=self.device)
            self.gemm(dz, width, 1, w16[layer][0], 1, width, m, HIDDEN, width,
                      epilogue=EPI_GELU_GRAD, zin=acts[f"z{layer - 1}"], ldz=HIDDEN, c=dprev,
                      ldc=HIDDEN)
            dz, width = dprev, HIDDEN
        return loss

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step += 1
        check(_bind().pg_mlp_adam(self.params.data_ptr(), self.grads.data_ptr(),
                                  self.m1.data_ptr(), self.m2.data_ptr(),
                                  self.params16.data_ptr(), self.params.numel(), lr, beta1,
                                  beta2, eps, self.step, weight_decay, self._stream()), "adam")

    def train(self, x16, target, epochs=5, batch=4096, lr=1e-3, seed=0, log=None):
        """Mini-batch Adam on (features, targets) device tensors."""
        n = x16.shape[0]
        gen = torch.Generator(device=self.device).manual_seed(seed)
        history = []
        for epoch in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=gen)
            total = 0.0
            steps = 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                xb = x16.index_select(0, idx).contiguous()
                tb = target.index_select(0, idx).contiguous()
                y, acts = self.forward(xb, keep=True)
                loss = self.backward(acts, y, tb)
                self.adam_step(lr=lr * (0.5 ** (epoch / max(1, epochs - 1))))
                total += float(loss.item()) if steps % 50 == 0 else 0.0
                steps += 1
            history.append(total)
            if log:
                log(f"epoch {epoch}: loss {total:.4g}")
        return history


def features(engine, spectra, model_c):
    """Input features (bf16 [num, FEATURE_STRIDE]) and a0 (FP64 [num])."""
    lib = _bind()
    n = spectra.num
    feat = torch.zeros(max(n, 1), FEATURE_STRIDE, dtype=torch.bfloat16, device=engine.device)
    a0 = torch.zeros(max(n, 1), dtype=torch.float64, device=engine.device)
    check(lib.pg_mlp_features(engine.plan.handle, ctypes.byref(spectra.c), ctypes.byref(model_c),
                              feat.data_ptr(), FEATURE_STRIDE, a0.data_ptr(), engine._stream()),
          "features")
    return feat, a0


def targets_from_fit(fit, a0):
    """(a/a0 - 1, b/a0) for converged forests; mask of usable rows."""
    a = fit["zero_point"]
    b = fit["slope"]
    ok = (fit["status"] == 0) & torch.isfinite(a) & (a0 != 0)
    t = torch.stack([a / a0 - 1.0, b / a0], dim=1).float()
    return t, ok


def predict_start(mlp, feat, a0):
    """Warm start (a, b) per forest, FP64 [num, 2] (the fused tensor-core
    forward pass)."""
    y = mlp.forward_fused(feat).double()
    return torch.stack([a0 * (1.0 + y[:, 0]), a0 * y[:, 1]], dim=1).contiguous()


CHI2_TOL = 1e-7
AB_TOL = 1e-5


def warm_fit(engine, spectra, mlp, warm_max_iter=3, mode=None, chi2_tol=CHI2_TOL,
             ab_tol=AB_TOL):
    """Warm-started fits (the features kernel, then the fused tcgen05
    network), each judged on the GPU by its own certificate
    (Dr16Gpu.fit_warm: the remaining Newton step and the chi2 excess over the
    local quadratic minimum, both bounded per forest); forests the network
    placed too far for ``warm_max_iter`` certified Newton steps are re-fitted
    by the plain fit, in place. Returns (fit dict, start, fallback mask)."""
    model_c, keep = engine._model()
    # features and network as two kernels: the one-kernel form
    # (WarmStartMLP.warm_start) is slower, its feature pass runs on the few
    # warps the tensor-core kernel leaves room for
    feat, a0 = features(engine, spectra, model_c)
    start = predict_start(mlp, feat, a0)
    fit = engine.fit_warm(spectra, start, max_iter=warm_max_iter, chi2_tol=chi2_tol,
                          ab_tol=ab_tol)
    fallback = fit["status"] != 0
    index = torch.nonzero(fallback).flatten().to(torch.int32)
    if index.numel():
        keep_fit = fit["_keep"]
        engine.fit(spectra, mode=mode, index=index, out=fit)
        fit["_keep"] = keep_fit
    del keep
    return fit, start, fallback


def collect_training(engine, spectra):
    """Run the plain Dr16 loop and collect (features, targets) at every
    iteration (the model the network sees changes between iterations)."""
    feats, targs = [], []
    fit = None
    for iteration in range(engine.num_iterations):
        model_c, keep = engine._model()
        feat, a0 = features(engine, spectra, model_c)
        fit = engine.fit(spectra)
        t, ok = targets_from_fit(fit, a0)
        feats.append(feat[ok])
        targs.append(t[ok])
        engine.update_model(spectra, fit, iteration == engine.num_iterations - 1)
        del keep
    return torch.cat(feats), torch.cat(targs), fit


def run_warm(engine, spectra, mlp, warm_max_iter=3, mode=None):
    """The Dr16 loop with learned warm starts (and plain-fit fallback) at
    every iteration. Returns (last fit, per-iteration statistics)."""
    stats = []
    fit = None
    for iteration in range(engine.num_iterations):
        fit, _, fallback = warm_fit(engine, spectra, mlp, warm_max_iter=warm_max_iter, mode=mode)
        engine.update_model(spectra, fit, iteration == engine.num_iterations - 1)
        stats.append({"fallback": int(fallback.sum().item()),
                      "iterations_mean": float(fit["iterations"].float().mean().item())})
    return fit, stats
