"""Fast metal distortion matrices on the GPU: calc_fast_metal_dmat of
picca_fast_metal_dmat.py (py/picca/bin/picca_fast_metal_dmat.py:30-251) and
picca_fast_metal_xdmat.py (py/picca/bin/picca_fast_metal_xdmat.py:28-215).

The reference approximates a metal matrix from the stacked deltas alone: the
stack's wavelength grid (with the stack weights) stands for every forest, so
the pairs are the n1 n2 pairs of two grids (or of the grid and the quasars'
redshift histogram) rather than pixel pairs of forest pairs. The pair
histograms run in ``pg_fast_metal_dmat`` (``csrc/pg_fastmetal.cu``); this
module prepares the two pixel lists (absorber distances from the fiducial
cosmology, redshift-evolution weights, optional rebinning), and finishes the
matrix on the host from the histograms: the normalised r_par matrix, the
r_trans matrix from the distance-ratio histogram spread over an oversampled
r_trans grid (O(nt^2) work), their Kronecker product and the effective
coordinates.
"""

import ctypes

import numpy as np
import torch

from . import _native
from .pairs import require_cuda

#: pairs whose true |r_par| is below this enter the distance-ratio histogram
#: (py/picca/bin/picca_fast_metal_dmat.py:173-177)
NEAR_R_PAR = 20.0
#: r_trans sub-bins per bin of the bin-migration sum (:184)
OVERSAMPLE = 7


class FastMetalSideC(ctypes.Structure):
    _fields_ = [("r_in", ctypes.c_void_p), ("r_out", ctypes.c_void_p),
                ("z_in", ctypes.c_void_p), ("weight", ctypes.c_void_p), ("num", ctypes.c_int64)]


class FastMetalParamsC(ctypes.Structure):
    _fields_ = [("r_par_min", ctypes.c_double), ("r_par_max", ctypes.c_double),
                ("near_r_par", ctypes.c_double), ("num_bins_r_par", ctypes.c_int32),
                ("num_ratio_bins", ctypes.c_int32), ("signed_r_par", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


SUM_KEYS = ("rp_dmat", "ratio_weights", "ratio_edges", "out_weight", "out_weight_rp",
            "out_weight_z")


class FastMetalSumsC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in SUM_KEYS]


def _bind():
    lib = _native.lib()
    if not getattr(lib, "_fast_metal_bound", False):
        lib.pg_fast_metal_dmat.restype = ctypes.c_int
        lib.pg_fast_metal_dmat.argtypes = [
            ctypes.c_void_p, ctypes.POINTER(FastMetalParamsC), ctypes.POINTER(FastMetalSideC),
            ctypes.POINTER(FastMetalSideC), ctypes.POINTER(FastMetalSumsC), ctypes.c_void_p]
        lib._fast_metal_bound = True
    return lib


def rebin(values, factor):
    """Mean over groups of ``factor`` consecutive entries, the tail dropped
    (py/picca/bin/picca_fast_metal_dmat.py:77-99)."""
    values = np.asarray(values, dtype=np.float64)
    if factor is None:
        return values
    n = values.size // factor
    return values[:n * factor].reshape(n, factor).mean(-1)


def stack_side(log_lambda, weight, lambda_in, lambda_out, alpha_sum, cosmo, rebin_factor=None):
    """A stack's wavelength grid as a pixel list: distances with the true
    absorber (wavelength ``lambda_in``) and the assumed one (``lambda_out``),
    the true redshift, and the weight times (1 + z_in)^(alpha_sum - 2)
    (py/picca/bin/picca_fast_metal_dmat.py:102-146)."""
    log_lambda = rebin(log_lambda, rebin_factor)
    weight = rebin(weight, rebin_factor)
    z_in = 10**log_lambda / lambda_in - 1.0
    z_out = 10**log_lambda / lambda_out - 1.0
    return {"r_in": np.asarray(cosmo.get_r_comov(z_in), dtype=np.float64),
            "r_out": np.asarray(cosmo.get_r_comov(z_out), dtype=np.float64),
            "z_in": z_in, "w": weight * (1 + z_in)**(alpha_sum - 2)}


def quasar_histogram(z_qso, weight_qso, num_bins):
    """Quasars compressed to a redshift histogram: weighted mean redshift and
    summed weight per bin, empty bins dropped
    (py/picca/bin/picca_fast_metal_xdmat.py:506-512)."""
    z_qso = np.asarray(z_qso, dtype=np.float64)
    weight_qso = np.asarray(weight_qso, dtype=np.float64)
    hw, edges = np.histogram(z_qso, bins=num_bins, weights=weight_qso)
    hwz, _ = np.histogram(z_qso, bins=edges, weights=weight_qso * z_qso)
    keep = hw > 0
    return hwz[keep] / hw[keep], hw[keep]


def quasar_side(z_qso, weight_qso, cosmo):
    """Quasars (or their redshift histogram) as a pixel list: the true and
    the assumed distance are the quasar's."""
    r = np.asarray(cosmo.get_r_comov(z_qso), dtype=np.float64)
    return {"r_in": r, "r_out": r, "z_in": np.asarray(z_qso, dtype=np.float64),
            "w": np.asarray(weight_qso, dtype=np.float64)}


class FastMetalEngine:
    """pg_fast_metal_dmat on one CUDA device."""

    def __init__(self, device=None):
        require_cuda()
        self.device = torch.device(device or "cuda")
        with torch.cuda.device(self.device):
            self.plan = _native.Plan()

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def upload(self, side):
        """Pixel list on the device (tensors kept alive by the returned dict)."""
        tensors = {k: torch.from_numpy(np.ascontiguousarray(side[k], dtype=np.float64))
                   .to(self.device) for k in ("r_in", "r_out", "z_in", "w")}
        n = int(tensors["w"].numel())
        c = FastMetalSideC(*[tensors[k].data_ptr() if n else None
                             for k in ("r_in", "r_out", "z_in", "w")], n)
        return {"tensors": tensors, "c": c}

    def alloc_sums(self, num_bins_r_par, num_ratio_bins):
        sizes = {"rp_dmat": num_bins_r_par * num_bins_r_par, "ratio_weights": num_ratio_bins,
                 "ratio_edges": num_ratio_bins + 1, "out_weight": num_bins_r_par,
                 "out_weight_rp": num_bins_r_par, "out_weight_z": num_bins_r_par}
        return {k: torch.empty(v, dtype=torch.float64, device=self.device)
                for k, v in sizes.items()}

    def histograms_device(self, dev1, dev2, r_par_min, r_par_max, num_bins_r_par,
                          num_bins_r_trans, signed, sums=None):
        """Launch the pair histograms (stream-ordered, no host sync)."""
        lib = _bind()
        nr = 4 * (num_bins_r_trans + 1)
        if sums is None:
            sums = self.alloc_sums(num_bins_r_par, nr)
        params = FastMetalParamsC(float(r_par_min), float(r_par_max), NEAR_R_PAR,
                                  int(num_bins_r_par), nr, 1 if signed else 0, 0)
        out = FastMetalSumsC(*[sums[k].data_ptr() for k in SUM_KEYS])
        with torch.cuda.device(self.device):
            _native.check(lib.pg_fast_metal_dmat(
                self.plan.handle, ctypes.byref(params), ctypes.byref(dev1["c"]),
                ctypes.byref(dev2["c"]), ctypes.byref(out), self._stream()),
                "fast metal distortion matrix")
        return sums

    def histograms(self, side1, side2, r_par_min, r_par_max, num_bins_r_par, num_bins_r_trans,
                   signed):
        sums = self.histograms_device(self.upload(side1), self.upload(side2), r_par_min,
                                      r_par_max, num_bins_r_par, num_bins_r_trans, signed)
        out = {k: v.cpu().numpy() for k, v in sums.items()}
        out["rp_dmat"] = out["rp_dmat"].reshape(num_bins_r_par, num_bins_r_par)
        return out


def finish(h, r_trans_max, num_bins_r_par, num_bins_r_trans):
    """Matrix and effective coordinates from the pair histograms
    (py/picca/bin/picca_fast_metal_dmat.py:157-249): columns of the r_par
    matrix normalised, the r_trans matrix from the ratio histogram over
    ``OVERSAMPLE`` sub-bins per r_trans bin (weight proportional to r_trans),
    normalised, their Kronecker product (index rt + nt rp), and r_par / z
    weighted on the output r_par bins, r_trans the area-weighted bin mean."""
    nt = num_bins_r_trans
    rp = np.array(h["rp_dmat"], dtype=np.float64).reshape(num_bins_r_par, num_bins_r_par)
    norm = rp.sum(axis=0)
    rp /= norm + (norm == 0)
    rt_edges = r_trans_max / nt * np.arange(nt + 1)
    ratios = (h["ratio_edges"][1:] + h["ratio_edges"][:-1]) / 2.0
    centres = (rt_edges[:-1] + rt_edges[1:]) / 2.0
    half = (rt_edges[1] - rt_edges[0]) / 2.0
    sub = np.linspace(-half, half * (1 - 2.0 / OVERSAMPLE), OVERSAMPLE)[None, :]
    rt = np.zeros((nt, nt))
    for col, centre in enumerate(centres):
        spread = (centre + sub)[None, :]
        rt[:, col], _ = np.histogram((ratios[:, None] * spread).ravel(), bins=rt_edges,
                                     weights=(h["ratio_weights"][:, None] * spread).ravel())
    norm = rt.sum(axis=0)
    rt /= norm + (norm == 0)
    dmat = np.kron(rp, rt)
    sw = h["out_weight"]
    r_par_1d = h["out_weight_rp"] / (sw + (sw == 0))
    z_1d = h["out_weight_z"] / (sw + (sw == 0))
    lo = np.arange(nt) * r_trans_max / nt
    hi = (1 + np.arange(nt)) * r_trans_max / nt
    r_trans_1d = (2 * (hi**3 - lo**3)) / (3 * (hi**2 - lo**2))
    index = np.arange(num_bins_r_par * nt)
    return dmat, r_par_1d[index // nt], r_trans_1d[index % nt], z_1d[index // nt]


def fast_metal_matrix(side1, side2, r_par_min, r_par_max, r_trans_max, num_bins_r_par,
                      num_bins_r_trans, signed, engine=None):
    """calc_fast_metal_dmat for two pixel lists: (dmat, r_par, r_trans, z)."""
    engine = engine or FastMetalEngine()
    h = engine.histograms(side1, side2, r_par_min, r_par_max, num_bins_r_par, num_bins_r_trans,
                          signed)
    return finish(h, r_trans_max, num_bins_r_par, num_bins_r_trans)


#: the silicon lines kept by --relevant-metals
#: (py/picca/bin/picca_fast_metal_dmat.py:15)
DEFAULT_SI_METALS = ["SiIII(1207)", "SiII(1190)", "SiII(1193)", "SiII(1260)"]


def absorber_pairs(lambda_abs, abs_igm, lambda_abs2=None, abs_igm2=None, relevant=False):
    """(abs1, abs2) pairs of picca_fast_metal_dmat.py:546-595: with no
    second tracer the second list is the first (--abs-igm2 is then ignored),
    and a second tracer pairs every absorber of the first list with every
    one of the second. ``relevant`` keeps LYA x silicon and CIV(eff) x
    CIV(eff) only (:571-575)."""
    if lambda_abs2 is None:
        lambda_abs2, abs_igm2 = lambda_abs, abs_igm
    first = [lambda_abs] + list(abs_igm)
    second = [lambda_abs2] + list(abs_igm2 or [])
    out = []
    for i1, a1 in enumerate(first):
        start = i1 if lambda_abs == lambda_abs2 else 0
        for i2, a2 in enumerate(second[start:]):
            if i1 == 0 and i2 == 0:
                continue
            if relevant and not (a1 == "LYA" and a2 in DEFAULT_SI_METALS) \
                    and not (a1 == "CIV(eff)" and a1 == a2):
                continue
            out.append((a1, a2))
    return out
