"""Native reading of delta files (``pg_read_delta_file``, ``pg_project_deltas``).

``io.read_deltas`` (py/picca/io.py:383-512) reads every file with fitsio,
builds one ``Delta`` per line of sight (py/picca/data.py:376-620) and then,
forest by forest, computes z, the comoving distances, the redshift evolution
of the weights and the projection. Here each file's bytes go to the C parser
(files in parallel threads; gunzip and the parser release the GIL), the
per-pixel quantities are computed once over the concatenated pixel arrays
(the same elementwise NumPy expressions), the projection runs in the native
library with NumPy's summation order, and the ``Delta`` objects are views
into those arrays. The result is bit-identical to the per-object path
(``tests/test_deltaio.py``).
"""

import ctypes
import os
import zlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _native
from .data import Delta

_P = ctypes.POINTER


class DeltaArraysC(ctypes.Structure):
    _fields_ = [("num_los", ctypes.c_int64), ("num_pixels", ctypes.c_int64),
                ("format", ctypes.c_int32), ("wave_is_lambda", ctypes.c_int32)] + [
        (k, ctypes.c_void_p) for k in ("los_id", "plate", "mjd", "fiberid", "ra", "dec", "z_qso",
                                       "pix_offset", "wave", "delta", "weights", "cont")]


LOS_KEYS = {"los_id": np.int64, "plate": np.int64, "mjd": np.int64, "fiberid": np.int64,
            "ra": np.float64, "dec": np.float64, "z_qso": np.float64}
PIX_KEYS = ("wave", "delta", "weights", "cont")


def _bind():
    lib = _native.lib()
    if not getattr(lib, "_deltaio_bound", False):
        lib.pg_read_delta_file.restype = ctypes.c_int
        lib.pg_read_delta_file.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                                           ctypes.c_double, _P(DeltaArraysC)]
        lib.pg_project_deltas.restype = ctypes.c_int
        lib.pg_project_deltas.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int32]
        lib._deltaio_bound = True
    return lib


def gunzip(raw):
    """Every gzip member of ``raw`` inflated (zlib checks each member's CRC
    in C, without the GIL)."""
    parts = []
    while raw[:2] == b"\x1f\x8b":
        d = zlib.decompressobj(wbits=31)
        parts.append(d.decompress(raw))
        parts.append(d.flush())
        raw = d.unused_data
    return b"".join(parts)


def file_bytes(path):
    """A delta file's bytes, gunzipped when they carry the gzip magic."""
    with open(path, "rb") as handle:
        raw = handle.read()
    return gunzip(raw) if raw[:2] == b"\x1f\x8b" else raw


def read_file(path, z_min_qso=0.0, z_max_qso=10.0, rebin_factor=None):
    """One delta file as arrays: per line of sight (los_id, plate, mjd,
    fiberid, ra, dec, z_qso, pix_offset) and per pixel (log_lambda, delta,
    weights, cont). With ``rebin_factor`` the forests are rebinned as
    py/picca/io.py:362-376 does (``rebin_arrays``); ``cont`` keeps the
    original pixels, at ``cont_offset``."""
    lib = _bind()
    raw = file_bytes(path)
    buf = np.frombuffer(raw, dtype=np.uint8)
    out = DeltaArraysC()
    _native.check(lib.pg_read_delta_file(buf.ctypes.data, buf.size, float(z_min_qso),
                                         float(z_max_qso), ctypes.byref(out)),
                  f"delta file {path}")
    nlos, npix = int(out.num_los), int(out.num_pixels)
    arrays = {k: np.zeros(max(nlos, 1), dtype=t) for k, t in LOS_KEYS.items()}
    arrays["pix_offset"] = np.zeros(nlos + 1, dtype=np.int64)
    for k in PIX_KEYS:
        arrays[k] = np.zeros(max(npix, 1), dtype=np.float64)
    for k, v in arrays.items():
        setattr(out, k, v.ctypes.data)
    _native.check(lib.pg_read_delta_file(buf.ctypes.data, buf.size, float(z_min_qso),
                                         float(z_max_qso), ctypes.byref(out)),
                  f"delta file {path}")
    for k in LOS_KEYS:
        arrays[k] = arrays[k][:nlos]
    for k in PIX_KEYS:
        arrays[k] = arrays[k][:npix]
    arrays["log_lambda"] = np.log10(arrays["wave"]) if out.wave_is_lambda else arrays["wave"]
    arrays["image"] = bool(out.format)
    if rebin_factor is not None:
        from . import fitsio_lite
        headers = fitsio_lite.hdu_headers(raw)
        card = headers[1]
        if out.format:
            card = next(h for h in headers if str(h.get("EXTNAME", "")).strip() == "LAMBDA")
        if card["WAVE_SOLUTION"] != "lin":
            raise ValueError("Delta rebinning only implemented for linear lambda bins")
        arrays["cont_offset"] = arrays["pix_offset"]
        (arrays["pix_offset"], arrays["log_lambda"], arrays["delta"],
         arrays["weights"]) = rebin_arrays(arrays["pix_offset"], arrays["log_lambda"],
                                           arrays["delta"], arrays["weights"], rebin_factor,
                                           card["DELTA_LAMBDA"])
    return arrays


def rebin_arrays(pix_offset, log_lambda, delta, weights, factor, dwave):
    """Delta.rebin (py/picca/data.py:657-686) of every forest at once: the
    wavelength bins of each forest start half a pixel below its bluest pixel
    and are ``factor`` pixels wide; a pixel goes to the bin that
    searchsorted(edges, wave) names, bins 1 .. num_bins - 1 are kept, and
    those with weight are returned (weighted mean delta, summed weight, bin
    centre). Every expression is the per-forest one evaluated elementwise,
    and the bin sums are one bincount over all forests, which adds each
    bin's pixels in the same order as the per-forest bincount: the result
    is bit-identical to rebinning the forests one by one."""
    po = np.asarray(pix_offset, dtype=np.int64)
    n = np.diff(po)
    nf = n.size
    if nf == 0:
        return po, log_lambda, delta, weights
    if np.any(n == 0):
        raise ValueError("zero-size array to reduction operation minimum which has no identity")
    wave = 10**log_lambda
    first, last = po[:-1], po[1:] - 1
    start = np.minimum.reduceat(wave, first) - dwave / 2
    num_bins = np.ceil(((wave[last] - wave[first]) / dwave + 1) / factor)
    nb = num_bins.astype(np.int64)
    eo = np.concatenate([[0], np.cumsum(nb)])
    k = (np.arange(eo[-1]) - np.repeat(eo[:-1], nb)).astype(np.float64)
    edges = k * dwave * factor + np.repeat(start, nb)
    # searchsorted(edges, wave) per forest: the number of edges below each
    # pixel, from a guess corrected against the edges themselves
    fpix = np.repeat(np.arange(nf), n)
    base, top = eo[fpix], nb[fpix]
    idx = np.clip(np.floor((wave - start[fpix]) / (dwave * factor)).astype(np.int64) + 1, 0, top)
    for _ in range(64):
        down = (idx > 0) & (edges[base + np.maximum(idx - 1, 0)] >= wave)
        up = (idx < top) & (edges[base + np.minimum(idx, top - 1)] < wave)
        if not (down.any() or up.any()):
            break
        idx += up.astype(np.int64) - down.astype(np.int64)
    else:
        raise RuntimeError("rebinning: bin search did not settle")
    seg = np.concatenate([[0], np.cumsum(nb + 1)])
    gid = seg[fpix] + idx
    binned_delta = np.bincount(gid, weights=delta * weights, minlength=seg[-1])
    binned_weight = np.bincount(gid, weights=weights, minlength=seg[-1])
    # bins 1 .. nb-1 of each forest, and the centres of those bins
    local = np.arange(seg[-1]) - np.repeat(seg[:-1], nb + 1)
    owner = np.repeat(np.arange(nf), nb + 1)
    inner = (local >= 1) & (local <= nb[owner] - 1)
    binned_delta, binned_weight = binned_delta[inner], binned_weight[inner]
    right = eo[owner[inner]] + local[inner]
    new_wave = (edges[right] + edges[right - 1]) / 2
    mask = binned_weight != 0
    binned_delta[mask] /= binned_weight[mask]
    counts = np.bincount(owner[inner][mask], minlength=nf)
    new_po = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return new_po, np.log10(new_wave[mask]), binned_delta[mask], binned_weight[mask]


def project(pix_offset, log_lambda, weights, delta, order, threads=None):
    """Delta.project of every line of sight, in place (native, NumPy's
    summation order)."""
    lib = _bind()
    num = int(len(pix_offset) - 1)
    order = np.ascontiguousarray(order, dtype=np.int32)
    threads = threads or min(32, os.cpu_count() or 1)
    _native.check(lib.pg_project_deltas(num, pix_offset.ctypes.data, log_lambda.ctypes.data,
                                        weights.ctypes.data, delta.ctypes.data, order.ctypes.data,
                                        int(threads)), "delta projection")


def per_pixel(func, arrays, threads=None, chunk=1 << 18):
    """``func(*arrays)`` for an elementwise ``func`` of equal-length 1-D
    arrays, evaluated on contiguous chunks in a thread pool (NumPy ufuncs and
    ``np.interp`` release the GIL). Elementwise means chunking changes no
    value: the result equals the one-call result bit for bit."""
    n = len(arrays[0])
    threads = threads or min(16, os.cpu_count() or 1)
    if n <= chunk or threads == 1:
        return np.asarray(func(*arrays), dtype=np.float64)
    out = np.empty(n, dtype=np.float64)
    edges = list(range(0, n, chunk)) + [n]

    def run(k):
        sl = slice(edges[k], edges[k + 1])
        out[sl] = func(*(a[sl] for a in arrays))

    with ThreadPoolExecutor(threads) as pool:
        list(pool.map(run, range(len(edges) - 1)))
    return out


def read_files(files, z_min_qso=0.0, z_max_qso=10.0, max_num_spec=None, threads=None,
               rebin_factor=None):
    """The files' arrays concatenated in file order (reading stops after the
    file that passes max_num_spec lines of sight, as io.read_deltas does)."""
    threads = threads or min(16, os.cpu_count() or 1)
    parts = []
    num = 0
    with ThreadPoolExecutor(threads) as pool:
        # without a cap every file is read: one queue keeps all threads busy;
        # with one, files go in waves so that reading stops near the cap
        step = len(files) if max_num_spec is None else max(threads, 1)
        for i in range(0, len(files), step):
            for part in pool.map(lambda f: read_file(f, z_min_qso, z_max_qso, rebin_factor),
                                 files[i:i + step]):
                parts.append(part)
                num += len(part["ra"])
                if max_num_spec is not None and num > max_num_spec:
                    break
            if max_num_spec is not None and num > max_num_spec:
                break
    out = {}
    for k in list(LOS_KEYS) + ["log_lambda", "delta", "weights", "cont"]:
        out[k] = (np.concatenate([p[k] for p in parts]) if parts
                  else np.zeros(0, dtype=LOS_KEYS.get(k, np.float64)))
    counts = np.concatenate([np.diff(p["pix_offset"]) for p in parts]) if parts else \
        np.zeros(0, dtype=np.int64)
    # cont keeps the pixels as read when the forests were rebinned
    cont_key = "cont_offset" if rebin_factor is not None else "pix_offset"
    cont_counts = np.concatenate([np.diff(p[cont_key]) for p in parts]) if parts else \
        np.zeros(0, dtype=np.int64)
    if max_num_spec is not None and len(counts) > max_num_spec:
        counts = counts[:max_num_spec]
        cont_counts = cont_counts[:max_num_spec]
        for k in LOS_KEYS:
            out[k] = out[k][:max_num_spec]
        npix = int(counts.sum())
        for k in ("log_lambda", "delta", "weights"):
            out[k] = out[k][:npix]
        out["cont"] = out["cont"][:int(cont_counts.sum())]
    out["pix_offset"] = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    if rebin_factor is not None:
        out["cont_offset"] = np.concatenate([[0], np.cumsum(cont_counts)]).astype(np.int64)
    return out


def make_deltas(arrays, order):
    """Delta objects whose pixel arrays are views into ``arrays``. The
    per-object trigonometry of QSO.__init__ (py/picca/data.py:60-104) is
    evaluated once over all lines of sight (the same NumPy expressions,
    elementwise), and the objects are filled without calling __init__."""
    po = arrays["pix_offset"]
    num = len(po) - 1
    ra, dec = arrays["ra"][:num], arrays["dec"][:num]
    cos_ra, sin_ra = np.cos(ra), np.sin(ra)
    cos_dec, sin_dec = np.cos(dec), np.sin(dec)
    x_cart, y_cart = cos_ra * cos_dec, sin_ra * cos_dec
    pix = [(k, arrays[k]) for k in ("z", "r_comov", "dist_m") if k in arrays]
    pix += [(k, arrays[k]) for k in ("weights", "log_lambda", "delta")]
    # Python scalars and offsets as lists: one conversion per array instead
    # of one NumPy scalar access per line of sight
    bounds = po.tolist()
    cont, cont_bounds = arrays["cont"], arrays.get("cont_offset", po).tolist()
    ra_l, dec_l, z_qso_l = ra.tolist(), dec.tolist(), arrays["z_qso"][:num].tolist()
    plate_l, mjd_l = arrays["plate"][:num].tolist(), arrays["mjd"][:num].tolist()
    fiber_l, los_l = arrays["fiberid"][:num].tolist(), arrays["los_id"][:num].tolist()
    deltas = []
    for f in range(num):
        lo, hi = bounds[f], bounds[f + 1]
        los_id = los_l[f]
        d = Delta.__new__(Delta)
        fields = {
            "ra": ra_l[f], "dec": dec_l[f], "plate": plate_l[f],
            "mjd": mjd_l[f], "fiberid": fiber_l[f],
            "x_cart": x_cart[f], "y_cart": y_cart[f], "z_cart": sin_dec[f],
            "cos_dec": cos_dec[f], "z_qso": z_qso_l[f], "los_id": los_id,
            "thingid": los_id, "weight": None, "order": order, "ivar": None,
            "exposures_diff": None, "mean_snr": None, "mean_reso": None, "mean_z": None,
            "z": None, "r_comov": None, "dist_m": None, "neighbours": None, "fname": None}
        for key, values in pix:
            fields[key] = values[lo:hi]
        fields["cont"] = cont[cont_bounds[f]:cont_bounds[f + 1]]
        d.__dict__.update(fields)
        deltas.append(d)
    return deltas


def pixel_step_records(grid, wave_solution):
    """Header records of the pixel step for the two delta layouts.

    The image layout rounds the step to two decimals
    (py/picca/delta_extraction/data.py:97-108); the table layout writes it
    unrounded (Forest.get_header,
    py/picca/delta_extraction/astronomical_objects/forest.py:580-601), and
    the rebinning of the reader takes it from there. Returns
    (image records, table records)."""
    grid = np.asarray(grid, dtype=np.float64)
    if wave_solution == "log":
        name, value = "DELTA_LOG_LAMBDA", grid[1] - grid[0]
    elif wave_solution == "lin":
        name, value = "DELTA_LAMBDA", 10**grid[1] - 10**grid[0]
    else:
        raise ValueError(f"Invalid wave_solution {wave_solution}; expected 'lin' or 'log'")
    return [{"name": name, "value": round(float(value), 2)}], [{"name": name, "value": float(value)}]


def write_deltas(out_dir, arrays, log_lambda_grid, grid_index, save_format="ImageHDU",
                 wave_solution="log", blinding="none", flux_units="10**-17 erg/(s cm2 Angstrom)"):
    """Delta files of delta_extraction (py/picca/delta_extraction/data.py:62-265):
    one ``delta-{healpix}.fits.gz`` per healpix under ``out_dir/Delta``.

    ``arrays``: per line of sight ``los_id``, ``ra``, ``dec``, ``z_qso``,
    ``healpix`` (and optionally ``mean_snr``), ``pix_offset``, and per pixel
    ``delta``, ``weights``, ``cont``; ``grid_index`` places each pixel on
    ``log_lambda_grid``. ``ImageHDU``: LAMBDA, METADATA (LOS_ID, RA, DEC, Z,
    MEANSNR; BLINDING), DELTA (DELTA_BLIND when blinded), WEIGHT and CONT
    images over the grid, NaN outside each forest. ``BinTableHDU``: one table
    per line of sight (LAMBDA or LOGLAM, DELTA, WEIGHT, CONT; header LOS_ID,
    RA, DEC, Z, MEANSNR, BLINDING, WAVE_SOLUTION and the pixel step, as
    Forest.get_header writes them,
    py/picca/delta_extraction/astronomical_objects/forest.py:551-610).
    Returns the paths written."""
    from . import fitsio_lite
    os.makedirs(os.path.join(out_dir, "Delta"), exist_ok=True)
    po = np.asarray(arrays["pix_offset"], dtype=np.int64)
    healpix = np.asarray(arrays["healpix"], dtype=np.int64)
    grid = np.asarray(log_lambda_grid, dtype=np.float64)
    index = np.asarray(grid_index, dtype=np.int64)
    mean_snr = np.asarray(arrays.get("mean_snr", np.zeros(len(healpix))), dtype=np.float64)
    delta_name = "DELTA" if blinding == "none" else "DELTA_BLIND"
    step_image, step_table = pixel_step_records(grid, wave_solution)
    paths = []
    for hp in np.unique(healpix):
        members = np.nonzero(healpix == hp)[0]
        path = os.path.join(out_dir, "Delta", f"delta-{int(hp)}.fits.gz")
        if save_format == "ImageHDU":
            shape = (members.size, grid.size)
            images = {k: np.full(shape, np.nan) for k in ("delta", "weights", "cont")}
            for row, f in enumerate(members):
                sl = slice(po[f], po[f + 1])
                for k in images:
                    images[k][row, index[sl]] = arrays[k][sl]
            meta = {"columns": [np.asarray(arrays["los_id"])[members].astype(np.int64),
                                np.asarray(arrays["ra"])[members],
                                np.asarray(arrays["dec"])[members],
                                np.asarray(arrays["z_qso"])[members], mean_snr[members]],
                    "names": ["LOS_ID", "RA", "DEC", "Z", "MEANSNR"],
                    "header": [{"name": "BLINDING", "value": blinding}],
                    "extname": "METADATA"}
            fitsio_lite.write_hdus(path, [
                ("image", "LAMBDA", 10**grid,
                 [{"name": "BUNIT", "value": "Angstrom"},
                  {"name": "WAVE_SOLUTION", "value": wave_solution}] + step_image),
                ("table", meta),
                ("image", delta_name, images["delta"], [{"name": "BUNIT", "value": ""}]),
                ("image", "WEIGHT", images["weights"], []),
                ("image", "CONT", images["cont"], [{"name": "BUNIT", "value": flux_units}])])
        elif save_format == "BinTableHDU":
            tables = []
            for f in members:
                sl = slice(po[f], po[f + 1])
                wave = 10**grid[index[sl]] if wave_solution == "lin" else grid[index[sl]]
                tables.append({
                    "columns": [wave, arrays["delta"][sl], arrays["weights"][sl],
                                arrays["cont"][sl]],
                    "names": ["LAMBDA" if wave_solution == "lin" else "LOGLAM", delta_name,
                              "WEIGHT", "CONT"],
                    "extname": str(int(arrays["los_id"][f])),
                    "header": [{"name": "LOS_ID", "value": int(arrays["los_id"][f])},
                               {"name": "RA", "value": float(arrays["ra"][f])},
                               {"name": "DEC", "value": float(arrays["dec"][f])},
                               {"name": "Z", "value": float(arrays["z_qso"][f])},
                               {"name": "MEANSNR", "value": float(mean_snr[f])},
                               {"name": "BLINDING", "value": blinding},
                               {"name": "WAVE_SOLUTION", "value": wave_solution}] + step_table})
            fitsio_lite.write_fits(path, tables)
        else:
            raise ValueError(f"Invalid format {save_format}; expected ImageHDU or BinTableHDU")
        paths.append(path)
    return paths
