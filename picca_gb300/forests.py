"""Structure-of-arrays view of a set of lines of sight.

The reference keeps one Python object per forest (``Delta``/``QSO``,
``py/picca/data.py``) in a ``{healpix: [objects]}`` dict. The GPU path needs
flat arrays instead: one contiguous pixel stream with per-forest offsets, and
per-forest scalars. :class:`ForestSet` builds that layout once, in the order
the reference visits forests (healpix ascending, then read order,
``py/picca/bin/picca_cf.py:454``), and records for every forest the output
row (rank of its healpix) that its pairs accumulate into.
"""

import numpy as np

PIXEL_FIELDS = ("z", "r_comov", "dist_m", "weights", "delta", "log_lambda")
FOREST_F64 = ("ra", "dec", "x_cart", "y_cart", "z_cart", "cos_dec", "z_qso",
              "obj_r_comov", "obj_dist_m", "obj_weight")
FOREST_I64 = ("thingid", "plate", "fiberid", "healpix", "order")


class ForestSet:
    """Flat arrays for ``num`` lines of sight.

    Pixel arrays (float64): ``z``, ``r_comov``, ``dist_m``, ``weights``,
    ``delta``, ``log_lambda``, indexed through ``pix_offset`` (int64,
    ``num + 1``). Per-forest arrays: positions and redshift (float64), ids
    (int64), ``healpix`` and ``row`` (int32, rank of the healpix among
    ``healpix_list``), ``order`` (int64, the continuum polynomial order of
    the deltas, -1 when unknown). Quasar sets carry ``obj_r_comov``, ``obj_dist_m`` and
    ``obj_weight`` and no pixels.
    """

    def __init__(self, **arrays):
        for key, val in arrays.items():
            setattr(self, key, val)
        self.num = int(len(self.ra))
        if not hasattr(self, "pix_offset"):
            self.pix_offset = np.zeros(self.num + 1, dtype=np.int64)
        for key in PIXEL_FIELDS:
            if not hasattr(self, key):
                setattr(self, key, np.zeros(0))
        for key in FOREST_F64:
            if not hasattr(self, key):
                setattr(self, key, np.zeros(self.num))
        if not hasattr(self, "order"):
            self.order = np.full(self.num, -1, dtype=np.int64)
        for key in FOREST_I64:
            if not hasattr(self, key):
                setattr(self, key, np.zeros(self.num, dtype=np.int64))
        if not hasattr(self, "healpix_list"):
            self.healpix_list = np.unique(self.healpix)
        if not hasattr(self, "row"):
            self.row = np.searchsorted(self.healpix_list, self.healpix).astype(np.int32)

    @property
    def num_pixels(self):
        return int(self.pix_offset[-1])

    @property
    def npix(self):
        return np.diff(self.pix_offset)

    @classmethod
    def from_deltas(cls, data, ang_correlation=False, healpixs=None):
        """Pack ``{healpix: [Delta]}``. With ``ang_correlation`` the r_comov
        and dist_m slots hold 10**log_lambda, as in py/picca/cf.py:186-208."""
        keys = sorted(data) if healpixs is None else list(healpixs)
        deltas = [d for hp in keys for d in data[hp]]
        hp_of = np.array([hp for hp in keys for _ in data[hp]], dtype=np.int64)
        npix = np.array([len(d.z) for d in deltas], dtype=np.int64)
        offset = np.zeros(len(deltas) + 1, dtype=np.int64)
        np.cumsum(npix, out=offset[1:])

        def cat(getter):
            if not deltas:
                return np.zeros(0)
            return np.concatenate([np.asarray(getter(d), dtype=float) for d in deltas])

        if ang_correlation:
            r_comov = cat(lambda d: 10.0**d.log_lambda)
            dist_m = r_comov.copy()
        else:
            r_comov = cat(lambda d: d.r_comov)
            dist_m = cat(lambda d: d.dist_m)
        fiberid = [d.fiberid for d in deltas]
        fiber_is_str = any(isinstance(f, str) for f in fiberid)
        return cls(
            pix_offset=offset,
            z=cat(lambda d: d.z), r_comov=r_comov, dist_m=dist_m,
            weights=cat(lambda d: d.weights), delta=cat(lambda d: d.delta),
            log_lambda=cat(lambda d: d.log_lambda),
            ra=np.array([d.ra for d in deltas], dtype=float),
            dec=np.array([d.dec for d in deltas], dtype=float),
            x_cart=np.array([d.x_cart for d in deltas], dtype=float),
            y_cart=np.array([d.y_cart for d in deltas], dtype=float),
            z_cart=np.array([d.z_cart for d in deltas], dtype=float),
            cos_dec=np.array([d.cos_dec for d in deltas], dtype=float),
            z_qso=np.array([d.z_qso for d in deltas], dtype=float),
            thingid=np.array([d.thingid for d in deltas], dtype=np.int64),
            plate=np.array([d.plate for d in deltas], dtype=np.int64),
            fiberid=np.array([0 if fiber_is_str else f for f in fiberid], dtype=np.int64),
            order=np.array([-1 if getattr(d, "order", None) is None else int(d.order)
                            for d in deltas], dtype=np.int64),
            healpix=hp_of, healpix_list=np.array(keys, dtype=np.int64),
            fiberid_is_str=fiber_is_str,
        )

    @classmethod
    def from_objects(cls, objs, ang_correlation=False):
        """Pack ``{healpix: [QSO]}`` (weights and distances already set)."""
        keys = sorted(objs)
        items = [o for hp in keys for o in objs[hp]]
        hp_of = np.array([hp for hp in keys for _ in objs[hp]], dtype=np.int64)
        if ang_correlation:
            r_comov = np.array([10.0**o.log_lambda for o in items], dtype=float)
            dist_m = r_comov.copy()
        else:
            r_comov = np.array([o.r_comov for o in items], dtype=float)
            dist_m = np.array([o.dist_m for o in items], dtype=float)
        return cls(
            ra=np.array([o.ra for o in items], dtype=float),
            dec=np.array([o.dec for o in items], dtype=float),
            x_cart=np.array([o.x_cart for o in items], dtype=float),
            y_cart=np.array([o.y_cart for o in items], dtype=float),
            z_cart=np.array([o.z_cart for o in items], dtype=float),
            cos_dec=np.array([o.cos_dec for o in items], dtype=float),
            z_qso=np.array([o.z_qso for o in items], dtype=float),
            obj_r_comov=r_comov, obj_dist_m=dist_m,
            obj_weight=np.array([o.weights for o in items], dtype=float),
            thingid=np.array([o.thingid for o in items], dtype=np.int64),
            plate=np.array([o.plate for o in items], dtype=np.int64),
            fiberid=np.array([o.fiberid for o in items], dtype=np.int64),
            healpix=hp_of, healpix_list=np.array(keys, dtype=np.int64),
        )

    def take(self, indices):
        """Forests ``indices`` (sorted), with rows renumbered over their healpix."""
        idx = np.asarray(indices, dtype=np.int64)
        npix = self.npix[idx]
        offset = np.zeros(len(idx) + 1, dtype=np.int64)
        np.cumsum(npix, out=offset[1:])
        starts = self.pix_offset[idx]
        fid = np.repeat(np.arange(len(idx)), npix)
        pix_idx = starts[fid] + (np.arange(offset[-1]) - offset[fid])
        kwargs = {"pix_offset": offset}
        if self.num_pixels:
            for key in PIXEL_FIELDS:
                kwargs[key] = getattr(self, key)[pix_idx]
        for key in FOREST_F64 + FOREST_I64:
            kwargs[key] = getattr(self, key)[idx]
        return ForestSet(**kwargs)

    def subset_rows(self, rows):
        """Forests whose row is in ``rows`` (keeps pixel data contiguous)."""
        rows = np.asarray(rows)
        keep = np.isin(self.row, rows)
        idx = np.where(keep)[0]
        npix = self.npix[idx]
        offset = np.zeros(len(idx) + 1, dtype=np.int64)
        np.cumsum(npix, out=offset[1:])
        pix_idx = (np.concatenate([np.arange(self.pix_offset[i], self.pix_offset[i + 1])
                                   for i in idx]) if len(idx) else np.zeros(0, dtype=np.int64))
        kwargs = {"pix_offset": offset}
        for key in PIXEL_FIELDS:
            kwargs[key] = getattr(self, key)[pix_idx]
        for key in FOREST_F64 + FOREST_I64:
            kwargs[key] = getattr(self, key)[idx]
        kwargs["healpix_list"] = self.healpix_list
        kwargs["row"] = self.row[idx]
        return ForestSet(**kwargs)
