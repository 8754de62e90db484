"""Host-side logic of the newer rows (no GPU): how costly Wick work units
are cut into slices, the absorber pairs of the fast metal script, and
blinded delta files through both readers."""

import os

import numpy as np

from picca_gb300 import constants, io


def test_slice_units_cover_each_unit_once():
    from picca_gb300 import wick
    cost = np.array([10.0, 3.0e5, 4.5e4, 1.0, 8.0e4])
    unit, sl, sls = wick.slice_units(cost)
    for u in range(cost.size):
        mine = np.nonzero(unit == u)[0]
        assert mine.size == sls[mine[0]]
        assert np.array_equal(np.sort(sl[mine]), np.arange(mine.size))
    per = (cost * cost / np.clip(np.ceil(cost * cost / wick.SLICE_TARGET), 1,
                                 wick.MAX_SLICES))[unit]
    assert np.all(np.diff(per) <= 0)  # costliest slices first
    assert sls.max() <= wick.MAX_SLICES


def test_fast_metal_relevant_pairs():
    from picca_gb300 import fast_metal
    metals = ["SiII(1190)", "SiIII(1207)", "CIV(eff)", "SiII(1526)"]
    pairs = fast_metal.absorber_pairs("LYA", metals, relevant=True)
    # LYA with the four DEFAULT_SI_METALS present, and CIV(eff) with itself
    # (py/picca/bin/picca_fast_metal_dmat.py:15, :571-575)
    assert pairs == [("LYA", "SiII(1190)"), ("LYA", "SiIII(1207)"), ("CIV(eff)", "CIV(eff)")]
    assert len(fast_metal.absorber_pairs("LYA", metals)) == 14


def test_blinded_files_read_the_same(tmp_path):
    from picca_gb300 import deltaio
    rng = np.random.default_rng(8)
    grid = 3.5563 + 3e-4 * np.arange(300)
    nf = 12
    lengths = rng.integers(40, 200, nf)
    starts = rng.integers(0, 100, nf)
    index = np.concatenate([np.arange(s, s + n) for s, n in zip(starts, lengths)])
    po = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    n = int(po[-1])
    arrays = {"los_id": np.arange(nf) + 40, "ra": rng.uniform(0, 0.05, nf),
              "dec": rng.uniform(0, 0.05, nf), "z_qso": rng.uniform(2.3, 3.0, nf),
              "healpix": np.zeros(nf, dtype=np.int64), "pix_offset": po,
              "delta": rng.normal(0, 0.3, n), "weights": rng.uniform(0.5, 3.0, n),
              "cont": rng.uniform(1.0, 2.0, n)}
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    for layout in ("ImageHDU", "BinTableHDU"):
        out = tmp_path / layout
        deltaio.write_deltas(str(out), arrays, grid, index, save_format=layout,
                             blinding="desi_y1")
        assert io.read_blinding(str(out / "Delta")) == "desi_y1"
        args = (str(out / "Delta") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9, 2.25, cosmo)
        got = io.read_deltas(*args, no_project=True, native=True)
        want = io.read_deltas(*args, no_project=True, native=False)
        assert got[1] == want[1] == nf
        for hp in want[0]:
            for a, b in zip(got[0][hp], want[0][hp]):
                assert np.array_equal(a.delta, b.delta) and np.array_equal(a.weights, b.weights)
        assert not os.path.exists(out / "Delta" / "delta-1.fits.gz")


def test_per_pixel_chunks_match_one_call():
    from picca_gb300 import deltaio
    rng = np.random.default_rng(3)
    ll = np.sort(rng.uniform(3.55, 3.75, 100_003))
    w = rng.uniform(0.1, 5.0, ll.size)
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    z = 10**ll / 1215.67 - 1.
    for chunk in (999, 4096):  # odd chunk: unaligned chunk starts
        zc = deltaio.per_pixel(lambda a: 10**a / 1215.67 - 1., [ll], threads=4, chunk=chunk)
        assert np.array_equal(zc, z)
        assert np.array_equal(deltaio.per_pixel(cosmo.get_r_comov, [z], 4, chunk),
                              cosmo.get_r_comov(z))
        got = deltaio.per_pixel(lambda a, b: a * ((1 + b) / 3.25)**2.8, [w, z], 4, chunk)
        assert np.array_equal(got, w * ((1 + z) / 3.25)**2.8)


def test_neighbour_groups_cover_every_neighbour():
    """The grouped neighbour search scans, for each healpix row of the
    query set, only the candidate rows of neighbour_groups: every pair of
    objects closer than ang_max must fall in a candidate row pair, and the
    block list must cover every query exactly once (within one row)."""
    import torch  # noqa: F401  (pairs imports torch)
    from picca_gb300 import pairs, synthetic
    fs = synthetic.make_forests(3000, 5, (140.0, 170.0), (-10.0, 20.0), 2.1, 3.5, "uniform")
    qs = synthetic.make_quasars(2500, 6, (140.0, 170.0), (-10.0, 20.0))
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    for other in (fs, qs):
        h1 = pairs.DeviceForests._host_arrays(fs, True)
        h2 = pairs.DeviceForests._host_arrays(other, True)
        g = pairs.neighbour_groups(h1, h2, fs.num, other.num, ang_max, block=64)
        assert g is not None
        row1 = np.asarray(h1["row"])
        start2 = g["start2"]
        grp2 = np.searchsorted(start2, np.arange(other.num), side="right") - 1
        v1 = np.stack([h1["x_cart"], h1["y_cart"], h1["z_cart"]], axis=1)
        v2 = np.stack([h2["x_cart"], h2["y_cart"], h2["z_cart"]], axis=1)
        ang = np.arccos(np.clip(v1 @ v2.T, -1, 1))
        i, j = np.nonzero(ang < ang_max * 1.001)
        # group index of set 1 = rank of its row run
        grp1 = np.searchsorted(np.unique(row1), row1)
        for a, b in zip(grp1[i], grp2[j]):
            lo, hi = g["cand_offsets"][a], g["cand_offsets"][a + 1]
            assert b in g["cand_groups"][lo:hi]
        for a in range(g["num_groups1"]):
            c = g["cand_groups"][g["cand_offsets"][a]:g["cand_offsets"][a + 1]]
            assert np.all(np.diff(c) > 0)
        covered = np.zeros(fs.num, dtype=int)
        for grp, first, end in zip(g["block_group"], g["block_first"], g["block_end"]):
            assert 0 < end - first <= 64
            covered[first:end] += 1
            assert np.all(grp1[first:end] == grp)
        assert np.all(covered == 1)


def test_tuning_cache_round_trip(tmp_path, monkeypatch):
    """The launch-shape cache: JSON round trip, a damaged file reads as
    empty, and the environment variable moves the cache."""
    from picca_gb300 import autotune
    path = str(tmp_path / "sub" / "tuning.json")
    table = {"GB300|cf|bins=2500|grid=log|mode=1": {
        "choice": [16, 0], "sample_items": 2000,
        "alternatives": [{"warps": 0, "ctas_per_sm": 0, "ms": 80.0},
                         {"warps": 16, "ctas_per_sm": 0, "ms": 79.0}]}}
    autotune._save(path, table)
    assert autotune._load(path) == table
    assert not [f for f in os.listdir(tmp_path / "sub") if ".tmp" in f]
    with open(path, "w") as fh:
        fh.write("{not json")
    assert autotune._load(path) == {}
    assert autotune._load(str(tmp_path / "missing.json")) == {}
    monkeypatch.setenv("PICCA_GB300_TUNE_CACHE", path)
    assert autotune.default_cache_path() == path
    monkeypatch.delenv("PICCA_GB300_TUNE_CACHE")
    assert autotune.default_cache_path().endswith(os.path.join("picca_gb300", "pair_tuning.json"))
