"""The metal distortion-matrix oracle (oracle/metal_dmat.py) against
picca's golden metal_dmat.fits.gz (py/picca/tests/test_3_cor.py:351-382:
SiIII(1207), rp 0-60, rt 60, 15x15 bins, rejection 0.99, one process;
absorber pairs LYA_SiIII(1207) with the swapped pass and
SiIII(1207)_SiIII(1207))."""

import os

import numpy as np

from conftest import golden
from oracle import metal_dmat as omd
from test_oracle_golden import compare_like_reference


def prepare_metal(picca_inputs):
    from picca_gb300 import constants, io, utils
    from picca_gb300.forests import ForestSet
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    data, _, z_min, _ = io.read_deltas(
        os.path.join(picca_inputs, "Delta_LYA") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9,
        2.25, cosmo, delta_attributes=os.path.join(picca_inputs, "delta_attributes.fits.gz"))
    fs = ForestSet.from_deltas(data)
    params = omd.MetalParams(0., 60., 60., 15, 15, z_ref=2.25,
                             alpha_abs={"LYA": 2.9, "SiIII(1207)": 1.0})
    ang_max = utils.compute_ang_max(cosmo, 60., z_min)
    return fs, cosmo, params, ang_max


def test_absorber_pairs():
    assert omd.absorber_pairs("LYA", ["SiIII(1207)"]) == [
        ("LYA", "SiIII(1207)"), ("SiIII(1207)", "SiIII(1207)")]
    assert omd.absorber_pairs("LYA", ["A", "B"]) == [
        ("LYA", "A"), ("LYA", "B"), ("A", "A"), ("A", "B"), ("B", "B")]


def test_pipeline_matches_golden_metal_dmat(picca_inputs):
    fs, cosmo, params, ang_max = prepare_metal(picca_inputs)
    got = omd.pipeline(fs, cosmo, params, ang_max, reject=0.99, abs_igm=["SiIII(1207)"])
    want = golden("cor_metal_dmat.npz")
    names = [str(x) for x in want["ABS_IGM"]]
    assert list(got) == names
    for k, name in enumerate(names):
        g = got[name]
        assert g["NPALL"] == int(want["NPALL"][k]) and g["NPUSED"] == int(want["NPUSED"][k])
        compare_like_reference({key: g[key] for key in ("RP", "RT", "Z", "DM", "WDM")},
                               {key: want[f"{key}_{name}"] for key in ("RP", "RT", "Z", "DM",
                                                                        "WDM")},
                               names=("RP", "RT", "Z", "DM", "WDM"))


def test_xpipeline_matches_golden_metal_xdmat(picca_inputs):
    from picca_gb300 import constants, io, utils
    from picca_gb300.forests import ForestSet
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    data, _, z_min, _ = io.read_deltas(
        os.path.join(picca_inputs, "Delta_LYA") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9,
        2.25, cosmo, delta_attributes=os.path.join(picca_inputs, "delta_attributes.fits.gz"))
    objs, z_min2 = io.read_objects(os.path.join(picca_inputs, "cat.fits"), 16, 0, 10, 1.0, 2.25,
                                   cosmo)
    fs, qs = ForestSet.from_deltas(data), ForestSet.from_objects(objs)
    params = omd.MetalParams(-60., 60., 60., 30, 15, z_ref=2.25, x_correlation=True,
                             alpha_abs={"LYA": 2.9, "SiIII(1207)": 1.0})
    ang_max = utils.compute_ang_max(cosmo, 60., z_min, z_min2)
    got = omd.xpipeline(fs, qs, cosmo, params, ang_max, reject=0.99, abs_igm=["SiIII(1207)"])
    want = golden("cor_metal_xdmat.npz")
    assert [str(x) for x in want["ABS_IGM"]] == ["SiIII(1207)"]
    g = got["SiIII(1207)"]
    assert g["NPALL"] == int(want["NPALL"][0]) and g["NPUSED"] == int(want["NPUSED"][0])
    compare_like_reference({k: g[k] for k in ("RP", "RT", "Z", "DM", "WDM")},
                           {k: want[f"{k}_QSO_SiIII(1207)"] for k in ("RP", "RT", "Z", "DM",
                                                                       "WDM")},
                           names=("RP", "RT", "Z", "DM", "WDM"))


def test_pipeline_matches_golden_metal_dmat_cross(picca_inputs):
    """py/picca/tests/test_3_cor.py:526-557: the same delta field twice,
    SiIII(1207) on both, r_par unfolded, same-half-plate veto."""
    from picca_gb300 import constants, io, utils
    from picca_gb300.forests import ForestSet
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    sets = []
    for _ in range(2):
        data, _, z_min, _ = io.read_deltas(
            os.path.join(picca_inputs, "Delta_LYA") + "/", 16, constants.ABSORBER_IGM["LYA"],
            2.9, 2.25, cosmo,
            delta_attributes=os.path.join(picca_inputs, "delta_attributes.fits.gz"))
        sets.append(ForestSet.from_deltas(data))
    params = omd.MetalParams(-60., 60., 60., 30, 15, x_correlation=True,
                             remove_same_half_plate_close_pairs=True, z_ref=2.25,
                             alpha_abs={"LYA": 2.9, "SiIII(1207)": 1.0})
    ang_max = utils.compute_ang_max(cosmo, 60., z_min, z_min)
    got = omd.pipeline(sets[0], cosmo, params, ang_max, reject=0.99, abs_igm=["SiIII(1207)"],
                       fs2=sets[1])
    want = golden("cor_metal_dmat_cross.npz")
    for k, name in enumerate(str(x) for x in want["ABS_IGM"]):
        g = got[name]
        assert g["NPALL"] == int(want["NPALL"][k]) and g["NPUSED"] == int(want["NPUSED"][k])
        compare_like_reference({key: g[key] for key in ("RP", "RT", "Z", "DM", "WDM")},
                               {key: want[f"{key}_{name}"] for key in ("RP", "RT", "Z", "DM",
                                                                        "WDM")},
                               names=("RP", "RT", "Z", "DM", "WDM"))
