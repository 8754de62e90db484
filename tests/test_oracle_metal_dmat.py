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
