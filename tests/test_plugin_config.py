"""Option handling of the Dr16ExpectedFlux drop-in (no GPU needed): the
accepted options and defaults are picca's
(py/picca/delta_extraction/expected_flux.py:14-26,
py/picca/delta_extraction/expected_fluxes/dr16_expected_flux.py:20-36)."""

import configparser

import pytest


def _module():
    return pytest.importorskip(
        "picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux")


def test_accepted_options_and_defaults():
    mod = _module()
    assert set(mod.accepted_options) == {
        "iter out prefix", "num bins variance", "num processors", "out dir", "var lss mod",
        "force stack delta to zero", "limit eta", "limit var lss", "min num qso in fit",
        "num iterations", "order", "use constant weight", "use ivar as weight"}
    assert mod.defaults["num iterations"] == 5
    assert mod.defaults["limit eta"] == (0.5, 1.5)
    assert mod.defaults["limit var lss"] == (0., 0.3)
    assert mod.defaults["min num qso in fit"] == 100
    assert mod.defaults["order"] == 1
    assert mod.defaults["force stack delta to zero"] is True


def test_option_parsing_from_section_proxy():
    mod = _module()
    parser = configparser.ConfigParser()
    parser.read_string("[expected flux]\nlimit eta = (0.4, 1.6)\norder = 0\n"
                       "use ivar as weight = True\nnum iterations = 7\n")
    section = parser["expected flux"]
    assert mod._option(section, "limit eta", tuple) == (0.4, 1.6)
    assert mod._option(section, "order", int) == 0
    assert mod._option(section, "use ivar as weight", bool) is True
    assert mod._option(section, "num iterations", int) == 7
    assert mod._option(section, "min num qso in fit", int) == 100


def test_rejects_unknown_option_and_folder_prefix():
    mod = _module()
    with pytest.raises(mod.ExpectedFluxError):
        mod.Dr16ExpectedFlux({"not an option": "1"}, grid=object())
    with pytest.raises(mod.ExpectedFluxError):
        mod.Dr16ExpectedFlux({"iter out prefix": "a/b"}, grid=object())
