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


def test_plugin_loads_through_picca_class_from_string():
    """The plugin loaded the way picca's Config loads an expected-flux class
    (config.py:367-393): ``class_from_string`` with the configured module
    name, the ExpectedFlux subclass check, and the options and defaults the
    module exports, in a separate process with the stand-ins of
    tests/golden/make_golden.py for picca's third-party imports. Needs a picca
    checkout: PICCA_REFERENCE_PY names its ``py`` directory (skipped
    otherwise)."""
    import os
    import subprocess
    import sys
    ref = os.environ.get("PICCA_REFERENCE_PY")
    if not ref or not os.path.isdir(os.path.join(ref, "picca")):
        pytest.skip("PICCA_REFERENCE_PY does not name a picca checkout's py directory")
    here = os.path.dirname(os.path.abspath(__file__))
    script = f"""
import sys
sys.dont_write_bytecode = True
sys.path.insert(0, {os.path.dirname(here)!r})
sys.path.insert(0, {os.path.join(here, 'golden')!r})
import make_golden
make_golden._install_stand_ins()
sys.path.insert(0, {ref!r})
from picca.delta_extraction.utils import class_from_string
from picca.delta_extraction.expected_flux import ExpectedFlux, accepted_options as base_opts
import picca.delta_extraction.expected_fluxes.dr16_expected_flux as ref_mod
cls, defaults, accepted = class_from_string(
    "Dr16ExpectedFlux", "picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux")
assert issubclass(cls, ExpectedFlux), cls.__mro__
assert cls.__module__ == "picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux"
want = set(ref_mod.accepted_options) | set(base_opts)
assert set(accepted) | set(base_opts) == want, (sorted(accepted), sorted(want))
for key, value in ref_mod.defaults.items():
    assert defaults[key] == value, (key, defaults[key], value)
print("loaded", cls.__name__, len(accepted))
"""
    res = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr[-3000:]
    assert "loaded Dr16ExpectedFlux" in res.stdout
