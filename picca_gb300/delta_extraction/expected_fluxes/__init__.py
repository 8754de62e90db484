"""Expected-flux classes: ``dr16_expected_flux.Dr16ExpectedFlux``."""
