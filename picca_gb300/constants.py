"""Physical constants, absorber wavelengths and the fiducial cosmology.

Mirrors ``py/picca/constants.py``: the same public names (``Cosmo``,
``SPEED_LIGHT``, ``SMALL_ANGLE_CUT_OFF``, ``ABSORBER_IGM``) and the same
arithmetic, so that comoving distances computed here are bit-identical to the
reference's for the same inputs (the correlation bins depend on them).
"""

import numpy as np
from scipy import interpolate
from scipy.constants import speed_of_light as _speed_light

# 2 arcsec in radians (py/picca/constants.py:16)
SMALL_ANGLE_CUT_OFF = 2. / 3600. * np.pi / 180.

# km/s (py/picca/constants.py:18)
SPEED_LIGHT = _speed_light / 1000.


class Cosmo:
    """Flat/curved LambdaCDM distance tables in Mpc/h.

    Follows ``Cosmo.__init__`` (py/picca/constants.py:159-233): H0 = 100, a
    10,000-step table on z in [0, 10) with step 1e-3, comoving distance from a
    cumulative trapezoid of c/H(z), and linear ``interp1d`` lookups. The
    CAMB-template branch (py/picca/constants.py:235-240) is not supported.
    """

    def __init__(self, Om, Ok=0., Or=0., wl=-1., blinding=False,
                 verbose=True, template=None):
        if template is not None:
            raise NotImplementedError(
                "distance templates need CAMB, which this package does not use")
        h0 = 100.0
        if verbose and blinding == "none":
            print("ATTENTION: Analysis is not blinded!", flush=True)
            print(f"Om={Om}, Or={Or}, wl={wl}", flush=True)

        omega_lambda = 1. - Ok - Om - Or
        num_bins = 10000
        z_max = 10.
        delta_z = z_max / num_bins
        z = np.arange(num_bins, dtype=float) * delta_z
        hubble = h0 * np.sqrt(omega_lambda * (1. + z)**(3. * (1. + wl)) +
                              Ok * (1. + z)**2 + Om * (1. + z)**3 +
                              Or * (1. + z)**4)

        # the recurrence is sequential; keep the reference's exact operation
        # order so every table entry matches bit for bit
        inv_h = 1. / hubble
        r_comov = np.zeros(num_bins)
        acc = 0.0
        for index in range(1, num_bins):
            acc = (SPEED_LIGHT * (inv_h[index - 1] + inv_h[index]) / 2. * delta_z
                   + acc)
            r_comov[index] = acc

        self.get_r_comov = interpolate.interp1d(z, r_comov)
        if Ok == 0.:
            dist_m = r_comov
        elif Ok < 0.:
            dist_m = (np.sin(h0 * np.sqrt(-Ok) / SPEED_LIGHT * r_comov) /
                      (h0 * np.sqrt(-Ok) / SPEED_LIGHT))
        else:
            dist_m = (np.sinh(h0 * np.sqrt(Ok) / SPEED_LIGHT * r_comov) /
                      (h0 * np.sqrt(Ok) / SPEED_LIGHT))
        self.get_hubble = interpolate.interp1d(z, hubble)
        self.distance_to_redshift = interpolate.interp1d(r_comov, z)
        self.get_dist_hubble = interpolate.interp1d(z, SPEED_LIGHT / hubble)
        self.get_dist_m = interpolate.interp1d(z, dist_m)
        dist_v = np.power(z * self.get_dist_m(z)**2 * self.get_dist_hubble(z),
                          1. / 3.)
        self.get_dist_v = interpolate.interp1d(z, dist_v)


# Rest-frame wavelengths of IGM absorbers in Angstrom. The CLIs select the
# tracer by name (--lambda-abs), so the names and values are the same as in
# py/picca/constants.py:243-312.
ABSORBER_IGM = {
    "Halpha": 6562.8,
    "Hbeta": 4862.68,
    "MgI(2853)": 2852.96,
    "MgII(2804)": 2803.5324,
    "MgII(eff)": 2798.75,
    "MgII(2796)": 2796.3511,
    "FeII(2600)": 2600.1724835,
    "FeII(2587)": 2586.6495659,
    "MnII(2577)": 2576.877,
    "FeII(2383)": 2382.7641781,
    "FeII(2374)": 2374.4603294,
    "FeII(2344)": 2344.2129601,
    "CIII(1908)": 1908.73,
    "AlIII(1863)": 1862.79113,
    "AlIII(1855)": 1854.71829,
    "AlII(1671)": 1670.7886,
    "FeII(1608)": 1608.4511,
    "CIV(1551)": 1550.77845,
    "CIV(eff)": 1549.06,
    "CIV(1548)": 1548.2049,
    "SiII(1527)": 1526.70698,
    "NiII(1455)": 1454.842,
    "SiIV(1403)": 1402.77291,
    "SiIV(eff)": 1396.76,
    "SiIV(1394)": 1393.76018,
    "NiII(1370)": 1370.132,
    "CII(1335)": 1334.5323,
    "NiII(1317)": 1317.217,
    "SiII(1304)": 1304.3702,
    "OI(1302)": 1302.1685,
    "SiII(1260)": 1260.4221,
    "SII(1254)": 1253.811,
    "SII(1251)": 1250.584,
    "NV(1243)": 1242.804,
    "NV(1239)": 1238.821,
    "LYA": 1215.67,
    "SiIII(1207)": 1206.500,
    "NI(1200)": 1200.,
    "SiII(1193)": 1193.2897,
    "SiII(1190)": 1190.4158,
    "PII(1153)": 1152.818,
    "FeII(1145)": 1144.9379,
    "FeII(1143)": 1143.2260,
    "NI(1134)": 1134.4149,
    "FeII(1125)": 1125.4477,
    "FeIII(1123)": 1122.526,
    "FeII(1097)": 1096.8769,
    "NII(1084)": 1083.990,
    "FeII(1082)": 1081.8748,
    "FeII(1063)": 1063.002,
    "OI(1039)": 1039.230,
    "OVI(1038)": 1037.613,
    "CII(1037)": 1036.7909,
    "OVI(1032)": 1031.912,
    "LYB": 1025.72,
    "SiII(1021)": 1020.6989,
    "SIII(1013)": 1012.502,
    "SiII(990)": 989.8731,
    "OI(989)": 988.7,
    "CIII(977)": 977.020,
    "LY3": 972.537,
    "LY4": 949.7431,
    "LY5": 937.8035,
    "LY6": 930.7483,
    "LY7": 926.2257,
    "LY8": 923.1504,
    "LY9": 920.9631,
    "LY10": 919.3514,
}
