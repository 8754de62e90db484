"""HEALPix pixel index in the RING scheme.

picca groups forests into healpix subsamples with ``healpy.ang2pix(nside,
theta, phi)`` (``py/picca/io.py:486-488``, ``:593-595``) and writes the pixel
numbers as the ``HEALPID`` column of the correlation output
(``py/picca/bin/picca_cf.py:570-580``). healpy is not available here, so this
module restates the RING-scheme ``ang2pix`` from the HEALPix definition
(Gorski et al. 2005, ApJ 622, 759, section 4 and appendix): equatorial zone
|cos(theta)| <= 2/3 indexed by the two families of iso-latitude edge lines,
polar caps indexed by ring number from the pole. Vectorised with numpy.
"""

import numpy as np


def ang2pix_ring(nside, theta, phi):
    """Return RING-scheme pixel indices for colatitude ``theta`` and
    longitude ``phi`` (radians). Arrays or scalars."""
    nside = int(nside)
    theta = np.asarray(theta, dtype=float)
    phi = np.asarray(phi, dtype=float)
    scalar = theta.ndim == 0 and phi.ndim == 0
    theta, phi = np.broadcast_arrays(np.atleast_1d(theta), np.atleast_1d(phi))

    z = np.cos(theta)
    za = np.abs(z)
    # longitude in units of pi/2, folded into [0, 4)
    tt = np.mod(phi, 2. * np.pi) * (2. / np.pi)
    tt = np.where(tt >= 4., tt - 4., tt)
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    pix = np.empty(theta.shape, dtype=np.int64)

    equator = za <= 2. / 3.
    if np.any(equator):
        t_eq = tt[equator]
        z_eq = z[equator]
        temp1 = nside * (0.5 + t_eq)
        temp2 = nside * z_eq * 0.75
        # indices of the ascending and descending edge lines
        jp = np.floor(temp1 - temp2).astype(np.int64)
        jm = np.floor(temp1 + temp2).astype(np.int64)
        ring = nside + 1 + jp - jm          # 1 .. 2*nside+1 from z = 2/3
        kshift = 1 - (ring & 1)
        ip = (jp + jm - nside + kshift + 1) // 2
        ip = np.mod(ip, 4 * nside)
        pix[equator] = ncap + (ring - 1) * 4 * nside + ip

    caps = ~equator
    if np.any(caps):
        t_c = tt[caps]
        z_c = z[caps]
        za_c = za[caps]
        frac = t_c - np.floor(t_c)
        # sqrt(3 (1 - |z|)) with the sin(theta) form near the poles for accuracy
        sth = np.sin(theta[caps])
        tmp = np.where(za_c > 0.99,
                       nside * sth / np.sqrt((1. + za_c) / 3.),
                       nside * np.sqrt(3. * (1. - za_c)))
        jp = np.floor(frac * tmp).astype(np.int64)
        jm = np.floor((1. - frac) * tmp).astype(np.int64)
        ring = jp + jm + 1                  # ring counted from the nearest pole
        ip = np.floor(t_c * ring).astype(np.int64)
        ip = np.mod(ip, 4 * ring)
        north = z_c > 0
        pix_c = np.where(north,
                         2 * ring * (ring - 1) + ip,
                         npix - 2 * ring * (ring + 1) + ip)
        pix[caps] = pix_c
    if scalar:
        return int(pix[0])
    return pix


def pix2ang_ring_center(nside, pix):
    """Colatitude/longitude of RING pixel centres (used by synthetic
    generators and tests)."""
    nside = int(nside)
    pix = np.asarray(pix, dtype=np.int64)
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    theta = np.empty(pix.shape)
    phi = np.empty(pix.shape)
    north = pix < ncap
    south = pix >= npix - ncap
    equ = ~(north | south)
    if np.any(north):
        p = pix[north]
        ring = ((1 + np.sqrt(1 + 2 * p)) // 2).astype(np.int64)
        ring = np.where(2 * ring * (ring - 1) > p, ring - 1, ring)
        ring = np.where(2 * (ring + 1) * ring <= p, ring + 1, ring)
        iphi = p - 2 * ring * (ring - 1)
        theta[north] = np.arccos(1. - ring**2 / (3. * nside**2))
        phi[north] = (iphi + 0.5) * np.pi / (2. * ring)
    if np.any(equ):
        p = pix[equ] - ncap
        ring = p // (4 * nside) + nside
        iphi = p % (4 * nside)
        shift = 0.5 * (1 + ((ring + nside) & 1))
        theta[equ] = np.arccos((2 * nside - ring) * 2. / (3. * nside))
        phi[equ] = (iphi + shift) * np.pi / (2. * nside)
    if np.any(south):
        p = npix - pix[south] - 1
        ring = ((1 + np.sqrt(1 + 2 * p)) // 2).astype(np.int64)
        ring = np.where(2 * ring * (ring - 1) > p, ring - 1, ring)
        ring = np.where(2 * (ring + 1) * ring <= p, ring + 1, ring)
        iphi = 4 * ring - 1 - (p - 2 * ring * (ring - 1))
        theta[south] = np.pi - np.arccos(1. - ring**2 / (3. * nside**2))
        phi[south] = (iphi + 0.5) * np.pi / (2. * ring)
    return theta, phi
