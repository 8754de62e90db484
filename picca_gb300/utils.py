"""Small helpers used by the correlation drivers.

``userprint`` (py/picca/utils.py:20-28), ``compute_ang_max``
(py/picca/utils.py:419-450) and ``shuffle_distrib_forests``
(py/picca/utils.py:453-500), with the reference's arithmetic.
"""

import sys

import numpy as np


def userprint(*args, **kwds):
    """print() followed by a flush of stdout."""
    print(*args, **kwds)
    sys.stdout.flush()


def compute_ang_max(cosmo, r_trans_max, z_min, z_min2=None):
    """Largest angular separation that can give r_trans < r_trans_max."""
    if z_min2 is None:
        z_min2 = z_min
    r_min = cosmo.get_dist_m(z_min)
    r_min2 = cosmo.get_dist_m(z_min2)
    if r_min + r_min2 < r_trans_max:
        return np.pi
    return 2. * np.arcsin(r_trans_max / (r_min + r_min2))


def shuffle_distrib_forests(data, seed):
    """Reassign angular positions among forests with a seeded permutation."""
    userprint(f"INFO: Shuffling the forests angular position with seed {seed}")
    param_list = ["ra", "dec", "x_cart", "y_cart", "z_cart", "cos_dec", "thingid"]
    info = {"healpix": []}
    for param in param_list:
        info[param] = []
    for healpix, deltas in data.items():
        for delta in deltas:
            info["healpix"].append(healpix)
            for param in param_list:
                info[param].append(getattr(delta, param))
    np.random.seed(seed)
    new_index = np.arange(len(info["ra"]))
    np.random.shuffle(new_index)
    index = 0
    shuffled = {}
    for deltas in data.values():
        for delta in deltas:
            for param in param_list:
                setattr(delta, param, info[param][new_index[index]])
            shuffled.setdefault(info["healpix"][new_index[index]], []).append(delta)
            index += 1
    return shuffled
