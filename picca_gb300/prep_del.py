"""Observed-wavelength stack of deltas used by the cross-correlation driver.

``picca_xcf.py`` removes the mean delta as a function of observed wavelength
before pairing (py/picca/bin/picca_xcf.py:435-468) with
``prep_del.stack(data, stack_from_deltas=True)`` (py/picca/prep_del.py:13-60).
This module restates that stack and the subtraction, host side.
"""

import numpy as np


class StackGrid:
    """The class-level wavelength grid the reference keeps on ``Forest``."""
    log_lambda_min = None
    log_lambda_max = None
    delta_log_lambda = None


def stack(data, grid=StackGrid):
    """Weighted mean delta per observed log-wavelength bin.

    Returns (stack_log_lambda, stack_delta, stack_weight)."""
    num_bins = int((grid.log_lambda_max - grid.log_lambda_min) /
                   grid.delta_log_lambda) + 1
    stack_log_lambda = grid.log_lambda_min + np.arange(num_bins) * grid.delta_log_lambda
    stack_delta = np.zeros(num_bins)
    stack_weight = np.zeros(num_bins)
    for healpix in sorted(list(data.keys())):
        for forest in data[healpix]:
            bins = ((forest.log_lambda - grid.log_lambda_min) /
                    grid.delta_log_lambda + 0.5).astype(int)
            rebin = np.bincount(bins, weights=forest.delta * forest.weights)
            stack_delta[:len(rebin)] += rebin
            rebin = np.bincount(bins, weights=forest.weights)
            stack_weight[:len(rebin)] += rebin
    w = stack_weight > 0
    stack_delta[w] /= stack_weight[w]
    return stack_log_lambda, stack_delta, stack_weight


def remove_mean_lambda_obs(data, z_min, z_max, lambda_abs):
    """Subtract the stacked mean delta at each pixel's observed wavelength
    (py/picca/bin/picca_xcf.py:435-468)."""
    grid = StackGrid
    grid.delta_log_lambda = None
    for healpix in data:
        for delta in data[healpix]:
            step = np.asarray([delta.log_lambda[index] - delta.log_lambda[index - 1]
                               for index in range(1, delta.log_lambda.size)]).min()
            if grid.delta_log_lambda is None:
                grid.delta_log_lambda = step
            else:
                grid.delta_log_lambda = min(step, grid.delta_log_lambda)
    grid.log_lambda_min = np.log10((z_min + 1.0) * lambda_abs) - grid.delta_log_lambda / 2.0
    grid.log_lambda_max = np.log10((z_max + 1.0) * lambda_abs) + grid.delta_log_lambda / 2.0
    _, mean_delta, _ = stack(data, grid)
    for healpix in data:
        for delta in data[healpix]:
            bins = ((delta.log_lambda - grid.log_lambda_min) / grid.delta_log_lambda +
                    0.5).astype(int)
            delta.delta -= mean_delta[bins]
