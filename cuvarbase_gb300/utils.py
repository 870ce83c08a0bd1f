"""Host-side utilities of the GLS path (numpy, FP64).

These mirror cuvarbase/utils.py: the same names, arguments and results, so
code written against the reference keeps working.  They prepare inputs on the
host exactly as the reference does before its kernels run; no periodogram
arithmetic happens here.
"""
from __future__ import annotations

from copy import deepcopy

import numpy as np


def weights(err):
    """Observation weights w = err^-2 / sum(err^-2) (cuvarbase/utils.py:10-13)."""
    w = np.power(err, -2)
    return w / sum(w)


def autofrequency(t, nyquist_factor=5, samples_per_peak=5,
                  minimum_frequency=None, maximum_frequency=None, **kwargs):
    """Frequency grid df * (nf0 + arange(Nf)) with df = 1 / (baseline * spp)
    (cuvarbase/utils.py:46-97).

    Nf = int(0.5 * samples_per_peak * nyquist_factor * len(t)) unless
    maximum_frequency is given, in which case Nf = int(fmax / df) - nf0;
    nf0 = max(1, int(minimum_frequency / df)).
    """
    baseline = max(t) - min(t)
    n_samples = len(t)
    df = 1. / (baseline * samples_per_peak)
    nf0 = 1
    if minimum_frequency is not None:
        nf0 = max([nf0, int(minimum_frequency / df)])
    if maximum_frequency is not None:
        Nf = int(maximum_frequency / df) - nf0
    else:
        Nf = int(0.5 * samples_per_peak * nyquist_factor * n_samples)
    return df * (nf0 + np.arange(Nf))


def get_autofreqs(t, **kwargs):
    """autofrequency with only its own keyword arguments (cuvarbase/utils.py:106-110)."""
    keys = ('minimum_frequency', 'maximum_frequency', 'nyquist_factor',
            'samples_per_peak')
    return autofrequency(t, **{k: v for k, v in kwargs.items() if k in keys})


def normalize_light_curves(data):
    """Subtract the unweighted nanmean from t and y of every light curve;
    other columns are copied unchanged (cuvarbase/utils.py:113-146)."""
    data = deepcopy(data)
    for i, lc in enumerate(data):
        cols = []
        for j in range(len(lc)):
            if j < 2:
                cols.append((lc[j] - np.nanmean(lc[j])).copy())
            else:
                cols.append(lc[j].copy())
        data[i] = tuple(cols)
    return data
