"""
Host helpers of the reference used on the path (src/helpers/misc.py).
"""
from __future__ import annotations

import numpy as np


def normalize(data, dst_min=0.0, dst_max=1.0, perc_low=None, perc_up=None, clip=True):
    """Min-max (or percentile) normalisation to [dst_min, dst_max], float64
    result (src/helpers/misc.py:63-114)."""
    data = np.asarray(data)
    use_percentiles = perc_low is not None or perc_up is not None
    if use_percentiles:
        perc_low = 0. if perc_low is None else perc_low
        perc_up = 100. if perc_up is None else perc_up
        src_min, src_max = np.percentile(data, [perc_low, perc_up])
    else:
        src_min = np.min(data)
        src_max = np.max(data)
    if src_max - src_min == 0:
        return np.ones_like(data, dtype=np.float64) * dst_min
    result = (1. / (src_max - src_min)) * (data.astype(np.float64) - src_min)
    if dst_max != 1 and dst_min == 0:
        result = result * dst_max
    elif dst_min != 0:
        result = result * (dst_max - dst_min) + dst_min
    if clip and use_percentiles:
        np.clip(result, dst_min, dst_max, out=result)
    return result
