"""Minimal stand-in for the two pandas helpers the reference imports
(``pd.unique`` keeps first-appearance order; ``pd.factorize`` numbers labels
in first-appearance order). Used only by make_golden.py to import the
reference in a container without pandas."""
import numpy as np


def unique(values):
    a = np.asarray(values)
    _, first = np.unique(a, return_index=True)
    return a[np.sort(first)]


def factorize(values):
    a = np.asarray(values)
    uniq, first, inv = np.unique(a, return_index=True, return_inverse=True)
    order = np.argsort(first)
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return rank[inv.reshape(-1)].astype(np.int64), uniq[order]


class DataFrame:  # never used on the paths the fixtures exercise
    def __init__(self, *args, **kwargs):
        raise NotImplementedError("pandas is not available")
