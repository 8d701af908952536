"""CCTOP score (beguidedoff/scoring.py:5-24), scalar and vectorised.

The reference computes ``sum(1.2 ** p for p in positions)`` with positions in
ascending order.  ``CCTOP_TERMS[p]`` holds the Python float ``1.2 ** p``.  The
vectorised form reproduces Python's ``sum`` bit for bit: on Python >= 3.12 the
builtin adds floats with Neumaier's compensated summation (Neumaier 1974,
"Rundungsfehleranalyse einiger Verfahren zur Summation endlicher Summen"),
on older interpreters it adds them left to right.
"""
import sys
from typing import List

import numpy as np

CCTOP_TERMS = np.array([0.0] + [1.2 ** p for p in range(1, 21)], dtype=np.float64)
COMPENSATED_SUM = sys.version_info >= (3, 12)


def calculate_cctop_score(mismatch_positions: List[int]) -> float:
    if not mismatch_positions:
        return 0.0
    return sum(1.2 ** pos for pos in mismatch_positions)


_RANKS = None


def score_ranks():
    """(rank_table, distinct_scores): rank_table[mask] (uint32, 2^20 entries)
    is the rank of mask's exact CCTOP score among ``distinct_scores``
    (ascending float64), so comparing ranks orders hits exactly by score."""
    global _RANKS
    if _RANKS is None:
        scores = cctop_from_masks(np.arange(1 << 20, dtype=np.int64))
        distinct, inverse = np.unique(scores, return_inverse=True)
        ranks = np.ascontiguousarray(inverse.astype(np.uint32))
        # read-only: engines keep a device copy keyed by this array's address
        ranks.flags.writeable = False
        distinct.flags.writeable = False
        _RANKS = (ranks, distinct)
    return _RANKS


def threshold_rank(threshold) -> int:
    """Largest rank whose score is <= threshold (-1 if none or no threshold)."""
    if threshold is None or threshold != threshold:  # None or NaN: nothing is <=
        return -1
    _, distinct = score_ranks()
    return int(np.searchsorted(distinct, float(threshold), side="right")) - 1


def scores_of_masks(masks: np.ndarray) -> np.ndarray:
    """cctop_from_masks through the score-rank table when it is built (the
    device epilogue builds it): the table's distinct scores are the same
    float64 values, so the lookup is exact and costs no per-position pass."""
    if _RANKS is None:
        return cctop_from_masks(masks)
    ranks, distinct = _RANKS
    return distinct[ranks[np.asarray(masks, dtype=np.int64)]]


def cctop_from_masks(masks: np.ndarray, compensated: bool = COMPENSATED_SUM) -> np.ndarray:
    """Scores of 20-bit mismatch masks (bit p-1 = position p), equal to
    ``calculate_cctop_score`` of the listed positions."""
    masks = np.asarray(masks, dtype=np.int64)
    s = np.zeros(masks.shape, dtype=np.float64)
    c = np.zeros(masks.shape, dtype=np.float64)
    for p in range(1, 21):
        on = ((masks >> (p - 1)) & 1).astype(bool)
        x = CCTOP_TERMS[p]
        t = s + x
        if compensated:
            big = np.abs(s) >= abs(x)
            comp = np.where(big, (s - t) + x, (x - t) + s)
            c = np.where(on, c + comp, c)
        s = np.where(on, t, s)
    return s + c if compensated else s
