"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

FLOAT_FIELDS = ("cord", "vel", "temp", "stress0", "area", "dvol", "strain", "aps", "visn",
                "e2sr", "se2sr", "shrheat", "sshrheat", "amass", "rmass", "phase_ratio")
INT_FIELDS = ("iphase", "ncod", "nmark_elem", "mark_id_elem", "mark_ntriag", "mark_phase", "mark_dead")


def rel_diff(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b|: the normalisation of the reference's
    benchmark/compare.py (differences relative to the field's largest value)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    d = float(np.max(np.abs(a - b))) if b.size else 0.0
    if scale == 0.0:
        return d
    return d / scale


def compare_states(gpu, ref, fields=FLOAT_FIELDS, ints=INT_FIELDS):
    out = {}
    for f in fields:
        out[f] = rel_diff(gpu[f], ref[f])
    bad_ints = [f for f in ints if not np.array_equal(gpu[f], ref[f])]
    return out, bad_ints


def oracle_state(path: str, **kw):
    """The oracle's own start-up state of an .inp file (its read_params and
    setflac chain; nothing of the product's host code)."""
    from oracle.oracle import new_state as oracle_new_state

    return oracle_new_state(path, **kw)
