"""The level schedule of the device's melting loops (CPU only).

change_phase.f90:264-483 cools each melting element's four corners in
place, in a serial order: columns ascending, rows downwards (three loops)
or, for flux melting, rows upwards.  The device runs each loop by levels,
2i + j (2i - j for the flux loop), one level after another and a level's
elements at once.  That equals the serial result when (a) every element
that shares a corner with a later one in the serial order lies on a lower
level, and (b) elements of one level share no corner.  Both are checked here
for random candidate sets on random meshes.
"""
import numpy as np
import pytest


def _share_corner(a, b):
    (ja, ia), (jb, ib) = a, b
    return abs(ja - jb) <= 1 and abs(ia - ib) <= 1 and a != b


def _serial(cands, upward):
    """(j, i) in the loop's serial order"""
    return sorted(cands, key=lambda t: (t[1], -t[0] if upward else t[0]))


@pytest.mark.parametrize("upward", [False, True])
@pytest.mark.parametrize("seed", range(6))
def test_levels_respect_the_serial_order(seed, upward):
    rng = np.random.default_rng(seed)
    nzr, nxr = rng.integers(3, 25, size=2)
    dens = rng.uniform(0.2, 0.9)
    cands = [(j, i) for i in range(nxr) for j in range(nzr) if rng.random() < dens]
    level = {t: (2 * t[1] - t[0]) if upward else (2 * t[1] + t[0]) for t in cands}
    order = _serial(cands, upward)
    for k, b in enumerate(order):
        for a in order[:k]:
            if _share_corner(a, b):
                assert level[a] < level[b], (a, b)
    by_level = {}
    for t in cands:
        by_level.setdefault(level[t], []).append(t)
    for group in by_level.values():
        for x in range(len(group)):
            for y in range(x + 1, len(group)):
                assert not _share_corner(group[x], group[y])


def test_level_schedule_reproduces_the_serial_cooling():
    """A toy of the loop: each element pulls its corners down by the excess
    of their mean over a threshold; by levels (numpy, a level at once) the
    result equals the serial loop exactly."""
    rng = np.random.default_rng(7)
    nz, nx = 12, 15
    T0 = rng.uniform(900.0, 1400.0, size=(nz + 1, nx + 1))
    sol = rng.uniform(1000.0, 1200.0, size=(nz, nx))
    cands = [(j, i) for i in range(nx) for j in range(nz) if rng.random() < 0.6]

    def cool(T, j, i):
        tm = 0.25 * (T[j, i] + T[j, i + 1] + T[j + 1, i] + T[j + 1, i + 1])
        if tm > sol[j, i]:
            over = tm - sol[j, i]
            T[j:j + 2, i:i + 2] -= over

    Ts = T0.copy()
    for j, i in _serial(cands, False):
        cool(Ts, j, i)
    Tl = T0.copy()
    levels = sorted({2 * i + j for j, i in cands})
    for lv in levels:
        group = [(j, i) for j, i in cands if 2 * i + j == lv]
        snap = Tl.copy()  # a level's elements all read the state before the level
        upd = []
        for j, i in group:
            tm = 0.25 * (snap[j, i] + snap[j, i + 1] + snap[j + 1, i] + snap[j + 1, i + 1])
            if tm > sol[j, i]:
                upd.append((j, i, tm - sol[j, i]))
        for j, i, over in upd:
            Tl[j:j + 2, i:i + 2] -= over
    assert np.array_equal(Ts, Tl)
