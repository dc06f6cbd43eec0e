"""Algorithmic bytes of the FLAC step (one place for the benchmark and the
roofline report).

Each persistent field is counted once read and once written per step (or per
launch for a single kernel); scratch that a fused kernel keeps on chip and
boundary arrays (bc, ncod) count 0; node fields are charged per element with
the node/element ratio N/E.
"""
from __future__ import annotations


def _r(mode: str) -> int:
    return 8 if mode == "fp64" else 4


def step_bytes_per_element(mode: str = "fp64", nphase: int = 2, n_over_e: float = 1.0043) -> float:
    """Bytes moved per element-step by the whole step."""
    r = _r(mode)
    elem = (16 * r * 2      # stress0 r+w
            + 4 * r * 2     # area r+w
            + 3 * r * 2     # strain r+w
            + r * 2         # aps r+w
            + 3 * r * 2     # se2sr r+w
            + r * 2         # sshrheat r+w
            + r             # visn r
            + 4             # iphase r
            + 8 * nphase    # phase_ratio r (FP64 in both modes)
            + 8             # source r
            + r)            # shrheat r
    node = (32      # cord r+w (FP64)
            + 32    # vel r+w (FP64)
            + 16    # temp r+w
            + 16)   # amass, rmass r
    return elem + node * n_over_e


def rheol_bytes_per_element(nphase: int = 2, mode: str = "fp64", n_over_e: float = 1.0043) -> float:
    """Bytes one launch of the fl_rheol kernel must move per element."""
    r = _r(mode)
    reads = (16 * r + 4 * r + 4 * r   # stress0, area, dvol
             + 3 * r + 3 * r + r + r + r  # se2sr, strain, sshrheat, aps, visn
             + 4 + 8 * nphase)        # iphase, phase_ratio
    writes = 16 * r + 3 * r + 3 * r + r + r  # stress0, se2sr, strain, sshrheat, aps
    if mode == "fp64":
        node = 32 * n_over_e  # cord + vel (x,z), FP64
    else:
        # hi/lo FP32 pairs of cord and vel; the corner forces of the node
        # gather (16 FP32 per element) and the FP32 p_ref split are written
        node = 32 * n_over_e
        reads += 4        # p_ref (hi part)
        writes += 16 * 4  # corner forces
    return reads + writes + node
