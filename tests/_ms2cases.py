"""MS2 test inputs: seeded random files (with many equal intensities, so the
quicksort's tie order decides which peaks survive the QALEN cut) and one
hand-written file with the reader's edge cases."""
from __future__ import annotations

import numpy as np

from oracle import ms2 as M

# (scale, base_int, min_int) combinations the cases run with
PICK = {"default": (100, 100000, 1000), "fine": (1000, 100000, 100), "coarse": (10, 5000, 0)}

EDGE = (
    "H\tCreationDate\tedge cases\n"
    "D\tsomething\n"
    "50.5 3.0\n"                      # a peak before the first S belongs to spectrum 1
    "S\t1\t1\t400.0\n"
    "I\tRTime\t1.5\n"
    "Z\t2\t801.5\n"
    "100.0 10.0\n"
    "100.0 10.0\n"                    # duplicate peak
    "  200.5   20.0\n"                # leading and repeated spaces
    "300.25\t30.0\n"                  # tab: one token, intensity takes the default
    "400.0\n"                         # no intensity
    "\r\n"                            # a lone CR is a peak line (m/z 0)
    "S\t2\t2\t500\n"                  # no peaks, no Z: inherits charge and precursor
    "S\t3\t3\t600\n"
    "Z\n"                             # Z without tokens: "1" and "0.01"
    "I\tRTime\n"                      # RTime without a value: 0.00
    "I\tOther\t5\n"
    "150.0 0.0\n"
    "250.0 0.0\n"                     # all-zero spectrum
    "S\t4\t4\t700\n"
    "Z\t-2\t900.0\n"                  # negative charge stays negative (unsigned MAX)
    "I\tRTime\t-3.0\n"                # negative retention time becomes 0
    + "".join(f"{100 + k * 7.25:.2f} {(k % 5) * 10 + 5:.1f}\n" for k in range(130))
    + "S\t5\t5\t800\n"
    "Z\t3\t1200.5x\n"                 # trailing garbage after the number
    "1e2 5e1\n"
    ".5 .25\n"
    "+7.5 -0.0\n"
    "S\t6\t6\t900\n"
    "Z\t2\t1000.0\r\n"                # CRLF line
    "I\tRTime\t7.0\r\n"
    "123.4 56.7\r\n"
    "223.4 56.7\r\n"
    "323.4 99.9"                      # last line without a newline
)


def random_spectra(seed: int, nspec: int, max_peaks: int = 400):
    rng = np.random.default_rng(seed)
    out = []
    for s in range(nspec):
        npk = int(rng.integers(0, max_peaks + 1))
        mzs = rng.uniform(100, 2000, npk)
        if rng.random() < 0.5:
            ints = rng.choice(np.round(rng.uniform(1, 5000, 6), 2), npk)
        else:
            ints = rng.uniform(0, 5000, npk)
        peaks = [(f"{a:.4f}", f"{b:.2f}") for a, b in zip(mzs, ints)]
        if npk and rng.random() < 0.1:
            peaks[int(rng.integers(0, npk))] = (peaks[0][0], "")
        rt = None if rng.random() < 0.3 else f"{rng.uniform(0, 100):.3f}"
        out.append((s + 1, f"{rng.uniform(400, 3000):.4f}", int(rng.integers(0, 5)), rt, peaks))
    return out


def write_case(path: str, name: str, seed: int = 0, nspec: int = 200, max_peaks: int = 400) -> tuple:
    """Writes case `name` to path; returns its (scale, base_int, min_int)."""
    if name == "edge":
        with open(path, "w", newline="") as f:
            f.write(EDGE)
        return PICK["default"]
    kind, pick = name.split("-")  # "lf-default", "crlf-coarse", ...
    M.write_ms2(path, random_spectra(seed, nspec, max_peaks), crlf=(kind == "crlf"))
    return PICK[pick]


def write_queries(path: str, q, scale: int) -> None:
    """A picked QueryBatch as MS2 text that reads back to the same integers."""
    from hicops_gb300 import synthetic as S
    S.write_ms2(path, q, scale)
