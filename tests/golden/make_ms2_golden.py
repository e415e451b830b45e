"""Generate the MS2 golden vectors in tests/golden/ from the reference itself.

Runs the unmodified reference MS2 reader and peak picker (MSQuery,
source/core/msquery.cpp, compiled by oracle/ref/Makefile and driven by
oracle/ref/ms2_driver.cpp) on the cases of tests/_ms2cases.py and stores each
input file's bytes together with the reference's output batch in
ms2_<case>.npz. Needs the reference sources.

    python tests/golden/make_ms2_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refrun  # noqa: E402
from tests import _ms2cases as MC  # noqa: E402

CASES = {
    # name: (seed, spectra, max raw peaks)
    "edge": (0, 0, 0),
    "lf-default": (0x5101, 60, 300),
    "crlf-coarse": (0x5102, 40, 250),
}


def make(name: str) -> str:
    seed, nspec, mx = CASES[name]
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "case.ms2")
        scale, base_int, min_int = MC.write_case(path, name, seed, nspec, mx)
        st, r = refrun.run_ms2(path, scale, base_int, min_int)
        raw = np.frombuffer(open(path, "rb").read(), dtype=np.uint8)
    out = os.path.join(HERE, f"ms2_{name}.npz")
    np.savez_compressed(out, ms2=raw, pick=np.array([scale, base_int, min_int], np.int64),
                        status=np.array([st], np.int32), **r)
    return out


if __name__ == "__main__":
    if not refrun.build():
        sys.exit("the reference sources are needed to regenerate the golden vectors")
    for n in CASES:
        print(make(n), os.path.getsize(os.path.join(HERE, f"ms2_{n}.npz")))
