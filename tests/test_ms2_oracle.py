"""The MS2 reader / peak-picker restatement (oracle/ms2.py) against the
reference's own MSQuery: the committed golden vectors everywhere, and fresh
seeded files where the reference was built here (oracle/_ref/ms2_driver)."""
import os

import numpy as np
import pytest

from oracle import ms2 as M
from oracle import refrun
from tests import _ms2cases as MC

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ("idx", "moz", "intensity", "precurse", "charges", "rtimes")


def _same(a: dict, b: dict):
    for k in KEYS:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.dtype.itemsize == y.dtype.itemsize and np.array_equal(x.view(np.uint8), y.view(np.uint8)), k


@pytest.mark.parametrize("case", ["edge", "lf-default", "crlf-coarse"])
def test_oracle_matches_golden(case, tmp_path):
    g = np.load(os.path.join(GOLDEN, f"ms2_{case}.npz"))
    path = tmp_path / "g.ms2"
    path.write_bytes(g["ms2"].tobytes())
    st, o = M.read_ms2(str(path), *[int(v) for v in g["pick"]])
    assert st == int(g["status"][0]) == 0
    _same(o, g)


def test_tie_order_matters():
    """Equal intensities keep the quicksort's order, which is not a stable sort's."""
    key = [5, 5, 1, 5, 3, 5]
    val = [0, 1, 2, 3, 4, 5]
    M.keyval_sort(key, val)
    assert key == sorted(key)
    stable = [v for _, v in sorted(zip([5, 5, 1, 5, 3, 5], range(6)), key=lambda t: t[0])]
    assert val != stable


def test_no_peaks_is_invalid_size(tmp_path):
    p = tmp_path / "empty.ms2"
    p.write_text("H\tx\nS\t1\t1\t500\nZ\t2\t999\n")
    st, _ = M.read_ms2(str(p), 100, 100000, 1000)
    assert st == M.ERR_INVLD_SIZE
    if refrun.ms2_available():
        st2, _ = refrun.run_ms2(str(p), 100, 100000, 1000)
        assert st2 == st


@pytest.mark.skipif(not refrun.ms2_available(), reason="reference MS2 reader not built here")
@pytest.mark.parametrize("case,seed", [("lf-default", 11), ("crlf-default", 12), ("lf-fine", 13),
                                       ("crlf-coarse", 14), ("lf-coarse", 15)])
def test_oracle_matches_reference(case, seed, tmp_path):
    path = str(tmp_path / "r.ms2")
    pick = MC.write_case(path, case, seed, nspec=150, max_peaks=400)
    st, r = refrun.run_ms2(path, *pick)
    st2, o = M.read_ms2(path, *pick)
    assert st == st2 == 0
    _same(o, r)


# ---- the library's host reader (hc_ms2_read / hc_ms2_raw: no device needed) ----

def _raw_same(path, scale):
    from hicops_gb300 import dslim
    st, spectra = M.read_raw(path, scale)
    assert st == 0
    r = dslim.read_ms2_raw(path, scale)
    assert r["off"].shape[0] == len(spectra) + 1
    mz = np.array([v for sp in spectra for v in sp[3]], np.uint32)
    it = np.array([v for sp in spectra for v in sp[4]], np.uint32)
    off = np.cumsum([0] + [len(sp[3]) for sp in spectra]).astype(np.uint64)
    assert np.array_equal(r["off"], off)
    assert np.array_equal(r["mz"], mz) and np.array_equal(r["intensity"], it)
    assert np.array_equal(r["prec"], np.array([sp[0] for sp in spectra], np.float64))
    assert np.array_equal(r["z"], np.array([sp[1] & 0xFFFFFFFF for sp in spectra], np.uint32))
    assert np.array_equal(r["rtime"], np.array([sp[2] for sp in spectra], np.float64))


@pytest.mark.parametrize("case", ["edge", "lf-default", "crlf-coarse"])
def test_host_reader_matches_restatement_golden(case, tmp_path):
    g = np.load(os.path.join(GOLDEN, f"ms2_{case}.npz"))
    path = tmp_path / "g.ms2"
    path.write_bytes(g["ms2"].tobytes())
    _raw_same(str(path), int(g["pick"][0]))


def test_host_reader_parallel_stretches(tmp_path):
    """A file of several MB is cut into stretches parsed by different threads;
    spectra without their own Z / RTime lines inherit across the cuts."""
    path = str(tmp_path / "big.ms2")
    specs = MC.random_spectra(31, 3000, 300)
    M.write_ms2(path, specs, crlf=False)
    # drop some Z lines so inheritance crosses stretch boundaries
    lines = open(path).read().split("\n")
    keep = [ln for k, ln in enumerate(lines) if not (ln.startswith("Z") and k % 7 == 0)]
    open(path, "w").write("\n".join(keep))
    assert os.path.getsize(path) > 4 << 20
    _raw_same(path, 100)


def test_host_reader_errors(tmp_path):
    from hicops_gb300 import dslim
    from hicops_gb300._lib import HcError
    with pytest.raises(HcError) as e:
        dslim.read_ms2_raw(str(tmp_path / "missing.ms2"), 100)
    assert e.value.status == -3013
    p = tmp_path / "nopeaks.ms2"
    p.write_text("H\tx\nS\t1\t1\t500\nZ\t2\t999\n")
    with pytest.raises(HcError) as e:
        dslim.read_ms2_raw(str(p), 100)
    assert e.value.status == -3004
    p2 = tmp_path / "noscan.ms2"
    p2.write_text("100.0 5.0\n")
    r = dslim.read_ms2_raw(str(p2), 100)
    assert r["off"].shape[0] == 1
