"""CPU tests of the library boundary and its host logic (no device compute)."""
import os
import re

import numpy as np
import pytest

from hicops_gb300 import _lib as L
from hicops_gb300 import synthetic as S
from hicops_gb300.params import gParams, parse_uparams
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    with open(os.path.join(ROOT, "include", "hicops_gb300.h")) as f:
        hdr = f.read()
    decl = set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(hc_[a-z_0-9]+)\s*\(", hdr, re.M))
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(lib, name), name
    assert set(L.EXPORTED) <= decl
    assert lib.hc_version() >= 10000


def _header_fields(hdr: str, name: str) -> list:
    """Field names, in order, of `typedef struct name { ... } name;` in the header."""
    body = re.search(r"typedef struct %s\s*\{(.*?)\}\s*%s;" % (name, name), hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"^(const\s+)?[A-Za-z_0-9]+\s+", "", decl)  # the type
        for v in decl.split(","):
            names.append(re.match(r"\s*\**\s*([A-Za-z_0-9]+)", v).group(1))
    return names


def test_ctypes_mirrors_match_the_header():
    """The Python mirrors of the ABI's structs list the header's fields in its
    order (a drift would pass values into the wrong fields)."""
    with open(os.path.join(ROOT, "include", "hicops_gb300.h")) as f:
        hdr = f.read()
    assert _header_fields(hdr, "hc_tuning") == [n for n, _ in L.HcTuning._fields_]
    assert _header_fields(hdr, "hc_params") == [n for n, _ in L.HcParams._fields_]
    assert _header_fields(hdr, "hc_entry") == list(L.ENTRY_DTYPE.names)
    assert _header_fields(hdr, "hc_result") == list(L.RESULT_DTYPE.names)


def test_ctx_create_without_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from hicops_gb300 import dslim
    with pytest.raises(L.HcError) as e:
        dslim.Index(S.SearchParams())
    assert e.value.status == -3022


def test_bad_params_rejected():
    import ctypes as C
    lib = L.load()
    p = S.SearchParams()
    p.max_len = 80
    h = C.c_void_p()
    assert lib.hc_ctx_create(0, C.byref(L.to_hc_params(p)), C.byref(h)) == -3002


@pytest.mark.parametrize("maxz", [1, 2, 3, 4, 5])
def test_division_constants_exact(maxz):
    lib = L.load()
    for Lp in range(2, 63):
        d = 2 * maxz * (Lp - 1)
        # exhaustive over the first 2^20 ids, plus the top of the 2^31 range
        assert lib.hc_check_division(d, 1 << 20) == 0, d


def _entries_c(p, L_, seqs):
    import ctypes as C
    lib = L.load()
    cp = L.to_hc_params(p)
    seqs = np.ascontiguousarray(seqs, np.uint8)
    n = lib.hc_make_entries(C.byref(cp), L_, L.ptr(seqs), seqs.shape[0], None, 0)
    out = np.zeros(n, L.ENTRY_DTYPE)
    assert lib.hc_make_entries(C.byref(cp), L_, L.ptr(seqs), seqs.shape[0], L.ptr(out), n) == n
    return out


@pytest.mark.parametrize("mods", [[], [("M", 15.99, 2)], [("M", 15.99, 2), ("STY", 79.97, 1)],
                                  [("M", 15.99, 2), S.NTERM_ACETYL], [S.NTERM_ACETYL, ("STY", 79.97, 1)]])
def test_host_entries_match_oracle(mods):
    p = S.SearchParams(maxz=3, vmods_per_pep=2 if mods else 0, mods=mods)
    db = S.make_database(800, 31, p)
    for L_ in (7, 15, 40):
        a = _entries_c(p, L_, db[L_])
        b = O.make_entries(db[L_], L_, p, sort=False)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), L_


def test_uparams_parser_quirks(tmp_path):
    f = tmp_path / "uparams.txt"
    f.write_text("\n".join(["/db/", "/ms2", "/ws", "8", "2", "7", "40", "3", "0.01", "500", "0.01", "100",
                            "500", "5000", "10", "20", "4", "4", "100", "0.01", "2048", "cyclic", "1", "2",
                            "M", "15.994915", "2"]) + "\n")
    p = parse_uparams(str(f))
    assert p.dF == 1 and p.scale == 100 and p.base_int == 100000 and p.min_int == 1000
    assert p.spadmem == 2048 * 1024 * 1024 and p.mods == [("M", 15.994915, 2)] and p.vmods_per_pep == 2
    assert p.mod_mass_scaled(0) == 1599


def test_generator_is_seeded():
    p = S.SearchParams(maxz=2)
    a = S.make_database(300, 5, p)
    b = S.make_database(300, 5, p)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    qa = S.make_queries(a, 20, 6, p)
    qb = S.make_queries(b, 20, 6, p)
    assert np.array_equal(qa.moz, qb.moz) and np.array_equal(qa.intensity, qb.intensity)
    # pickpeaks: at most QALEN peaks, ascending intensity, top = base_int
    for s in range(qa.nspec):
        i0, i1 = qa.idx[s], qa.idx[s + 1]
        it = qa.intensity[i0:i1]
        assert i1 - i0 <= 100 and np.all(np.diff(it.astype(np.int64)) >= 0)
        if i1 > i0:
            assert it[-1] == p.base_int and it.min() >= p.min_int


def test_nterm_mod_variants():
    """An N-terminal mod (residue code '^', an extension) gives every peptide one
    variant: site bit 63, the mod's condition in the first modnum nibble, the
    precursor mass raised by the mod's scaled mass; with a residue mod as well,
    the N-terminal branch comes first in the walk and its mod is the first nibble."""
    p = S.SearchParams(maxz=2, vmods_per_pep=1, mods=[S.NTERM_ACETYL])
    db = S.make_database(300, 41, p)
    L_ = 12
    e = _entries_c(p, L_, db[L_])
    npep = db[L_].shape[0]
    assert e.shape[0] == 2 * npep
    v = e[npep:]
    assert np.all(v["sites"] == np.uint64(1) << np.uint64(63)) and np.all(v["modnum"] == 1)
    assert np.array_equal(v["seqid"], np.arange(npep))
    add = np.float32(p.mod_mass_scaled(0)) / np.float32(p.scale)
    assert np.array_equal(v["mass"], (e["mass"][:npep] + add).astype(np.float32))
    p2 = S.SearchParams(maxz=2, vmods_per_pep=2, mods=[("M", 15.99, 1), S.NTERM_ACETYL])
    e2 = O.make_entries(db[L_], L_, p2, sort=False)
    nt = (e2["sites"] >> np.uint64(63)) & np.uint64(1) == 1
    assert nt.sum() >= npep
    assert np.all((e2["modnum"][nt] & 0xF) == 2)  # condition 1 (the N-terminus) is the first mod
