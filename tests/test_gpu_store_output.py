"""GPU tests of the on-disk index (hc_dslim_save / hc_dslim_restore) and of the
PSM TSV writer (hc_write_psms, the columns of DFile_PrintScore,
dslim_fileout.cpp:112-152).
"""
import os

import numpy as np
import pytest

from tests._util import case
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    from hicops_gb300 import dslim
    p, db, q = case("mods", 6000, 400, 861)
    ix = dslim.Index(p)
    ix.construct_all(db)
    res, hist = ix.query(q)
    path = str(tmp_path_factory.mktemp("idx") / "index.hcd")
    ix.save(path)
    yield p, db, q, ix, res, hist, path
    ix.close()


def test_restore_gives_the_same_index_and_results(built):
    from hicops_gb300 import dslim
    p, db, q, ix, res, hist, path = built
    ix2 = dslim.Index(p)
    ix2.restore(path)
    for L in (p.min_len, (p.min_len + p.max_len) // 2, p.max_len):
        a, b = ix.export(L), ix2.export(L)
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)), f"length {L} differs"
    r2, h2 = ix2.query(q)
    assert np.array_equal(res.view(np.uint8), r2.view(np.uint8))
    assert np.array_equal(hist, h2)
    ix2.close()


def test_restore_rejects_other_parameters_and_bad_files(built, tmp_path):
    from hicops_gb300 import dslim
    from hicops_gb300._lib import HcError
    p, db, q, ix, res, hist, path = built
    p2, _, _ = case("plain", 10, 1, 1)  # other fragment charges and mods
    ix2 = dslim.Index(p2)
    with pytest.raises(HcError) as e:
        ix2.restore(path)
    assert e.value.status == -3002
    ix2.close()
    ix3 = dslim.Index(p)
    with pytest.raises(HcError) as e:
        ix3.restore(str(tmp_path / "missing.hcd"))
    assert e.value.status == -3006
    cut = tmp_path / "cut.hcd"
    with open(path, "rb") as f:
        cut.write_bytes(f.read(os.path.getsize(path) // 2))
    with pytest.raises(HcError) as e:
        ix3.restore(str(cut))
    assert e.value.status == -3013
    ix3.close()


def _first_length_layout(blob: bytes):
    """Offsets of the first length's query postings and ions in an index file
    ("HCDSLIM2" | hash | count, then per length L, npep, n, shift | npost | nb | qtotal
    and the arrays seqs, mass, seqid, sites, modnum, bA, qA, qp, ions)."""
    assert blob[:8] == b"HCDSLIM2"
    o = 8 + 8 + 4
    L, npep, n, shift = np.frombuffer(blob, np.uint32, 4, o)
    npost, = np.frombuffer(blob, np.uint64, 1, o + 16)
    nb, = np.frombuffer(blob, np.uint32, 1, o + 24)
    qtotal, = np.frombuffer(blob, np.uint64, 1, o + 28)
    o += 36 + int(npep) * int(L) + 4 * int(n) * 3 + 8 * int(n) + 8 * (int(nb) + 1)
    return int(L), int(n), int(shift), int(qtotal), o, o + 4 * int(qtotal)


def test_restore_rejects_corrupt_postings(built, tmp_path):
    """A posting naming an entry past the length's last, an ion past its spectrum,
    or a b/y bit that does not match its ion makes the file invalid."""
    from hicops_gb300 import dslim
    from hicops_gb300._lib import HcError
    p, db, q, ix, res, hist, path = built
    blob = bytearray(open(path, "rb").read())
    L, n, shift, qtotal, o_qp, o_ion = _first_length_layout(bytes(blob))
    assert shift == 3 and qtotal > 0
    qp = np.frombuffer(bytes(blob), np.uint32, qtotal, o_qp)
    k = int(np.nonzero(qp != 0xFFFFFFFF)[0][0])  # a real posting
    speclen = 2 * p.maxz * (L - 1)

    def rejected(mutate):
        b = bytearray(blob)
        mutate(b)
        bad = tmp_path / "bad.hcd"
        bad.write_bytes(bytes(b))
        ix2 = dslim.Index(p)
        try:
            with pytest.raises(HcError) as e:
                ix2.restore(str(bad))
            return e.value.status
        finally:
            ix2.close()

    def entry_past_end(b):
        b[o_qp + 4 * k:o_qp + 4 * k + 4] = np.uint32((n + 5) << 3).tobytes()

    def ion_past_end(b):
        b[o_ion + 2 * k:o_ion + 2 * k + 2] = np.uint16(speclen).tobytes()

    def wrong_series(b):
        x = int(qp[k]) ^ 4  # flip the b/y bit, keep the ion
        b[o_qp + 4 * k:o_qp + 4 * k + 4] = np.uint32(x).tobytes()

    for f in (entry_past_end, ion_past_end, wrong_series):
        assert rejected(f) == -3013, f.__name__


def test_psm_tsv_columns(built, tmp_path):
    p, db, q, ix, res, hist, path = built
    out = tmp_path / "psms.tsv"
    ix.write_psms(str(out), res, q, file_label="run1.ms2", spec_base=100)
    lines = out.read_text().splitlines()
    assert lines[0].split("\t") == ["file", "scan_num", "prec_mass", "charge", "retention_time", "peptide",
                                    "matched_ions", "total_ions", "calc_pep_mass", "mass_diff", "mod_info",
                                    "hyperscore", "expectscore", "num_hits"]
    rep = np.nonzero(res["reported"] == 1)[0]
    assert len(lines) - 1 == rep.size and rep.size > 0
    ents = {}
    for k, i in enumerate(rep):
        row = lines[k + 1].split("\t")
        r = res[i]
        L = p.min_len + int(r["idxoffset"])
        if L not in ents:
            ents[L] = ix.entries(L)
        e = ents[L][int(r["psid"])]
        pep = bytes(db[L][int(e["seqid"])]).decode()
        pm = np.float32(q.precurse[i])
        exp = ["run1.ms2", str(100 + i + 1), "%f" % pm, str(int(q.charges[i])), "%f" % np.float32(q.rtimes[i]),
               pep, str(int(r["sharedions"])), str(int(r["totalions"])), "%f" % np.float32(e["mass"]),
               "%f" % np.float32(pm - np.float32(e["mass"])), "", "%f" % np.float32(r["hyperscore"]),
               "%f" % float(r["evalue"]), str(int(r["cpsms"]))]
        assert row == exp, (row, exp)
    # appending adds rows without a second header
    ix.write_psms(str(out), res, q, file_label="run2.ms2", append=True)
    assert len(out.read_text().splitlines()) == 1 + 2 * rep.size
