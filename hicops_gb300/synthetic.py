"""Seeded synthetic peptide databases and MS/MS query batches.

Stands in for the FASTA-derived ``<len>.peps`` database parts and the MS2 query
files that the reference reads (source/core/lbe_internal.cpp:369-467 and
source/core/msquery.cpp:300-569). No public dataset is used: peptides and
spectra are drawn from seeded generators with the shapes and value
distributions of the workloads this package is measured on.

Peptides
    length ~ U{min_len..max_len}; residues i.i.d. from the 20 standard amino
    acids at natural frequencies (UniProtKB/Swiss-Prot amino-acid composition
    statistics, rounded to 0.01 %); the last residue is K or R (tryptic);
    deduplicated per length; kept only if min_mass <= mass <= max_mass, with the
    mass computed exactly as the loader does (single-precision running sum,
    source/core/utils.cpp:290-303, filter at lbe_internal.cpp:413).

Spectra
    80 % come from a random database entry: every b/y ion of charge 1..maxz is
    kept with p = 0.6, its m/z jittered by N(0, 0.005 Da); precursor = entry
    mass * (1 + N(0, 5 ppm)). 20 % are random: precursor ~ U[min_mass,
    max_mass]. Uniform noise peaks in [100, 2000] m/z fill each spectrum up to
    its peak count. Intensities ~ LogNormal(0, 1) are read as the MS2 reader
    does (x1000, msquery.cpp:425) and normalised by a restatement of
    ``MSQuery::pickpeaks`` (msquery.cpp:509-569): top peak = base_int, keep at
    most QALEN peaks with intensity >= min_int, ascending-intensity order,
    m/z key = (uint)(mz * scale).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from .params import gParams

QALEN = 100
PROTON = 1.00727647
H2O_F32 = np.float32(18.015)

# Residue masses and the static carbamidomethyl-C mod, as single-precision
# constants (values of source/core/utils.cpp:41-98; 'B','J','O','U','X','Z' are
# not amino acids and never generated).
_AA_MASS = {
    'A': 71.03712, 'C': 103.00919, 'D': 115.030, 'E': 129.0426, 'F': 147.068,
    'G': 57.02146, 'H': 137.060, 'I': 113.084, 'K': 128.094, 'L': 113.084,
    'M': 131.0405, 'N': 114.043, 'P': 97.0527, 'Q': 128.05858, 'R': 156.1012,
    'S': 87.032, 'T': 101.0476, 'V': 99.06841, 'W': 186.0793, 'Y': 163.0633,
}
NAA = -20000.0
AA_MASS_F32 = np.full(26, NAA, dtype=np.float32)
for _k, _v in _AA_MASS.items():
    AA_MASS_F32[ord(_k) - 65] = np.float32(_v)
STAT_MODS_F32 = np.zeros(26, dtype=np.float32)
STAT_MODS_F32[ord('C') - 65] = np.float32(57.021464)

# UniProtKB/Swiss-Prot amino-acid composition (percent), rounded.
_NATURAL_FREQ = {
    'A': 8.25, 'R': 5.53, 'N': 4.06, 'D': 5.46, 'C': 1.38, 'Q': 3.93, 'E': 6.72,
    'G': 7.07, 'H': 2.27, 'I': 5.91, 'L': 9.65, 'K': 5.80, 'M': 2.41, 'F': 3.86,
    'P': 4.74, 'S': 6.63, 'T': 5.35, 'W': 1.10, 'Y': 2.92, 'V': 6.86,
}
_AA_CODES = np.array([ord(k) for k in _NATURAL_FREQ], dtype=np.uint8)
_AA_P = np.array(list(_NATURAL_FREQ.values()), dtype=np.float64)
_AA_P /= _AA_P.sum()
_KR = np.array([ord('K'), ord('R')], dtype=np.uint8)
_KR_P = np.array([_NATURAL_FREQ['K'], _NATURAL_FREQ['R']]) / (_NATURAL_FREQ['K'] + _NATURAL_FREQ['R'])


class SearchParams(gParams):
    """gParams with the defaults of the measured workloads (report everything)."""

    def __init__(self, **kw):
        kw.setdefault("min_len", 7)
        kw.setdefault("expect_max", 1e300)
        super().__init__(**kw)


def pep_mass_f32(seqs: np.ndarray) -> np.ndarray:
    """Peptide mass in single precision, residue by residue.

    Restates UTILS_CalculatePepMass (source/core/utils.cpp:290-303): start from
    H2O = 18.015f, then for every residue add AAMass and, separately, StatMods,
    each addition rounded to float.
    """
    idx = seqs.astype(np.int64) - 65
    m = np.full(seqs.shape[0], H2O_F32, dtype=np.float32)
    for l in range(seqs.shape[1]):
        m = (m + AA_MASS_F32[idx[:, l]]).astype(np.float32)
        m = (m + STAT_MODS_F32[idx[:, l]]).astype(np.float32)
    return m


def make_database(n_peptides: int, seed: int, params: SearchParams) -> dict[int, np.ndarray]:
    """Return {length: uint8[n_L, L]} of unique tryptic peptides in file order."""
    rng = np.random.default_rng(seed)
    lens = np.arange(params.min_len, params.max_len + 1)
    out: dict[int, list] = {int(L): [] for L in lens}
    seen: dict[int, set] = {int(L): set() for L in lens}
    total = 0
    while total < n_peptides:
        batch = max(1024, int((n_peptides - total) * 1.08) + 64)
        blen = rng.integers(params.min_len, params.max_len + 1, size=batch)
        for L in lens:
            L = int(L)
            sel = int((blen == L).sum())
            if sel == 0:
                continue
            s = rng.choice(_AA_CODES, size=(sel, L), p=_AA_P)
            s[:, -1] = rng.choice(_KR, size=sel, p=_KR_P)
            mass = pep_mass_f32(s)
            ok = (mass >= np.float32(params.min_mass)) & (mass <= np.float32(params.max_mass))
            for row in s[ok]:
                key = row.tobytes()
                if key not in seen[L]:
                    seen[L].add(key)
                    out[L].append(row)
        total = sum(len(v) for v in out.values())
    # trim to exactly n_peptides, keeping generation order inside each length
    excess = total - n_peptides
    db = {L: np.array(v, dtype=np.uint8).reshape(-1, L) for L, v in out.items()}
    order = sorted(db, key=lambda L: -db[L].shape[0])
    i = 0
    while excess > 0:  # total >= n_peptides, so this ends (a length may become empty)
        L = order[i % len(order)]
        if db[L].shape[0] > 0:
            db[L] = db[L][:-1]
            excess -= 1
        i += 1
    return db


def write_peps(db: dict[int, np.ndarray], dbdir: str) -> None:
    os.makedirs(dbdir, exist_ok=True)
    for L, s in db.items():
        with open(os.path.join(dbdir, f"{L}.peps"), "wb") as f:
            if s.shape[0]:
                f.write(b"\n".join(r.tobytes() for r in s) + b"\n")


@dataclasses.dataclass
class QueryBatch:
    """CSR batch with the layout of the reference ``Queries`` (slm_dsts.h:422-559)."""
    idx: np.ndarray        # uint32[n+1]
    moz: np.ndarray        # uint32[npeaks]
    intensity: np.ndarray  # uint32[npeaks]
    precurse: np.ndarray   # float32[n]
    charges: np.ndarray    # int32[n]
    rtimes: np.ndarray     # float32[n]
    dM: np.ndarray | None = None  # optional float64[n] per-spectrum precursor tolerance (Da)
    source: np.ndarray | None = None  # int64[n]: (length<<32 | seqid) of the source, -1 if random

    @property
    def nspec(self) -> int:
        return int(self.precurse.shape[0])

    def slice(self, s0: int, s1: int) -> "QueryBatch":
        a, b = int(self.idx[s0]), int(self.idx[s1])
        return QueryBatch(
            idx=(self.idx[s0:s1 + 1] - a).astype(np.uint32),
            moz=self.moz[a:b].copy(), intensity=self.intensity[a:b].copy(),
            precurse=self.precurse[s0:s1].copy(), charges=self.charges[s0:s1].copy(),
            rtimes=self.rtimes[s0:s1].copy(),
            dM=None if self.dM is None else self.dM[s0:s1].copy(),
            source=None if self.source is None else self.source[s0:s1].copy())

    def write(self, path: str) -> None:
        with open(path, "wb") as f:
            np.array([self.nspec, self.moz.shape[0]], dtype=np.uint32).tofile(f)
            self.idx.astype(np.uint32).tofile(f)
            self.moz.astype(np.uint32).tofile(f)
            self.intensity.astype(np.uint32).tofile(f)
            self.precurse.astype(np.float32).tofile(f)
            self.charges.astype(np.int32).tofile(f)
            self.rtimes.astype(np.float32).tofile(f)


def write_ms2(path: str, q: "QueryBatch", scale: int, nspec: int | None = None) -> None:
    """The first `nspec` spectra of a batch as an MS2 text file (S, I RTime, Z
    lines, then one "m/z intensity" line per peak) that the reference's reader
    (MSQuery::readspectrum, msquery.cpp:300-505) turns back into the same
    integers: each value is written half a unit above itself, so atof * scale
    (or * 1000) truncates to it; nine digits bring a float32 precursor back."""
    n = q.nspec if nspec is None else min(int(nspec), q.nspec)
    idx = np.asarray(q.idx[:n + 1], dtype=np.int64)
    a, b = int(idx[0]), int(idx[-1])
    mz = (q.moz[a:b].astype(np.float64) + 0.5) / scale
    it = (q.intensity[a:b].astype(np.float64) + 0.5) / 1000.0
    lines = np.char.add(np.char.add(np.char.mod("%.6f", mz), " "), np.char.mod("%.5f", it))
    with open(path, "w") as f:
        f.write("H\tCreationDate\tsynthetic\n")
        for s in range(n):
            pm = f"{float(q.precurse[s]):.9g}"
            f.write(f"S\t{s + 1}\t{s + 1}\t{pm}\nI\tRTime\t{float(q.rtimes[s]):.9g}\n"
                    f"Z\t{int(q.charges[s])}\t{pm}\n")
            k0, k1 = int(idx[s]) - a, int(idx[s + 1]) - a
            if k1 > k0:
                f.write("\n".join(lines[k0:k1].tolist()))
                f.write("\n")


def _pickpeaks(mz_key: np.ndarray, raw_int: np.ndarray, valid: np.ndarray, params: SearchParams):
    """Vectorised restatement of MSQuery::pickpeaks (source/core/msquery.cpp:509-569).

    Rows are spectra; ``valid`` masks the raw peaks. Returns per-row kept
    (moz, intensity) in ascending-intensity order as a padded matrix + counts.
    """
    n, w = raw_int.shape
    key = np.where(valid, raw_int.astype(np.int64), -1)
    order = np.argsort(key, axis=1, kind="stable")
    s_int = np.take_along_axis(raw_int.astype(np.uint64), order, axis=1)
    s_mz = np.take_along_axis(mz_key, order, axis=1)
    s_valid = np.take_along_axis(valid, order, axis=1)
    nvalid = valid.sum(axis=1)
    top = s_int[:, -1].astype(np.float64)
    factor = np.where(nvalid > 0, np.float64(params.base_int) / np.maximum(top, 1.0), 0.0)
    scaled = np.floor(s_int.astype(np.float64) * factor[:, None]).astype(np.uint64)
    scaled[:, -1] = params.base_int
    pos_from_top = (w - 1) - np.arange(w)[None, :]
    in_top = (pos_from_top < QALEN) & s_valid
    keep = in_top & (scaled >= np.uint64(max(params.min_int, 0)))
    keep[:, -1] = nvalid > 0
    return s_mz, scaled.astype(np.uint32), keep


def make_queries(db: dict[int, np.ndarray], n_spectra: int, seed: int, params: SearchParams,
                 peaks: tuple[int, int] = (100, 100), frac_from_db: float = 0.8,
                 window_mix: list | None = None) -> QueryBatch:
    """Generate a query batch. ``peaks`` = (min, max) raw peak count per spectrum.

    ``window_mix`` = list of (probability, kind, value) with kind 'ppm' or 'da'
    gives each spectrum its own precursor tolerance (stored in ``QueryBatch.dM``).
    """
    rng = np.random.default_rng(seed)
    lens = sorted(db)
    counts = np.array([db[L].shape[0] for L in lens], dtype=np.int64)
    from_db = rng.random(n_spectra) < frac_from_db
    target = rng.integers(peaks[0], peaks[1] + 1, size=n_spectra)
    W = int(max(peaks[1], 2 * (params.max_len - 1) * params.maxz))
    mz = np.zeros((n_spectra, W), dtype=np.float64)
    valid = np.zeros((n_spectra, W), dtype=bool)
    prec = np.zeros(n_spectra, dtype=np.float32)
    source = np.full(n_spectra, -1, dtype=np.int64)

    # --- spectra made from database peptides, grouped by length ---
    pick_len = rng.choice(len(lens), size=n_spectra, p=counts / counts.sum())
    mod_mass = [float(m[1]) for m in params.mods]
    mod_res = [m[0] for m in params.mods]
    for li, L in enumerate(lens):
        rows = np.nonzero(from_db & (pick_len == li))[0]
        if rows.size == 0:
            continue
        pid = rng.integers(0, db[L].shape[0], size=rows.size)
        seq = db[L][pid]
        source[rows] = (np.int64(L) << 32) | pid.astype(np.int64)
        rmass = (AA_MASS_F32[seq - 65] + STAT_MODS_F32[seq - 65]).astype(np.float32).astype(np.float64)
        modd = np.zeros(seq.shape, dtype=np.float64)
        pmass = pep_mass_f32(seq)
        if params.mods and params.vmods_per_pep > 0:
            # random variant: each modifiable residue picked with p=0.5, at most the limit;
            # an N-terminal mod ('^', an extension) first, on the first residue's mass
            first_mod = np.full(rows.size, -1, dtype=np.int64)
            nm = np.zeros(rows.size, dtype=np.int64)
            for mi, rs in enumerate(mod_res):
                if rs == "^":
                    take = (rng.random(rows.size) < 0.5) & (nm < params.vmods_per_pep)
                    modd[take, 0] += mod_mass[mi]
                    first_mod = np.where(take & (first_mod < 0), mi, first_mod)
                    nm += take
            for pos in range(L):
                for mi, rs in enumerate(mod_res):
                    if rs == "^":
                        continue
                    can = np.isin(seq[:, pos], np.frombuffer(rs.encode(), dtype=np.uint8))
                    take = can & (rng.random(rows.size) < 0.5) & (nm < params.vmods_per_pep)
                    modd[take, pos] += mod_mass[mi]
                    first_mod = np.where(take & (first_mod < 0), mi, first_mod)
                    nm += take
            # precursor mass as the loader computes it: only the first mod's
            # scaled mass enters (source/core/utils.cpp:350-358)
            has = first_mod >= 0
            if has.any():
                add = np.array([np.float32(params.mod_mass_scaled(int(m))) / np.float32(params.scale)
                                for m in first_mod[has]], dtype=np.float32)
                pmass = pmass.copy()
                pmass[has] = (pmass[has] + add).astype(np.float32)
        tot = rmass + modd
        nb = L - 1
        cb = np.cumsum(tot, axis=1)[:, :nb]                     # b1..b_{L-1}
        cy = np.cumsum(tot[:, ::-1], axis=1)[:, :nb] + np.float64(H2O_F32)
        ions = []
        for z in range(1, params.maxz + 1):
            ions.append((cb + z * PROTON) / z)
            ions.append((cy + z * PROTON) / z)
        ions = np.concatenate(ions, axis=1)
        keep = rng.random(ions.shape) < 0.6
        jit = ions + rng.normal(0.0, 0.005, size=ions.shape)
        k = ions.shape[1]
        mz[rows, :k] = jit
        valid[rows, :k] = keep & (jit > 0)
        prec[rows] = (pmass.astype(np.float64) * (1.0 + rng.normal(0.0, 5e-6, size=rows.size))).astype(np.float32)

    rnd = np.nonzero(~from_db)[0]
    prec[rnd] = rng.uniform(params.min_mass, params.max_mass, size=rnd.size).astype(np.float32)

    # --- noise fill up to the target peak count ---
    have = valid.sum(axis=1)
    need = np.maximum(target - have, 0)
    col = np.arange(W)[None, :]
    free_rank = np.cumsum(~valid, axis=1) - 1
    noise = (~valid) & (free_rank < need[:, None])
    mz = np.where(noise, rng.uniform(100.0, 2000.0, size=mz.shape), mz)
    valid = valid | noise
    del col

    raw_int = np.floor(rng.lognormal(0.0, 1.0, size=mz.shape) * 1000.0).astype(np.uint64)
    mz_key = np.floor(mz * params.scale).astype(np.uint64).astype(np.uint32)
    s_mz, s_int, keep = _pickpeaks(mz_key, raw_int, valid, params)
    cnt = keep.sum(axis=1)
    idx = np.zeros(n_spectra + 1, dtype=np.uint32)
    idx[1:] = np.cumsum(cnt)
    moz = s_mz[keep].astype(np.uint32)
    inten = s_int[keep].astype(np.uint32)

    dM = None
    if window_mix:
        probs = np.array([w[0] for w in window_mix], dtype=np.float64)
        cls = rng.choice(len(window_mix), size=n_spectra, p=probs / probs.sum())
        dM = np.zeros(n_spectra, dtype=np.float64)
        for ci, (_, kind, val) in enumerate(window_mix):
            sel = cls == ci
            if kind == "ppm":
                dM[sel] = prec[sel].astype(np.float64) * val * 1e-6
            else:
                dM[sel] = val
    return QueryBatch(idx=idx, moz=moz, intensity=inten, precurse=prec,
                      charges=rng.integers(2, 4, size=n_spectra).astype(np.int32),
                      rtimes=(np.arange(n_spectra) * 0.1).astype(np.float32), dM=dM, source=source)


# A variable N-terminal acetylation: residue code '^' marks the peptide's
# N-terminus (an extension; the reference's mods are residue letters only).
NTERM_ACETYL = ("^", 42.010565, 1)

# --- the measured workloads (seeds fixed) ---

def workload(name: str):
    """(params, n_peptides, db_seed, n_spectra, q_seed, query kwargs) of a named workload."""
    if name == "plain-20k":       # 20,000 peptides, 2,000 spectra, dF 0.02 Da, dM 100 Da, z 1-2
        p = SearchParams(maxz=2, dF=2, dM=100.0)
        return p, 20000, 0xC0, 2000, 0xC1, {}
    if name == "open-2m":         # 2M peptides + M-ox (<=2), 100k spectra, dF 0.01, dM 500, z 1-3
        p = SearchParams(maxz=3, dF=1, dM=500.0, vmods_per_pep=2, mods=[("M", 15.99, 2)])
        return p, 2000000, 0xC10, 100000, 0xC11, {}
    if name == "open-200k":       # open-2m's shape at 1/10 of the database, 5,000 spectra (profiling)
        p = SearchParams(maxz=3, dF=1, dM=500.0, vmods_per_pep=2, mods=[("M", 15.99, 2)])
        return p, 200000, 0xC12, 5000, 0xC13, {}
    if name == "open-500k":       # open-2m's shape at 1/4 of the database, 2,000 spectra (kernel profiles)
        p = SearchParams(maxz=3, dF=1, dM=500.0, vmods_per_pep=2, mods=[("M", 15.99, 2)])
        return p, 500000, 0xC14, 2000, 0xC15, {}
    if name == "full-8m":         # 8M peptides + M-ox + N-term acetyl, 1M spectra of the mixed-window batch, 50k batches
        p = SearchParams(maxz=3, dF=1, dM=500.0, vmods_per_pep=3, mods=[("M", 15.99, 2), NTERM_ACETYL])
        return p, 8000000, 0xC40, 1000000, 0xC41, dict(
            peaks=(20, 150), window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)])
    if name == "mixed-2m":        # open-2m index, 200k spectra, 20-150 peaks, mixed windows
        p = SearchParams(maxz=3, dF=1, dM=500.0, vmods_per_pep=2, mods=[("M", 15.99, 2)])
        return p, 2000000, 0xC10, 200000, 0xC21, dict(
            peaks=(20, 150), window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)])
    raise KeyError(name)
