"""CPU restatement of the reference MS2 reader and peak picker.

TEST INFRASTRUCTURE ONLY: the oracle for the device MS2 path
(hicops_gb300/csrc/hc_ms2.cu). Pure Python, for files of a few thousand
spectra.

Follows, step by step:
  * MSQuery::initialize (source/core/msquery.cpp:88-178): one spectrum per
    line starting with 'S'; no peak line at all is ERR_INVLD_SIZE;
  * MSQuery::readspectrum (msquery.cpp:300-505): lines split on '\\n' only;
    empty, 'H' and 'D' lines skipped; 'Z' sets the charge (atoi of the 2nd
    token, default "1") and the precursor (atof of the 3rd, default "0.01");
    'I' with "RTime" as 2nd token sets the retention time (default "0.00");
    any other line is a peak: tokens split on ' ' only, m/z =
    uint(atof * scale), intensity = uint(atof * 1000), with "0.01" for a
    missing token in the first spectrum and "0.0" afterwards. Charge,
    precursor and retention time carry over from the previous spectrum when a
    spectrum has no line for them;
  * MSQuery::pickpeaks (msquery.cpp:509-569) with KeyVal_Parallel_Internal
    (source/core/include/keyval.h:48-104): Hoare quicksort of the peaks by
    intensity around the middle key (the order of equal intensities is that
    algorithm's), top peak := base_int, the next QALEN-1 scaled by
    base_int / top (truncated), the highest ones >= min_int kept; charge =
    MAX(1, Z) compared unsigned, retention time = MAX(0.0, rtime).
"""
from __future__ import annotations

import math
import re

import numpy as np

QALEN = 100
ERR_INVLD_SIZE = -3004  # slmerr.h value of ERR_INVLD_SIZE, as hc_status mirrors it

_FLOAT = re.compile(rb"[ \t\n\v\f\r]*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))", re.I)
_INT = re.compile(rb"[ \t\n\v\f\r]*([+-]?\d+)")


def atof(tok: bytes) -> float:
    """C atof on a decimal token: the longest numeric prefix, 0.0 if none."""
    m = _FLOAT.match(tok)
    if not m:
        return 0.0
    return float(m.group(1))


def atoi(tok: bytes) -> int:
    m = _INT.match(tok)
    v = int(m.group(1)) if m else 0
    return ((v + 2**31) % 2**32) - 2**31


def _tokens(line: bytes, delims: bytes) -> list[bytes]:
    """strtok_r: runs of delimiter bytes separate tokens; empty ones vanish."""
    out, cur = [], bytearray()
    for b in line:
        if b in delims:
            if cur:
                out.append(bytes(cur))
                cur = bytearray()
        else:
            cur.append(b)
    if cur:
        out.append(bytes(cur))
    return out


def _to_u32(x: float) -> int:
    """(uint_t) of a double in [0, 2^32): truncation toward zero."""
    if math.isnan(x) or math.isinf(x):
        return 0
    return int(x) & 0xFFFFFFFF


def read_raw(path: str, scale: int):
    """Raw spectra as readspectrum leaves them: list of (prec, Z, rtime, mz[], intn[])."""
    data = open(path, "rb").read()
    lines = data.split(b"\n")
    if lines and lines[-1] == b"":
        lines.pop()
    nS = sum(1 for ln in lines if ln[:1] == b"S")
    npk = sum(1 for ln in lines if ln and ln[:1] not in (b"S", b"H", b"I", b"D", b"Z"))
    if npk == 0:
        return ERR_INVLD_SIZE, []
    spectra = []
    z, prec, rt = 0, 0.0, 0.0
    mz, it = [], []
    started = False
    for ln in lines:
        if not ln or ln[:1] in (b"H", b"D"):
            continue
        c = ln[:1]
        if c == b"Z":
            t = _tokens(ln, b" \t")
            z = atoi(t[1] if len(t) > 1 else b"1")
            prec = atof(t[2] if len(t) > 2 else b"0.01")
        elif c == b"I":
            t = _tokens(ln, b" \t")
            if len(t) > 1 and t[1] == b"RTime":
                rt = atof(t[2] if len(t) > 2 else b"0.00")
        elif c == b"S":
            if started:
                spectra.append((prec, z, rt, mz, it))
                mz, it = [], []
            started = True
        else:
            dflt = b"0.01" if not spectra else b"0.0"
            t = _tokens(ln, b" ")
            mz.append(_to_u32(atof(t[0] if len(t) > 0 else dflt) * scale))
            it.append(_to_u32(atof(t[1] if len(t) > 1 else dflt) * 1000))
    if started:
        spectra.append((prec, z, rt, mz, it))
    return 0, spectra[:nS]


def keyval_sort(key: list, val: list) -> None:
    """KeyVal_Parallel_Internal (keyval.h:48-104) in place. Its two recursive
    calls cover disjoint ranges, so a stack visits them in any order."""
    n = len(key)
    if n == 0:
        return
    stack = [(0, n - 1)]
    while stack:
        left, right = stack.pop()
        i, j = left, right
        pivot = key[(left + right) // 2]
        while i <= j:
            while key[i] < pivot:
                i += 1
            while key[j] > pivot:
                j -= 1
            if i <= j:
                key[i], key[j] = key[j], key[i]
                val[i], val[j] = val[j], val[i]
                i += 1
                j -= 1
        if left < j:
            stack.append((left, j))
        if i < right:
            stack.append((i, right))


def pickpeaks(mz: list, intn: list, base_int: int, min_int: int):
    """Kept (moz, intensity) in ascending-intensity order."""
    key, val = list(intn), list(mz)
    keyval_sort(key, val)
    n = len(key)
    speclen = 0
    if n > 0:
        top = key[n - 1]
        factor = (float(base_int) / top) if top else math.inf
        key[n - 1] = base_int & 0xFFFFFFFF
        speclen = 1
        lmin = min_int & 0xFFFFFFFF
        j = n - 2
        while j >= n - QALEN and j >= 0:
            key[j] = _to_u32(key[j] * factor) if top else 0
            if key[j] >= lmin:
                speclen += 1
            j -= 1
    return val[n - speclen:], key[n - speclen:]


def read_ms2(path: str, scale: int, base_int: int, min_int: int):
    """The batch the reference hands to the search for the whole file:
    (status, idx, moz, intensity, precurse f32, charges i32, rtimes f32)."""
    st, spectra = read_raw(path, scale)
    if st:
        return st, None
    idx, moz, inten, prec, ch, rts = [0], [], [], [], [], []
    for (p, z, rt, mz, it) in spectra:
        km, ki = pickpeaks(mz, it, base_int, min_int)
        moz += km
        inten += ki
        idx.append(idx[-1] + len(km))
        prec.append(p)
        zu = z & 0xFFFFFFFF
        ch.append(1 if zu == 0 else ((zu + 2**31) % 2**32) - 2**31)
        rts.append(0.0 if 0.0 > rt else rt)
    return 0, dict(idx=np.array(idx, np.uint32), moz=np.array(moz, np.uint32),
                   intensity=np.array(inten, np.uint32), precurse=np.array(prec, np.float64).astype(np.float32),
                   charges=np.array(ch, np.int32), rtimes=np.array(rts, np.float64).astype(np.float32))


def write_ms2(path: str, spectra, crlf: bool = False) -> None:
    """Write spectra [(scan, prec, z, rtime|None, [(mz_text, int_text)])] as an MS2 file
    (test inputs; the m/z and intensity are written as given text)."""
    nl = "\r\n" if crlf else "\n"
    with open(path, "w", newline="") as f:
        f.write("H\tCreationDate\tsynthetic" + nl)
        for scan, prec, z, rt, peaks in spectra:
            f.write(f"S\t{scan}\t{scan}\t{prec}" + nl)
            if rt is not None:
                f.write(f"I\tRTime\t{rt}" + nl)
            f.write(f"Z\t{z}\t{prec}" + nl)
            for a, b in peaks:
                f.write(f"{a} {b}" + nl)
