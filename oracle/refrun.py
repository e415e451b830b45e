"""Run the compiled reference DSLIM path (oracle/_ref/ref_driver) on a workload.

TEST INFRASTRUCTURE ONLY: used by tests and by tests/golden/make_golden.py to
pin the CPU restatement and to produce golden vectors. The driver exists only
where the reference sources were present at build time; callers skip when
``available()`` is False.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(HERE, "_ref", "ref_driver")
HIST_BINS = 1002

RECORD_DTYPE = np.dtype([
    ("reported", "<i4"), ("psid", "<i4"), ("idxoffset", "<i4"), ("sharedions", "<i4"),
    ("totalions", "<i4"), ("hyperscore", "<f4"), ("e_x", "<f8"), ("npsms", "<i4"),
    ("mu", "<i4"), ("beta", "<i4"), ("minhyp", "<i4"), ("nexthyp", "<i4"), ("maxhyp", "<i4"),
    ("seqid", "<u4"), ("modnum", "<u4"), ("sites", "<u8"), ("pepmass", "<f4"), ("pad", "<u4"),
    ("hist", "<u4", (HIST_BINS,)), ("pad2", "<u4", (2,)),
])
assert RECORD_DTYPE.itemsize == 4096


def available() -> bool:
    return os.path.exists(DRIVER)


def reference_dir() -> str:
    """Where the reference sources are mounted: $HC_REFERENCE_DIR, else the
    read-only mount of the build container."""
    return os.environ.get("HC_REFERENCE_DIR") or "/root/reference"


def build(ref_root: str | None = None) -> bool:
    """Compile the reference into oracle/_ref when its sources are present."""
    ref_root = ref_root or reference_dir()
    if not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}",
                    f"-j{os.cpu_count() or 4}"], check=True)
    return available()


def run(params, db: dict, queries, dump_index: bool = False, workdir: str | None = None):
    """Run the reference on (params, db, queries); returns a dict of outputs."""
    from hicops_gb300.synthetic import write_peps
    tmp = workdir or tempfile.mkdtemp(prefix="hcref_")
    dbdir = os.path.join(tmp, "db")
    out = os.path.join(tmp, "out")
    os.makedirs(out, exist_ok=True)
    write_peps(db, dbdir)
    params.write_ref_params(os.path.join(tmp, "params.txt"))
    queries.write(os.path.join(tmp, "queries.bin"))
    cmd = [DRIVER, os.path.join(tmp, "params.txt"), dbdir, os.path.join(tmp, "queries.bin"), out]
    if dump_index:
        cmd.append("--dump-index")
    env = dict(os.environ, OMP_NUM_THREADS=str(params.threads))
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"ref_driver failed ({r.returncode}): {r.stderr[-2000:]}")
    res = {"records": np.fromfile(os.path.join(out, "results.bin"), dtype=RECORD_DTYPE),
           "lengths": {}, "timing": {}}
    with open(os.path.join(out, "timing.txt")) as f:
        for line in f:
            k, v = line.split()
            res["timing"][k] = float(v)
    for L in range(params.min_len, params.max_len + 1):
        p = os.path.join(out, f"len{L}")
        cnt = np.fromfile(p + "_count.bin", dtype=np.uint32)
        d = {"n": int(cnt[0]), "npep": int(cnt[1]),
             "mass": np.fromfile(p + "_mass.bin", dtype=np.float32),
             "seqid": np.fromfile(p + "_seqid.bin", dtype=np.uint32),
             "modnum": np.fromfile(p + "_modnum.bin", dtype=np.uint32),
             "sites": np.fromfile(p + "_sites.bin", dtype=np.uint64)}
        if dump_index:
            d["bA"] = np.fromfile(p + "_bA.bin", dtype=np.uint32)
            d["iA"] = np.fromfile(p + "_iA.bin", dtype=np.uint32)
        res["lengths"][L] = d
    return res


MS2_DRIVER = os.path.join(HERE, "_ref", "ms2_driver")


def ms2_available() -> bool:
    return os.path.exists(MS2_DRIVER)


def run_ms2(path: str, scale: int, base_int: int, min_int: int):
    """The reference MS2 reader + pickpeaks on one file (oracle/ref/ms2_driver.cpp):
    (status, dict of idx, moz, intensity, precurse, charges, rtimes)."""
    fd, out = tempfile.mkstemp(prefix="hcms2_", suffix=".bin")
    os.close(fd)
    try:
        r = subprocess.run([MS2_DRIVER, path, str(scale), str(base_int), str(min_int), out],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ms2_driver failed ({r.returncode}): {r.stderr[-2000:]}")
        d = np.fromfile(out, dtype="<u4")
    finally:
        os.unlink(out)
    st = int(d[:1].view("<i4")[0])
    n, npk = int(d[1]), int(d[2])
    o = 3
    res = {}
    for k, cnt, dt in (("idx", n + 1, "<u4"), ("moz", npk, "<u4"), ("intensity", npk, "<u4"),
                       ("precurse", n, "<f4"), ("charges", n, "<i4"), ("rtimes", n, "<f4")):
        res[k] = d[o:o + cnt].view(dt).copy()
        o += cnt
    return st, res
