"""Times the oracle port (oracle/hc_oracle.c) against the reference's own
DSLIM query compiled unmodified (oracle/_ref/ref_driver) on the same
workloads, databases, spectra and thread count. TEST INFRASTRUCTURE: it says
what the CPU baseline the GPU is compared with is worth. The reference cannot
run on a machine without its sources, so the measured ratio is written to
oracle/port_vs_reference.json, which the CPU-baseline legs of bench.py report.

  python -m oracle.time_port_vs_ref [--threads N]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

from hicops_gb300 import synthetic as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refrun  # noqa: E402

# (workload, peptides, spectra): the reference's CPU index build bounds the sizes
CASES = [("plain-20k", 20000, 2000), ("open-200k", 200000, 1000), ("open-2m", 2000000, 500)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 8)
    args = ap.parse_args()
    if not refrun.available() and not refrun.build():
        raise SystemExit("the reference driver is not built (its sources are not mounted)")
    out = {"host": platform.machine(), "cpu_count": os.cpu_count(), "threads": args.threads, "cases": {}}
    for name, npep, nq in CASES:
        p, _, dbs, _, qs, kw = S.workload(name)
        p.threads = args.threads
        p.spadmem = 8_000_000_000
        db = S.make_database(npep, dbs, p)
        q = S.make_queries(db, nq, qs, p, **kw)
        ref = refrun.run(p, db, q)
        t_ref = ref["timing"]["query_s"]
        oi = O.OracleIndex(db, p)
        oi.query(q.slice(0, min(64, q.nspec)), threads=args.threads, want_hist=False)
        t = time.perf_counter()
        res, _ = oi.query(q, threads=args.threads, want_hist=False)
        t_port = time.perf_counter() - t
        rec = ref["records"]
        same = bool(np.array_equal(res["cpsms"][rec["reported"] == 1], rec["npsms"][rec["reported"] == 1]))
        out["cases"][name] = {"peptides": npep, "spectra": q.nspec, "reference_query_s": t_ref,
                              "port_query_s": t_port, "reference_spectra_per_s": q.nspec / t_ref,
                              "port_spectra_per_s": q.nspec / t_port, "port_vs_reference_speed": t_ref / t_port,
                              "same_cpsms": same}
        print(name, json.dumps(out["cases"][name]), flush=True)
    with open(os.path.join(HERE, "port_vs_reference.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
