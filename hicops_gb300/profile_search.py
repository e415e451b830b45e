"""A search case for kernel profilers: one warm-up query and one measured query
of a named synthetic workload with a given launch shape, nothing else.

    python -m hicops_gb300.profile_search --workload open-500k --spectra 2000 \
        --tuning '{"threads": 512, "tile": 10240, "ctas_per_sm": 2, "pairs_per_warp": 4, "schedule": 2}'

Each query launches k_windows, k_search (packed), k_search (wide, on the
spectra that overflowed) and k_tailfit; with schedule 2 also k_cost and
k_order. So `ncu -k regex:k_search -s 2 -c 1` captures the measured query's
packed search launch. Prints the search time of the measured query (CUDA
events) and its algorithmic bytes (4 x the postings the reference visits).
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="open-500k")
    ap.add_argument("--spectra", type=int, default=2000)
    ap.add_argument("--tuning", default="{}", help="hc_tuning fields as JSON (unset fields keep the defaults)")
    args = ap.parse_args()
    from . import dslim, synthetic as S
    from ._lib import RESULT_DTYPE
    p, npep, db_seed, _, q_seed, kw = S.workload(args.workload)
    db = S.make_database(npep, db_seed, p)
    q = S.make_queries(db, args.spectra, q_seed, p, **kw)
    ix = dslim.Index(p, device=0)
    ix.construct_all(db)
    tun = json.loads(args.tuning)
    if tun:
        ix.set_tuning(**tun)
    ix.set_profiling(True)
    for _ in range(2):
        res, _ = ix.query(q, want_hist=False)
    t = ix.stage_times()
    print(json.dumps({"workload": args.workload, "spectra": q.nspec, "tuning": ix.tuning(),
                      "search_ms": t.get("search"), "alg_bytes": float(np.sum(res["post_bytes"])),
                      "result_bytes": RESULT_DTYPE.itemsize * q.nspec}))
    ix.close()


if __name__ == "__main__":
    main()
