"""Benchmark of the GB300 DSLIM search (open search, 2M peptides + M-ox, 100k spectra).

One step = one search of the whole query batch (100,000 spectra, 100 peaks,
dF 0.01 Da, dM +-500 Da, fragment charges 1-3) against the device-resident
index of 2,000,000 synthetic tryptic peptides with variable M-oxidation (<= 2).
`value` is spectra/s with the batch resident in HBM; `e2e` is the same through
the host-buffer C-ABI call (pinned inputs copied in, results copied out).
The index (~2 GB of postings) is far larger than L2, so no L2 flush is needed
between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`--impl reference` times the CPU restatement of the reference's DSLIM query
(oracle/hc_oracle.c, all host threads) on a bounded sample of the same
workload. Multi-GPU runs are independent replicas (spectrum sharding needs no
collective): each rank searches its own batch; timings are max-reduced.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spectra/s & postings GB/s vs HBM peak: batched+learned vs plain GPU, same PSMs"
WORKLOAD = os.environ.get("HC_WORKLOAD", "open-2m")
CPU_SAMPLE = int(os.environ.get("HC_CPU_SAMPLE", "2000"))


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_spectrum():
    """DRAM bytes per spectrum of the search kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_search_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_spectrum"])
    return None


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self, device: int):
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={device}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    mx = max(mx, float(c[2]))
                except ValueError:
                    continue
                for n, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(n_gpus: int):
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group("nccl" if os.environ.get("HC_DIST_BACKEND", "nccl") == "nccl" else "gloo")
    return dist.get_rank(), dist.get_world_size(), dist


def make_workload(rank: int):
    from hicops_gb300 import synthetic as S
    p, npep, dbs, nq, qs, kw = S.workload(WORKLOAD)
    p.threads = os.cpu_count() or 8
    t = time.time()
    db = S.make_database(npep, dbs, p)
    log(f"[bench] database: {sum(v.shape[0] for v in db.values())} peptides in {time.time() - t:.1f}s")
    t = time.time()
    q = S.make_queries(db, nq, qs + 1000 * rank, p, **kw)
    log(f"[bench] queries: {q.nspec} spectra, {q.moz.shape[0]} peaks in {time.time() - t:.1f}s")
    return p, db, q


def cpu_baseline(p, db, q, threads: int, sample: int):
    """The oracle (CPU restatement of DSLIM_QuerySpectrum) on a bounded sample."""
    from oracle import oracle as O
    t = time.time()
    oi = O.OracleIndex(db, p)
    log(f"[bench] oracle index built in {time.time() - t:.1f}s")
    qs = q.slice(0, min(sample, q.nspec))
    oi.query(qs.slice(0, min(64, qs.nspec)), threads=threads, want_hist=False)  # warm
    t = time.perf_counter()
    oi.query(qs, threads=threads, want_hist=False)
    dt = time.perf_counter() - t
    return {"value": qs.nspec / dt, "unit": "spectra/s", "cores": threads, "kind": "port",
            "sample": f"first {qs.nspec} spectra of the {q.nspec}-spectrum batch, one pass, "
                      f"{dt:.1f}s wall"}, oi


def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    p, db, q = make_workload(0)
    threads = os.cpu_count() or 8
    from oracle import oracle as O
    oi = O.OracleIndex(db, p)
    per_step = int(os.environ.get("HC_REF_STEP_SPECTRA", "500"))
    times = []
    for i in range(args.warmup + args.steps):
        s0 = (i * per_step) % max(1, q.nspec - per_step)
        qs = q.slice(s0, s0 + per_step)
        t = time.perf_counter()
        oi.query(qs, threads=threads, want_hist=False)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            times.append(dt)
    tot = sum(times)
    v = per_step * len(times) / tot
    out = {"metric": METRIC, "value": v, "unit": "spectra/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000 * tot / len(times), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
           "config": {"workload": WORKLOAD, "peptides": 2000000, "spectra_per_step": per_step,
                      "dF_bins": p.dF, "dM_da": p.dM, "maxz": p.maxz, "mods": "M+15.99 <=2"},
           "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "spectra/s", "cores": threads, "kind": "port",
                            "sample": f"{per_step} spectra per step of the 100k-spectrum batch"},
           "e2e": {"value": v, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, world, dist):
    import torch
    from hicops_gb300 import dslim
    from hicops_gb300._lib import RESULT_DTYPE, HC_HIST_BINS
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p, db, q = make_workload(rank)
    t = time.time()
    ix = dslim.Index(p, device=dev)
    ix.construct_all(db)
    torch.cuda.synchronize()
    t_build = time.time() - t
    log(f"[bench] device index built in {t_build:.1f}s")
    n = q.nspec
    npk = int(q.moz.shape[0])
    # device-resident inputs and outputs
    d_idx = torch.from_numpy(q.idx.astype(np.int32)).cuda()
    d_moz = torch.from_numpy(q.moz.view(np.int32)).cuda()
    d_int = torch.from_numpy(q.intensity.view(np.int32)).cuda()
    d_prec = torch.from_numpy(q.precurse).cuda()
    d_out = torch.empty(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_hist = torch.empty(n * HC_HIST_BINS, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    ix.set_profiling(True)

    def step():
        ix.query_device(d_idx.data_ptr(), d_moz.data_ptr(), d_int.data_ptr(), d_prec.data_ptr(), None, n, npk,
                        d_out.data_ptr(), d_hist.data_ptr(), stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    stream.synchronize()
    clocks = Clocks(dev) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    search_ms, launches = [], 0
    ev0.record(stream)
    for _ in range(args.steps):
        step()
        search_ms.append(ix.kernel_times()["search"])   # waits for this step's events
        launches += ix.last_launch_count()
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop() if clocks else None
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    res = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=RESULT_DTYPE)
    alg_bytes = float(res["post_bytes"].sum())
    value = n * world * args.steps / (ms / 1000.0)
    # end to end through the host-buffer call: pinned inputs in, results out
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    from hicops_gb300 import synthetic as S
    qh = S.QueryBatch(idx=pin(q.idx), moz=pin(q.moz), intensity=pin(q.intensity), precurse=pin(q.precurse),
                      charges=q.charges, rtimes=q.rtimes)
    ix.set_profiling(False)
    ix.query(qh, want_hist=False)  # warm the staging buffers
    e2e_t = []
    for _ in range(max(1, min(args.steps, 3))):
        t = time.perf_counter()
        r2, _ = ix.query(qh, want_hist=False)
        e2e_t.append(time.perf_counter() - t)
    e2e = n / statistics.median(e2e_t)
    same = bool(np.array_equal(r2["psid"], res["psid"]) and np.array_equal(r2["cpsms"], res["cpsms"]))
    peak, peak_kind = measured_peaks()
    s_ms = statistics.median(search_ms)
    achieved = alg_bytes / (s_ms / 1000.0) / 1e9
    tps = traffic_per_spectrum()
    out = {"metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
           "config": {"workload": WORKLOAD, "peptides": sum(v.shape[0] for v in db.values()), "entries": None, "postings": None,
                      "spectra_per_step": n, "peaks_per_spectrum": 100, "dF_bins": p.dF, "dM_da": p.dM,
                      "maxz": p.maxz, "mods": "M+15.99 <=2", "parallelism": f"replicas{world}",
                      "l2": "index (~2 GB postings) larger than L2; no flush", "form": "plain",
                      "tuning": ix.tuning()},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_source": peak_kind,
                        "traffic": None if tps is None else tps * n, "kernel": "k_search",
                        "alg_bytes_per_launch": alg_bytes, "kernel_ms": s_ms},
           "e2e": {"value": e2e, "unit": "spectra/s",
                   "h2d_bytes_per_step": int(q.idx.nbytes + q.moz.nbytes + q.intensity.nbytes + q.precurse.nbytes),
                   "d2h_bytes_per_step": int(n * RESULT_DTYPE.itemsize), "same_results": same},
           "gpu_launches": launches, "index_build_s": t_build, "clocks": clk}
    cfg = out["config"]
    cfg["entries"] = int(sum(ix.info(L)[0] for L in range(p.min_len, p.max_len + 1)))
    cfg["postings"] = int(sum(ix.info(L)[1] for L in range(p.min_len, p.max_len + 1)))
    if rank == 0 and not args.no_cpu:
        try:
            cb, _ = cpu_baseline(p, db, q, os.cpu_count() or 8, CPU_SAMPLE)
            out["cpu_baseline"] = cb
        except Exception as e:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    ix.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default=None, help="open-2m (default), open-200k, plain-20k, mixed-2m")
    args = ap.parse_args()
    if args.workload:
        global WORKLOAD
        WORKLOAD = args.workload
    rank, world, dist = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_gpu(args, rank, world, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
