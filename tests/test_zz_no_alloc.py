"""GPU test of the allocation-free query entry point (hc_dslim_query_noalloc),
called through the C ABI and compared with hc_dslim_query_device on the same
device buffers. Collected last so that it also runs after every other test
has used the library in this process; one case runs in a fresh process,
where the entry point is the first search, and checks that after its set-up
call no call changes the device's free memory.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests._util import case, compare
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_SPECTRA = 16384
HC_ERR_INVLD_SIZE = -3004


def _dev(q):
    import torch
    d = dict(idx=torch.from_numpy(q.idx.astype(np.int32)).cuda(),
             moz=torch.from_numpy(q.moz.view(np.int32)).cuda(),
             inten=torch.from_numpy(q.intensity.view(np.int32)).cuda(),
             prec=torch.from_numpy(q.precurse).cuda(),
             dM=None if q.dM is None else torch.from_numpy(q.dM).cuda())
    return d


def _out(n):
    import torch
    from hicops_gb300._lib import HC_HIST_BINS
    return (torch.full((n * 64,), 0xA5, dtype=torch.uint8, device="cuda"),
            torch.full((n * HC_HIST_BINS,), 7, dtype=torch.int32, device="cuda"))


def _args(d, n, npeaks, out, hist):
    return (C.c_void_p(d["idx"].data_ptr()), C.c_void_p(d["moz"].data_ptr()), C.c_void_p(d["inten"].data_ptr()),
            C.c_void_p(d["prec"].data_ptr()), None if d["dM"] is None else C.c_void_p(d["dM"].data_ptr()),
            n, npeaks, C.c_void_p(out.data_ptr()), C.c_void_p(hist.data_ptr()))


def _results(out, hist, n):
    from hicops_gb300._lib import RESULT_DTYPE, HC_HIST_BINS
    r = np.frombuffer(out.cpu().numpy().tobytes(), dtype=RESULT_DTYPE).copy()
    h = hist.cpu().numpy().view(np.uint32).reshape(n, HC_HIST_BINS).copy()
    return r, h


def test_noalloc_matches_query_device_two_calls():
    import torch
    from hicops_gb300 import dslim
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    db = S.make_database(4000, 1301, p)
    batches = [S.make_queries(db, 500, 1302, p, peaks=(20, 150),
                              window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)]),
               S.make_queries(db, 300, 1303, p)]
    ix = dslim.Index(p)
    ix.construct_all(db)
    lib = ix.lib
    s = torch.cuda.Stream()
    for k, (q, sched) in enumerate(zip(batches, (0, 2))):
        ix.set_tuning(schedule=sched)
        d = _dev(q)
        n, npk = q.nspec, int(q.moz.shape[0])
        ref_out, ref_hist = _out(n)
        rc = lib.hc_dslim_query_device(ix.ctx, *_args(d, n, npk, ref_out, ref_hist), None)
        assert rc == 0, lib.hc_last_error(ix.ctx)
        torch.cuda.synchronize()
        na_out, na_hist = _out(n)
        rc = lib.hc_dslim_query_noalloc(ix.ctx, *_args(d, n, npk, na_out, na_hist), C.c_void_p(s.cuda_stream))
        assert rc == 0, lib.hc_last_error(ix.ctx)
        s.synchronize()
        r_ref, h_ref = _results(ref_out, ref_hist, n)
        r_na, h_na = _results(na_out, na_hist, n)
        st = compare(r_na, h_na, r_ref, h_ref)
        assert st["reported"] > 0, (k, st)
    ix.close()


def test_noalloc_rejects_oversized_batch():
    import torch
    from hicops_gb300 import dslim
    p, db, _ = case("plain", 500, 10, 1311)
    ix = dslim.Index(p)
    ix.construct_all(db)
    n = MAX_SPECTRA + 1
    # a valid batch of empty spectra, so that the buffers cover every index
    d = dict(idx=torch.zeros(n + 1, dtype=torch.int32, device="cuda"),
             moz=torch.zeros(16, dtype=torch.int32, device="cuda"),
             inten=torch.zeros(16, dtype=torch.int32, device="cuda"),
             prec=torch.zeros(n, dtype=torch.float32, device="cuda"), dM=None)
    out, hist = _out(n)
    rc = ix.lib.hc_dslim_query_noalloc(ix.ctx, *_args(d, n, 0, out, hist), None)
    assert rc == HC_ERR_INVLD_SIZE
    assert b"16384" in ix.lib.hc_last_error(ix.ctx)
    rc = ix.lib.hc_dslim_query_noalloc(ix.ctx, *_args(d, MAX_SPECTRA, 0, out, hist), None)
    assert rc == 0, ix.lib.hc_last_error(ix.ctx)
    torch.cuda.synchronize()
    ix.close()


# Child process: the index is built (that allocates), then the first search
# of the process is the allocation-free one (its set-up call). Free device
# memory is read after it and after three more calls with other launch shapes
# (persistent in batch order, longest-first with another lists-in-flight
# count, one CTA per spectrum); only then does hc_dslim_query_device run, for
# the comparison.
_CHILD = r"""
import ctypes as C, json, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from hicops_gb300 import dslim, synthetic as S
from tests.test_zz_no_alloc import _dev, _out, _args, _results
from tests._util import compare
p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
db = S.make_database(3000, 1321, p)
q = S.make_queries(db, 400, 1322, p, peaks=(20, 150),
                   window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)])
ix = dslim.Index(p)
ix.construct_all(db)
lib = ix.lib
d = _dev(q)
n, npk = q.nspec, int(q.moz.shape[0])
outs = [_out(n) for _ in range(4)]
ref_out, ref_hist = _out(n)
torch.cuda.synchronize()
free = []
shapes = [dict(schedule=0), dict(schedule=2, pairs_per_warp=4, threads=512), dict(schedule=0, pairs_per_warp=8, threads=512),
          dict(schedule=1, pairs_per_warp=1)]
for k, (o, h) in enumerate(outs):
    ix.set_tuning(**shapes[k])
    rc = lib.hc_dslim_query_noalloc(ix.ctx, *_args(d, n, npk, o, h), None)
    assert rc == 0, lib.hc_last_error(ix.ctx)
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
ix.set_tuning(schedule=0)
rc = lib.hc_dslim_query_device(ix.ctx, *_args(d, n, npk, ref_out, ref_hist), None)
assert rc == 0, lib.hc_last_error(ix.ctx)
torch.cuda.synchronize()
r_ref, h_ref = _results(ref_out, ref_hist, n)
rep = 0
for o, h in outs:
    r, hh = _results(o, h, n)
    rep = compare(r, hh, r_ref, h_ref)["reported"]
ix.close()
print("RESULT " + json.dumps({"free": free, "reported": rep}))
"""


def test_noalloc_first_call_in_fresh_process_then_no_allocation():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _CHILD, root], capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("RESULT ")][-1]
    out = json.loads(line[7:])
    free = out["free"]
    # after the set-up call (free[0]) no call changed the free device memory
    assert all(f == free[0] for f in free[1:]), free
    assert out["reported"] > 0
