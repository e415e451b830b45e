"""Reference-facing host interface of the GB300 DSLIM search.

Mirrors the reference's DSLIM entry points (source/core/include/dslim.h) on
top of the C ABI: ``DSLIM_Construct`` builds one peptide length's index on the
device, ``DSLIM_QuerySpectrum`` searches a CSR batch (the ``Queries`` layout,
slm_dsts.h:422-559) and returns, per spectrum, what the reference hands to
``DFile_PrintScore`` (dslim_fileout.cpp:112-152). Status codes follow
slmerr.h; a failing call raises HcError carrying the code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .params import gParams


class Index:
    """Device-resident SLM index of all peptide lengths (the reference's Index[])."""

    def __init__(self, params: gParams, device: int = 0):
        self.params = params
        self._cp = L.to_hc_params(params)
        lib = L.load()
        h = C.c_void_p()
        rc = lib.hc_ctx_create(device, C.byref(self._cp), C.byref(h))
        if rc != 0:
            raise L.HcError(rc, "hc_ctx_create")
        self.ctx = h
        self.lib = lib
        self.seqs: dict[int, np.ndarray] = {}

    def close(self):
        if self.ctx:
            self.lib.hc_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise L.HcError(rc, what, self.lib.hc_last_error(self.ctx).decode())

    # -- tuning --
    def tuning(self) -> dict:
        t = L.HcTuning()
        self._check(self.lib.hc_ctx_get_tuning(self.ctx, C.byref(t)), "hc_ctx_get_tuning")
        return {k: getattr(t, k) for k, _ in L.HcTuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = L.HcTuning(**cur)
        self._check(self.lib.hc_ctx_set_tuning(self.ctx, C.byref(t)), "hc_ctx_set_tuning")

    # -- index --
    def construct(self, L_: int, seqs: np.ndarray, order: np.ndarray | None = None):
        """DSLIM_Construct for one length (dslim.h:49)."""
        seqs = np.ascontiguousarray(seqs, dtype=np.uint8).reshape(-1, L_)
        self.seqs[L_] = seqs
        o = None if order is None else np.ascontiguousarray(order, dtype=L.ENTRY_DTYPE)
        self._check(self.lib.hc_dslim_construct(self.ctx, L_, L.ptr(seqs), seqs.shape[0], L.ptr(o),
                                                0 if o is None else o.shape[0]), "hc_dslim_construct")

    def construct_all(self, db: dict, orders: dict | None = None):
        for L_ in range(self.params.min_len, self.params.max_len + 1):
            self.construct(L_, db.get(L_, np.zeros((0, L_), np.uint8)),
                           None if orders is None else orders.get(L_))

    def load(self, L_: int, seqs: np.ndarray, entries: np.ndarray, bA: np.ndarray, iA: np.ndarray):
        """Load a host-built index as-is (bA/iA as the reference's DSLIM_Construct lays them out)."""
        seqs = np.ascontiguousarray(seqs, dtype=np.uint8).reshape(-1, L_)
        self.seqs[L_] = seqs
        e = np.ascontiguousarray(entries, dtype=L.ENTRY_DTYPE)
        bA = np.ascontiguousarray(bA, dtype=np.uint32)
        iA = np.ascontiguousarray(iA, dtype=np.uint32)
        self._check(self.lib.hc_dslim_load(self.ctx, L_, L.ptr(seqs), seqs.shape[0], L.ptr(e), e.shape[0],
                                           L.ptr(bA), L.ptr(iA)), "hc_dslim_load")

    def info(self, L_: int):
        n = C.c_uint32()
        m = C.c_uint64()
        self._check(self.lib.hc_dslim_info(self.ctx, L_, C.byref(n), C.byref(m)), "hc_dslim_info")
        return n.value, m.value

    def export(self, L_: int):
        n, m = self.info(L_)
        e = np.zeros(n, dtype=L.ENTRY_DTYPE)
        bA = np.zeros(self.params.max_mass * self.params.scale + 1, dtype=np.uint32)
        iA = np.zeros(m, dtype=np.uint32)
        self._check(self.lib.hc_dslim_export(self.ctx, L_, L.ptr(e), L.ptr(bA), L.ptr(iA)), "hc_dslim_export")
        return e, bA, iA

    def entries(self, L_: int) -> np.ndarray:
        n, _ = self.info(L_)
        e = np.zeros(n, dtype=L.ENTRY_DTYPE)
        self._check(self.lib.hc_dslim_export(self.ctx, L_, L.ptr(e), None, None), "hc_dslim_export")
        return e

    # -- query --
    def query(self, q, want_hist: bool = True):
        """DSLIM_QuerySpectrum (dslim.h:184) on a host CSR batch; returns (results, hist)."""
        n = q.nspec
        out = np.zeros(n, dtype=L.RESULT_DTYPE)
        hist = np.zeros((n, L.HC_HIST_BINS), dtype=np.uint32) if want_hist else None
        idx = np.ascontiguousarray(q.idx, dtype=np.uint32)
        moz = np.ascontiguousarray(q.moz, dtype=np.uint32)
        inten = np.ascontiguousarray(q.intensity, dtype=np.uint32)
        prec = np.ascontiguousarray(q.precurse, dtype=np.float32)
        dM = None if getattr(q, "dM", None) is None else np.ascontiguousarray(q.dM, dtype=np.float64)
        self._check(self.lib.hc_dslim_query(self.ctx, L.ptr(idx), L.ptr(moz), L.ptr(inten), L.ptr(prec),
                                            L.ptr(dM), n, L.ptr(out), L.ptr(hist)), "hc_dslim_query")
        return out, hist

    def save(self, path: str):
        """Writes the built lengths to an index file (hc_dslim_save)."""
        self._check(self.lib.hc_dslim_save(self.ctx, path.encode()), "hc_dslim_save")

    def restore(self, path: str, seqs: dict | None = None):
        """Reads an index file written with the same index parameters (hc_dslim_restore)."""
        self._check(self.lib.hc_dslim_restore(self.ctx, path.encode()), "hc_dslim_restore")
        if seqs is not None:
            self.seqs.update(seqs)

    def write_psms(self, path: str, res: np.ndarray, q, file_label: str = "", spec_base: int = 0,
                   append: bool = False):
        """DFile_PrintScore's TSV (dslim_fileout.cpp:112-152) for the reported spectra of `res`."""
        res = np.ascontiguousarray(res, dtype=L.RESULT_DTYPE)
        prec = np.ascontiguousarray(q.precurse, dtype=np.float32)
        chg = None if q.charges is None else np.ascontiguousarray(q.charges, dtype=np.int32)
        rt = None if q.rtimes is None else np.ascontiguousarray(q.rtimes, dtype=np.float32)
        self._check(self.lib.hc_write_psms(self.ctx, path.encode(), file_label.encode(), spec_base, L.ptr(res),
                                           res.shape[0], L.ptr(prec), L.ptr(chg), L.ptr(rt), int(append)),
                    "hc_write_psms")

    def query_stream(self, q, batch: int, mlp=None, want_hist: bool = False):
        """Streams a host batch through the device in sub-batches (DSLIM_SearchManager's
        batch loop, dslim_query.cpp:160-420); returns (results, hist, learned log10 e)."""
        n = q.nspec
        out = np.zeros(n, dtype=L.RESULT_DTYPE)
        hist = np.zeros((n, L.HC_HIST_BINS), dtype=np.uint32) if want_hist else None
        learned = np.full(n, np.nan, dtype=np.float32) if mlp is not None else None
        idx = np.ascontiguousarray(q.idx, dtype=np.uint32)
        moz = np.ascontiguousarray(q.moz, dtype=np.uint32)
        inten = np.ascontiguousarray(q.intensity, dtype=np.uint32)
        prec = np.ascontiguousarray(q.precurse, dtype=np.float32)
        dM = None if getattr(q, "dM", None) is None else np.ascontiguousarray(q.dM, dtype=np.float64)
        self._check(self.lib.hc_dslim_query_stream(
            self.ctx, L.ptr(idx), L.ptr(moz), L.ptr(inten), L.ptr(prec), L.ptr(dM), n, batch,
            None if mlp is None else mlp.h, L.ptr(out), L.ptr(hist), L.ptr(learned)),
            "hc_dslim_query_stream")
        return out, hist, learned

    def query_device(self, d_idx: int, d_moz: int, d_int: int, d_prec: int, d_dM: int | None, nspec: int,
                     npeaks: int, d_out: int, d_hist: int, stream: int | None = None):
        """Device-buffer query (raw device pointers); enqueued on `stream`."""
        self._check(self.lib.hc_dslim_query_device(
            self.ctx, C.c_void_p(d_idx), C.c_void_p(d_moz), C.c_void_p(d_int), C.c_void_p(d_prec),
            None if d_dM is None else C.c_void_p(d_dM), nspec, npeaks, C.c_void_p(d_out),
            C.c_void_p(d_hist), None if stream is None else C.c_void_p(stream)), "hc_dslim_query_device")

    def last_launch_count(self) -> int:
        return self.lib.hc_last_launch_count(self.ctx)

    def set_profiling(self, on: bool = True):
        self._check(self.lib.hc_ctx_set_profiling(self.ctx, int(on)), "hc_ctx_set_profiling")

    def kernel_times(self) -> dict:
        """Device ms of each query stage of the last query (profiling on)."""
        t = [C.c_float() for _ in range(4)]
        self._check(self.lib.hc_last_kernel_times(self.ctx, *[C.byref(x) for x in t]), "hc_last_kernel_times")
        return dict(zip(("windows", "search", "wide", "tailfit"), (x.value for x in t)))

    def stage_times(self) -> dict:
        """Device ms of each stage of the last query (profiling on), with the learned tail if it ran."""
        t = (C.c_float * 5)()
        k = C.c_int()
        self._check(self.lib.hc_last_stage_times(self.ctx, t, C.byref(k)), "hc_last_stage_times")
        names = ("windows", "search", "wide", "tailfit", "learned")
        return {names[i]: t[i] for i in range(k.value)}

    def identity(self, res: np.ndarray):
        """(seqid, modnum, sites) of each top hit (-1 where none)."""
        n = res.shape[0]
        sid = np.full(n, -1, dtype=np.int64)
        mod = np.zeros(n, dtype=np.uint32)
        site = np.zeros(n, dtype=np.uint64)
        cache = {}
        for i in np.nonzero(res["idxoffset"] >= 0)[0]:
            L_ = int(res["idxoffset"][i]) + self.params.min_len
            if L_ not in cache:
                cache[L_] = self.entries(L_)
            e = cache[L_][int(res["psid"][i])]
            sid[i], mod[i], site[i] = e["seqid"], e["modnum"], e["sites"]
        return sid, mod, site


class MSQuery:
    """MS2 file reader with device peak picking: the reference's MSQuery
    (source/core/include/msquery.hpp:73-113). ``initialize`` reads the file
    (hc_ms2_open), ``extractbatch`` returns the next batch of at most `count`
    picked spectra as a Queries-layout batch (hc_ms2_extract)."""

    def __init__(self, index: Index):
        self.ix = index
        self.h = None
        self.QAcount = 0
        self.maxslen = 0
        self.running_count = 0

    def initialize(self, path: str):
        h = C.c_void_p()
        n, mx = C.c_uint32(), C.c_uint32()
        self.ix._check(self.ix.lib.hc_ms2_open(self.ix.ctx, path.encode(), C.byref(h), C.byref(n), C.byref(mx)),
                       "hc_ms2_open")
        self.DeinitQueryFile()
        self.h, self.QAcount, self.maxslen, self.running_count = h, n.value, mx.value, 0
        return self

    def getQAcount(self) -> int:
        return self.QAcount

    def extract(self, first: int, count: int):
        """Spectra [first, first+count) (clamped) as a QueryBatch."""
        from .synthetic import QueryBatch
        count = max(0, min(count, self.QAcount - first))
        idx = np.zeros(count + 1, dtype=np.uint32)
        moz = np.zeros(max(count * L.HC_QALEN, 1), dtype=np.uint32)
        inten = np.zeros_like(moz)
        prec = np.zeros(count, dtype=np.float32)
        chg = np.zeros(count, dtype=np.int32)
        rt = np.zeros(count, dtype=np.float32)
        nout, npk = C.c_uint32(), C.c_uint64()
        self.ix._check(self.ix.lib.hc_ms2_extract(self.ix.ctx, self.h, first, count, L.ptr(idx), L.ptr(moz),
                                                  L.ptr(inten), L.ptr(prec), L.ptr(chg), L.ptr(rt),
                                                  C.byref(nout), C.byref(npk)), "hc_ms2_extract")
        k = int(npk.value)
        return QueryBatch(idx=idx, moz=moz[:k].copy(), intensity=inten[:k].copy(), precurse=prec, charges=chg,
                          rtimes=rt)

    def extractbatch(self, count: int):
        """The next batch and the number of spectra left (MSQuery::extractbatch, msquery.cpp:239-297)."""
        b = self.extract(self.running_count, count)
        self.running_count += b.nspec
        return b, self.QAcount - self.running_count

    def DeinitQueryFile(self):
        if self.h:
            self.ix.lib.hc_ms2_close(self.h)
            self.h = None
        self.QAcount = self.running_count = self.maxslen = 0

    def __del__(self):
        try:
            self.DeinitQueryFile()
        except Exception:
            pass


def read_ms2_raw(path: str, scale: int) -> dict:
    """An MS2 file's raw spectra as the reference's readspectrum leaves them
    (before pickpeaks): host only, no device needed (hc_ms2_read + hc_ms2_raw)."""
    lib = L.load()
    h = C.c_void_p()
    n, mx = C.c_uint32(), C.c_uint32()
    rc = lib.hc_ms2_read(path.encode(), scale, C.byref(h), C.byref(n), C.byref(mx))
    if rc != 0:
        raise L.HcError(rc, "hc_ms2_read")
    try:
        ns = n.value
        off = np.zeros(ns + 1, dtype=np.uint64)
        rc = lib.hc_ms2_raw(h, 0, ns, L.ptr(off), None, None, None, None, None)
        if rc != 0:
            raise L.HcError(rc, "hc_ms2_raw")
        npk = int(off[-1])
        mz = np.zeros(max(npk, 1), dtype=np.uint32)
        it = np.zeros_like(mz)
        prec = np.zeros(ns, dtype=np.float64)
        z = np.zeros(ns, dtype=np.uint32)
        rt = np.zeros(ns, dtype=np.float64)
        rc = lib.hc_ms2_raw(h, 0, ns, L.ptr(off), L.ptr(mz), L.ptr(it), L.ptr(prec), L.ptr(z), L.ptr(rt))
        if rc != 0:
            raise L.HcError(rc, "hc_ms2_raw")
        return dict(off=off, mz=mz[:npk], intensity=it[:npk], prec=prec, z=z, rtime=rt, maxslen=mx.value)
    finally:
        lib.hc_ms2_close(h)


def DSLIM_Construct(index: Index, L_: int, seqs: np.ndarray) -> int:
    """dslim.h:49 — build one length's index on the device; returns SLM_SUCCESS."""
    index.construct(L_, seqs)
    return 0


def DSLIM_QuerySpectrum(queries, index: Index):
    """dslim.h:184 — search a batch; returns (results, histograms)."""
    return index.query(queries)


def _tune_device(ix: Index, d_idx, d_moz, d_int, d_prec, d_dM, nspec, npeaks, d_out, d_hist):
    """hc_tune on device buffers; returns (tuning dict, best ms)."""
    t = L.HcTuning()
    ms = C.c_float()
    ix._check(ix.lib.hc_tune(ix.ctx, C.c_void_p(d_idx), C.c_void_p(d_moz), C.c_void_p(d_int), C.c_void_p(d_prec),
                             None if d_dM is None else C.c_void_p(d_dM), nspec, npeaks, C.c_void_p(d_out),
                             C.c_void_p(d_hist), C.byref(t), C.byref(ms)), "hc_tune")
    return {k: getattr(t, k) for k, _ in L.HcTuning._fields_}, ms.value


Index.tune_device = _tune_device


def _query_graph(ix: Index, d_idx, d_moz, d_int, d_prec, d_dM, nspec, npeaks, d_out, d_hist, stream=None):
    """Batched form: the query pipeline replayed from a captured CUDA graph."""
    ix._check(ix.lib.hc_dslim_query_graph(
        ix.ctx, C.c_void_p(d_idx), C.c_void_p(d_moz), C.c_void_p(d_int), C.c_void_p(d_prec),
        None if d_dM is None else C.c_void_p(d_dM), nspec, npeaks, C.c_void_p(d_out), C.c_void_p(d_hist),
        None if stream is None else C.c_void_p(stream)), "hc_dslim_query_graph")


Index.query_graph = _query_graph


def _phase_cycles(ix: Index) -> dict:
    """Summed SM cycles per search-kernel phase since the last call (phase timing on)."""
    out = (C.c_uint64 * 10)()
    ix._check(ix.lib.hc_phase_cycles(ix.ctx, out), "hc_phase_cycles")
    return dict(zip(("setup", "stream", "score1", "score2", "clear", "rest", "n_tiles", "n_tiles_scanned",
                     "n_listed", "n_exact"), list(out)))


def _set_phase_timing(ix: Index, on: bool = True):
    ix._check(ix.lib.hc_ctx_set_phase_timing(ix.ctx, int(on)), "hc_ctx_set_phase_timing")


Index.phase_cycles = _phase_cycles
Index.set_phase_timing = _set_phase_timing


def _query_learned(ix: Index, mlp, d_idx, d_moz, d_int, d_prec, d_dM, nspec, npeaks, d_out, d_hist,
                   d_learned=None, stream=None):
    """Batched+learned form: search, learned tail and expeRT on the rest, replayed from a CUDA graph."""
    ix._check(ix.lib.hc_dslim_query_learned(
        ix.ctx, mlp.h, C.c_void_p(d_idx), C.c_void_p(d_moz), C.c_void_p(d_int), C.c_void_p(d_prec),
        None if d_dM is None else C.c_void_p(d_dM), nspec, npeaks, C.c_void_p(d_out), C.c_void_p(d_hist),
        None if d_learned is None else C.c_void_p(d_learned), None if stream is None else C.c_void_p(stream)),
        "hc_dslim_query_learned")


Index.query_learned = _query_learned


class MLP:
    """The learned e-value tail (256 -> 128 -> 64 -> 4), on the device of an Index."""

    N_IN, N_OUT = 256, 4

    def __init__(self, ix: Index, seed: int = 1):
        self.ix = ix
        h = C.c_void_p()
        ix._check(ix.lib.hc_mlp_create(ix.ctx, C.c_uint64(seed), C.byref(h)), "hc_mlp_create")
        self.h = h
        self.nparams = ix.lib.hc_mlp_num_params()

    def close(self):
        if self.h:
            self.ix.lib.hc_mlp_destroy(self.h)
            self.h = None

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, np.float32)
        self.ix._check(self.ix.lib.hc_mlp_get_params(self.h, L.ptr(out)), "hc_mlp_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self.ix._check(self.ix.lib.hc_mlp_set_params(self.h, L.ptr(p)), "hc_mlp_set_params")

    def gate(self) -> tuple[float, int]:
        r, k = C.c_float(), C.c_uint32()
        self.ix._check(self.ix.lib.hc_mlp_get_gate(self.h, C.byref(r), C.byref(k)), "hc_mlp_get_gate")
        return r.value, k.value

    def set_gate(self, max_resid: float = 0.1, radius: int = 4):
        self.ix._check(self.ix.lib.hc_mlp_set_gate(self.h, C.c_float(max_resid), radius), "hc_mlp_set_gate")

    def gradients(self, d_X: int, d_Y: int, n: int):
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        self.ix._check(self.ix.lib.hc_mlp_gradients(self.h, C.c_void_p(d_X), C.c_void_p(d_Y), n, L.ptr(g),
                                                    C.byref(loss)), "hc_mlp_gradients")
        return g, loss.value

    def train(self, d_X: int, d_Y: int, n: int, batch: int = 4096, epochs: int = 1, lr: float = 1e-3) -> float:
        loss = C.c_float()
        self.ix._check(self.ix.lib.hc_mlp_train(self.h, C.c_void_p(d_X), C.c_void_p(d_Y), n, batch, epochs,
                                                C.c_float(lr), C.byref(loss)), "hc_mlp_train")
        return loss.value

    def forward(self, d_X: int, n: int, d_out: int, stream: int | None = None):
        self.ix._check(self.ix.lib.hc_mlp_forward(self.h, C.c_void_p(d_X), n, C.c_void_p(d_out),
                                                  None if stream is None else C.c_void_p(stream)), "hc_mlp_forward")

    def features(self, d_hist: int, d_res: int, n: int, d_X: int, stream: int | None = None):
        self.ix._check(self.ix.lib.hc_mlp_features(self.ix.ctx, C.c_void_p(d_hist), C.c_void_p(d_res), n,
                                                   C.c_void_p(d_X), None if stream is None else C.c_void_p(stream)),
                       "hc_mlp_features")

    def targets(self, d_hist: int, d_res: int, n: int, d_Y: int, stream: int | None = None):
        """Y[n,4] from expeRT's own window: slope, intercept, first bin, residual (NaN: no target)."""
        self.ix._check(self.ix.lib.hc_mlp_targets(self.ix.ctx, C.c_void_p(d_hist), C.c_void_p(d_res), n,
                                                  C.c_void_p(d_Y), None if stream is None else C.c_void_p(stream)),
                       "hc_mlp_targets")

    def probe(self, d_X: int | None, d_hist: int, d_res: int, n: int, d_learned: int, d_aux: int,
              baseline: bool = False, stream: int | None = None):
        """Learned log10 e-values without the residual gate and, per spectrum, {predicted residual,
        residual, offset of the confirmed first bin} (NaN where no bin was confirmed)."""
        self.ix._check(self.ix.lib.hc_mlp_tail_probe(self.h, None if d_X is None else C.c_void_p(d_X),
                                                     C.c_void_p(d_hist), C.c_void_p(d_res), n, int(baseline),
                                                     C.c_void_p(d_learned), C.c_void_p(d_aux),
                                                     None if stream is None else C.c_void_p(stream)),
                       "hc_mlp_tail_probe")

    def learned_mask(self, d_X: int, d_hist: int, d_res: int, n: int, res: np.ndarray):
        """(learned, log10 e) of the n spectra as the gated learned tail decides them (host arrays)."""
        import torch
        lg = torch.empty(n, dtype=torch.float32, device="cuda")
        aux = torch.empty(3 * n, dtype=torch.float32, device="cuda")
        self.probe(d_X, d_hist, d_res, n, lg.data_ptr(), aux.data_ptr())
        torch.cuda.synchronize()
        lg, aux = lg.cpu().numpy(), aux.cpu().numpy().reshape(n, 3)
        gres, _ = self.gate()
        ok = (res["reported"] == 1) & (res["evalue"] > 0)
        return ok & np.isfinite(lg) & (aux[:, 0] <= gres), lg


def fit_learned_tail(ix: Index, d_hist, d_res, n: int, train: np.ndarray, cal: np.ndarray, seed: int = 5,
                     epochs: int = 30, batch: int = 512, lr: float = 1e-3, max_resid: float = 0.1,
                     radius: int = 4) -> tuple["MLP", dict]:
    """Trains the learned tail on histograms the GPU search produced.

    d_hist / d_res: device tensors (torch) of a search with expeRT e-values over
    n spectra; train / cal: disjoint spectrum indices. The targets are expeRT's
    own window (first bin), line and residual on every spectrum with a fit;
    the report gives the learned share and the agreement with expeRT on the
    `cal` spectra. Returns the network and the report.
    """
    import time
    import torch
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=L.RESULT_DTYPE)
    m = MLP(ix, seed=seed)
    m.set_gate(max_resid, radius)
    dX = torch.empty(n * 256, dtype=torch.float32, device=d_hist.device)
    dY = torch.empty(n * 4, dtype=torch.float32, device=d_hist.device)
    m.features(d_hist.data_ptr(), d_res.data_ptr(), n, dX.data_ptr())
    m.targets(d_hist.data_ptr(), d_res.data_ptr(), n, dY.data_ptr())
    torch.cuda.synchronize()
    Y = dY.view(n, 4).cpu().numpy()
    train = np.asarray(train, np.int64)
    train = train[np.isfinite(Y[train, 2])]  # spectra with an expeRT window
    X2, Y2 = dX.view(n, 256), dY.view(n, 4)
    tr = torch.from_numpy(train).to(d_hist.device)
    t0 = time.time()
    Xt, Yt = X2[tr].contiguous(), Y2[tr].contiguous()
    loss = m.train(Xt.data_ptr(), Yt.data_ptr(), Xt.shape[0], batch=batch, epochs=epochs, lr=lr)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del Xt, Yt
    cal = np.asarray(cal, np.int64)
    ca = torch.from_numpy(cal).to(d_hist.device)
    rsel = d_res.view(-1, 64)[ca].contiguous()
    hsel = d_hist.view(n, -1)[ca].contiguous()
    Xc = X2[ca].contiguous()
    used, lg = m.learned_mask(Xc.data_ptr(), hsel.data_ptr(), rsel.data_ptr(), int(cal.size), res[cal])
    rc = res[cal]
    ok = (rc["reported"] == 1) & (rc["evalue"] > 0)
    dl = np.abs(lg[used] - np.log10(rc["evalue"][used])) if used.any() else np.zeros(1)
    return m, {"trained_on": int(train.size), "checked_on": int(cal.size), "epochs": epochs, "final_loss": loss,
               "train_s": t_train, "max_resid": max_resid, "radius": radius,
               "learned_share": float(used.sum() / max(1, ok.sum())), "dlog10e_max": float(dl.max()),
               "dlog10e_p99": float(np.percentile(dl, 99))}
