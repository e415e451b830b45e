"""GPU tests of the batched form (schedules, CUDA-graph replay, autotuner)
and of the learned e-value tail (MLP gradients against a float64 numpy
restatement, the fused inference kernel, training, the confirmed window and
the expeRT fallback, and what the trained network gains).
"""
import numpy as np
import pytest

from tests._util import case, compare
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _dev(q, n_hist=True):
    import torch
    from hicops_gb300._lib import HC_HIST_BINS
    n = q.nspec
    d = dict(idx=torch.from_numpy(q.idx.astype(np.int32)).cuda(),
             moz=torch.from_numpy(q.moz.view(np.int32)).cuda(),
             inten=torch.from_numpy(q.intensity.view(np.int32)).cuda(),
             prec=torch.from_numpy(q.precurse).cuda(),
             dM=None if q.dM is None else torch.from_numpy(q.dM).cuda(),
             out=torch.zeros(n * 64, dtype=torch.uint8, device="cuda"),
             hist=torch.zeros(n * HC_HIST_BINS, dtype=torch.int32, device="cuda"))
    args = (d["idx"].data_ptr(), d["moz"].data_ptr(), d["inten"].data_ptr(), d["prec"].data_ptr(),
            None if d["dM"] is None else d["dM"].data_ptr(), n, int(q.moz.shape[0]), d["out"].data_ptr(),
            d["hist"].data_ptr())
    return d, args


def _results(d, n):
    from hicops_gb300._lib import RESULT_DTYPE, HC_HIST_BINS
    r = np.frombuffer(d["out"].cpu().numpy().tobytes(), dtype=RESULT_DTYPE).copy()
    h = d["hist"].cpu().numpy().view(np.uint32).reshape(n, HC_HIST_BINS).copy()
    return r, h


def test_schedules_graph_and_tuner_agree():
    import torch
    from hicops_gb300 import dslim
    from oracle import oracle as O
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    db = S.make_database(4000, 1201, p)
    q = S.make_queries(db, 500, 1202, p, peaks=(20, 150),
                       window_mix=[(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)])
    ores, ohist = O.OracleIndex(db, p).query(q, tie_rule=1)
    ix = dslim.Index(p)
    ix.construct_all(db)
    d, args = _dev(q)
    full = ix.tuning()["tile"]
    for t in (dict(schedule=0), dict(schedule=1), dict(schedule=2),
              dict(schedule=2, ctas_per_sm=2, tile=(full // 2 - 4096) // 2048 * 2048, threads=256, pairs_per_warp=2)):
        ix.set_tuning(**t)
        ix.query_device(*args)
        torch.cuda.synchronize()
        r, h = _results(d, q.nspec)
        compare(r, h, ores, ohist)
    s = torch.cuda.Stream()
    d["out"].zero_()
    for _ in range(2):
        ix.query_graph(*args, stream=s.cuda_stream)
    s.synchronize()
    r, h = _results(d, q.nspec)
    compare(r, h, ores, ohist)
    best, ms = ix.tune_device(*args)
    assert ms > 0 and best["threads"] in (256, 512, 1024)
    ix.query_device(*args)
    torch.cuda.synchronize()
    r, h = _results(d, q.nspec)
    compare(r, h, ores, ohist)
    ix.close()


@pytest.mark.parametrize("small_log2", [0, 15, 40])
def test_mixed_windows_persistent_edge_cases(small_log2):
    """The persistent longest-first schedule on one batch that mixes +-10 ppm,
    +-5 Da and +-500 Da windows, with variable mods and N-terminal acetylation,
    a spectrum without valid peaks, intensities that overflow the packed
    scorecard, and a +-1e-5 Da spectrum whose peaks repeat keys: all equal the
    oracle. small_log2: the spectra whose windows hold fewer than 2^small_log2
    candidates run in a second, small-block launch (none; the narrow windows;
    every spectrum)."""
    import torch
    from hicops_gb300 import dslim
    from oracle import oracle as O
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=3,
                       mods=[("M", 15.99, 2), S.NTERM_ACETYL])
    db = S.make_database(12000, 1301, p)
    q = S.make_queries(db, 700, 1302, p, peaks=(20, 150),
                       window_mix=[(0.5, "ppm", 10.0), (0.2, "da", 5.0), (0.3, "da", 500.0)])
    # spectrum 0: no valid peaks; spectrum 1: every peak twice (keys shared by two peaks);
    # spectrum 2: intensities >= 2^17
    idx, moz, inten = q.idx.astype(np.int64), q.moz.copy(), q.intensity.copy()
    moz[idx[0]:idx[1]] = 0
    a, b = idx[1], idx[2]
    half = (b - a) // 2
    moz[a + half:a + 2 * half] = moz[a:a + half]
    inten[idx[2]:idx[3]] = inten[idx[2]:idx[3]] + (1 << 17)
    q = S.QueryBatch(idx=q.idx, moz=moz, intensity=inten, precurse=q.precurse, charges=q.charges,
                     rtimes=q.rtimes, dM=q.dM)
    q.dM[1] = 1e-5  # a narrow window for the repeated-key spectrum
    ores, ohist = O.OracleIndex(db, p).query(q, tie_rule=1)
    ix = dslim.Index(p)
    ix.construct_all(db)
    d, args = _dev(q)
    ix.set_tuning(schedule=2, small_log2=small_log2)
    ix.query_device(*args)
    torch.cuda.synchronize()
    r, h = _results(d, q.nspec)
    compare(r, h, ores, ohist)
    assert (ores["cpsms"][q.dM < 1.0] > 0).any() and (ores["cpsms"][q.dM > 100.0] > 0).any()
    ix.close()


def _np_forward_backward(P, X, Y):
    """float64 restatement of the MLP loss and its gradients (the CPU oracle);
    NaN targets add no loss."""
    ni, h1, h2, no = 256, 128, 64, 4
    o = 0
    W1 = P[o:o + ni * h1].reshape(ni, h1); o += ni * h1
    b1 = P[o:o + h1]; o += h1
    W2 = P[o:o + h1 * h2].reshape(h1, h2); o += h1 * h2
    b2 = P[o:o + h2]; o += h2
    W3 = P[o:o + h2 * no].reshape(h2, no); o += h2 * no
    b3 = P[o:o + no]
    sc = np.array([10.0, 0.25, 0.1, 5.0])
    a1 = np.maximum(X @ W1 + b1, 0)
    a2 = np.maximum(a1 @ W2 + b2, 0)
    out = a2 @ W3 + b3
    T = Y * sc
    n = X.shape[0]
    diff = np.where(np.isnan(T), 0.0, out - T)
    loss = (diff ** 2).sum() / (n * no)
    dout = 2 * diff / (n * no)
    gW3 = a2.T @ dout; gb3 = dout.sum(0)
    da2 = (dout @ W3.T) * (a2 > 0)
    gW2 = a1.T @ da2; gb2 = da2.sum(0)
    da1 = (da2 @ W2.T) * (a1 > 0)
    gW1 = X.T @ da1; gb1 = da1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3]), loss, out


def test_mlp_gradients_match_float64_reference():
    import torch
    from hicops_gb300 import dslim
    p = S.SearchParams(maxz=2)
    ix = dslim.Index(p)
    m = dslim.MLP(ix, seed=7)
    rng = np.random.default_rng(3)
    n = 300
    X = rng.normal(-2, 1.5, size=(n, 256)).astype(np.float32)
    Y = np.stack([rng.uniform(-0.5, -0.05, n), rng.uniform(0, 6, n), rng.uniform(0, 80, n),
                  rng.uniform(-3, 0, n)], 1).astype(np.float32)
    Y[::3, 3] = np.nan  # the error column has no target there
    dX, dY = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    g, loss = m.gradients(dX.data_ptr(), dY.data_ptr(), n)
    P = m.params().astype(np.float64)
    g64, loss64, out64 = _np_forward_backward(P, X.astype(np.float64), Y.astype(np.float64))
    assert abs(loss - loss64) <= 1e-4 * max(1.0, abs(loss64))
    err = np.abs(g - g64) / (np.abs(g64).max() + 1e-12)
    assert err.max() < 2e-4, err.max()
    # the fused inference kernel gives the same outputs as the float64 forward pass
    dout = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    m.forward(dX.data_ptr(), n, dout.data_ptr())
    torch.cuda.synchronize()
    o = dout.cpu().numpy().reshape(n, 4)
    assert np.abs(o - out64).max() <= 1e-4 * max(1.0, np.abs(out64).max()), np.abs(o - out64).max()
    m.close()
    ix.close()


@pytest.fixture(scope="module")
def learned_setup():
    """Open search (+-500 Da) on a 50k-peptide index: a training batch and a held-out batch
    searched with expeRT e-values, and a learned tail fitted and calibrated on the first."""
    import torch
    from hicops_gb300 import dslim
    p = S.SearchParams(maxz=3, dF=1, dM=500.0, threads=8, vmods_per_pep=2, mods=[("M", 15.99, 2)])
    db = S.make_database(50000, 1301, p)
    ix = dslim.Index(p)
    ix.construct_all(db)
    qt = S.make_queries(db, 6000, 1302, p)
    qh = S.make_queries(db, 3000, 1303, p)
    dt, at = _dev(qt)
    ix.query_device(*at)
    torch.cuda.synchronize()
    n = qt.nspec
    m, rep = dslim.fit_learned_tail(ix, dt["hist"], dt["out"], n, np.arange(0, 4500), np.arange(4500, n),
                                    seed=11, epochs=60, batch=256)
    dh, ah = _dev(qh)
    ix.query_device(*ah)
    torch.cuda.synchronize()
    r0, h0 = _results(dh, qh.nspec)
    yield p, db, ix, m, rep, qh, dh, ah, r0, h0
    m.close()
    ix.close()


def test_learned_query_replaces_the_fit(learned_setup):
    """hc_dslim_query_learned on held-out spectra: integer results and histograms
    equal the plain search's; spectra left to expeRT carry its exact result;
    learned spectra carry their line in mu / beta, expeRT's bins, and an e-value
    within FP32 rounding of expeRT's (the window is expeRT's own)."""
    import torch
    p, db, ix, m, rep, qh, dh, ah, r0, h0 = learned_setup
    n = qh.nspec
    assert rep["learned_share"] > 0.3, rep
    d, args = _dev(qh)
    lg = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    for _ in range(2):  # capture, then replay
        ix.query_learned(m, *args, d_learned=lg.data_ptr(), stream=s.cuda_stream)
    s.synchronize()
    r1, h1 = _results(d, n)
    for f in ("cpsms", "idxoffset", "psid", "sharedions", "totalions", "hyperscore", "post_bytes"):
        assert np.array_equal(r1[f], r0[f]), f
    assert np.array_equal(h1, h0)
    used = (r1["flags"] & 0x200) != 0
    ok = (r0["reported"] == 1) & (r0["evalue"] > 0)
    assert used.sum() >= 0.3 * ok.sum(), (int(used.sum()), int(ok.sum()))
    assert not (used & ~ok).any()
    fb = ok & ~used
    # the fallback is expeRT itself: every field as the plain search wrote it
    assert np.array_equal(r1[fb].view(np.uint8), r0[fb].view(np.uint8))
    # spectra without an e-value are identical too
    assert np.array_equal(r1[~ok].view(np.uint8), r0[~ok].view(np.uint8))
    dl = np.abs(np.log10(r1["evalue"][used]) - np.log10(r0["evalue"][used]))
    assert dl.max() <= 0.05, np.percentile(dl, [50, 99, 100])
    assert np.percentile(dl, 99) <= 1e-3, np.percentile(dl, [50, 99, 100])
    # the line: expeRT's slope and intercept (x 1e6) to FP32 rounding
    assert np.percentile(np.abs(r1["mu"][used].astype(np.int64) - r0["mu"][used]), 99) <= 50
    l1 = lg.cpu().numpy()
    assert np.array_equal(np.isnan(l1), ~used)
    assert np.allclose(l1[used], np.log10(r1["evalue"][used]), atol=2e-5)
    e = 10.0 ** (r1["mu"][used] / 1e6 * r1["maxhyp"][used] + r1["beta"][used] / 1e6) * r1["cpsms"][used]
    assert np.allclose(e, r1["evalue"][used], rtol=1e-9)
    for f in ("minhyp", "nexthyp", "maxhyp"):
        assert np.array_equal(r1[f][used], r0[f][used]), f


def test_targets_are_experts_fit(learned_setup):
    """The training targets come from expeRT's own window on the FP32 curve: the
    first bin equals the tail fit's, and the e-value of the target line equals
    expeRT's for every spectrum that has one (no near tie)."""
    import torch
    p, db, ix, m, rep, qh, dh, ah, r0, h0 = learned_setup
    n = qh.nspec
    Y = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    m.targets(dh["hist"].data_ptr(), dh["out"].data_ptr(), n, Y.data_ptr())
    torch.cuda.synchronize()
    Y = Y.cpu().numpy().reshape(n, 4)
    ok = (r0["reported"] == 1) & (r0["evalue"] > 0)
    have = ok & np.isfinite(Y[:, 0])
    assert have.sum() >= 0.9 * ok.sum()
    lg = (np.trunc(Y[:, 0].astype(np.float64) * 1e6) / 1e6 * r0["maxhyp"]
          + np.trunc(Y[:, 1].astype(np.float64) * 1e6) / 1e6 + np.log10(np.maximum(r0["cpsms"], 1)))
    d = np.abs(lg[have] - np.log10(r0["evalue"][have]))
    assert d.max() <= 1e-2, np.percentile(d, [50, 99, 100])
    # the first bin of expeRT's window (stt1 + mark >= minhyp)
    assert (Y[have, 2] >= r0["minhyp"][have]).all()
    assert (Y[have, 3] >= 0).all()


def test_trained_network_gains_over_the_method_without_it(learned_setup):
    """On held-out spectra, the share of reported spectra the learned tail takes
    (predicted residual within 0.1 and a first bin confirmed within the radius)
    with the trained network, against the same search without the network
    (starting at the curve's first point) and against an untrained network."""
    import torch
    from hicops_gb300 import dslim
    p, db, ix, m, rep, qh, dh, ah, r0, h0 = learned_setup
    n = qh.nspec
    ok = (r0["reported"] == 1) & (r0["evalue"] > 0)
    X = torch.empty(n * 256, dtype=torch.float32, device="cuda")
    m.features(dh["hist"].data_ptr(), dh["out"].data_ptr(), n, X.data_ptr())

    def share(net, baseline):
        lg = torch.empty(n, dtype=torch.float32, device="cuda")
        aux = torch.empty(3 * n, dtype=torch.float32, device="cuda")
        net.probe(None if baseline else X.data_ptr(), dh["hist"].data_ptr(), dh["out"].data_ptr(), n,
                  lg.data_ptr(), aux.data_ptr(), baseline=baseline)
        torch.cuda.synchronize()
        lg, a = lg.cpu().numpy(), aux.cpu().numpy().reshape(n, 3)
        took = ok & np.isfinite(lg) & (baseline | (a[:, 0] <= 0.1))
        if took.any():
            d = np.abs(lg[took] - np.log10(r0["evalue"][took]))
            assert d.max() <= 0.05, d.max()  # a confirmed window is expeRT's, whoever proposed it
        return float(took.sum() / ok.sum())

    trained = share(m, False)
    base = share(m, True)
    m0 = dslim.MLP(ix, seed=12)
    untrained = share(m0, False)
    m0.close()
    assert trained > 2 * base and trained > 2 * untrained, (trained, base, untrained)
