"""GPU tests of the streaming query (hc_dslim_query_stream): sub-batches that
alternate between two staging slots must give exactly what one host-buffer
call gives (every result field and the histograms), including a ragged last
sub-batch, per-spectrum precursor windows and the learned e-values.
"""
import numpy as np
import pytest

from tests._util import case, compare
from tests.test_gpu_batched_learned import _dev, _results
from hicops_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MIX = [(0.5, "ppm", 10.0), (0.3, "da", 50.0), (0.2, "da", 500.0)]


@pytest.fixture(scope="module")
def setup():
    from hicops_gb300 import dslim
    p, db, _ = case("mods", 20000, 10, 851)
    q = S.make_queries(db, 1500, 852, p, peaks=(20, 150), window_mix=MIX)
    ix = dslim.Index(p)
    ix.construct_all(db)
    yield p, db, q, ix
    ix.close()


@pytest.mark.parametrize("batch", [137, 500, 1500, 4000])
def test_stream_equals_single_call(setup, batch):
    p, db, q, ix = setup
    r0, h0 = ix.query(q)
    r1, h1, _ = ix.query_stream(q, batch, want_hist=True)
    assert np.array_equal(r0.view(np.uint8), r1.view(np.uint8)), "stream results differ from one call"
    assert np.array_equal(h0, h1), "stream histograms differ from one call"


def test_stream_matches_oracle(setup):
    from oracle import oracle as O
    p, db, q, ix = setup
    r1, h1, _ = ix.query_stream(q.slice(0, 300), 64, want_hist=True)
    ores, ohist = O.OracleIndex(db, p).query(q.slice(0, 300), tie_rule=1)
    compare(r1, h1, ores, ohist)


def test_stream_with_learned_evalues(setup):
    """Streamed sub-batches with the learned tail give exactly what the
    batched+learned device call gives on the whole batch."""
    import torch
    from hicops_gb300 import dslim
    p, db, q, ix = setup
    n = q.nspec
    d, args = _dev(q)
    ix.query_device(*args)
    torch.cuda.synchronize()
    m, rep = dslim.fit_learned_tail(ix, d["hist"], d["out"], n, np.arange(0, n, 2), np.arange(1, n, 2), seed=3,
                                    epochs=20, batch=256)
    lg = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    ix.query_learned(m, *args, d_learned=lg.data_ptr())
    torch.cuda.synchronize()
    r0, _ = _results(d, n)
    r1, _, l1 = ix.query_stream(q, 333, mlp=m)
    assert np.array_equal(r0.view(np.uint8), r1.view(np.uint8)), "streamed learned results differ"
    l0 = lg.cpu().numpy()
    assert np.array_equal(np.isnan(l0), np.isnan(l1))
    both = ~np.isnan(l0)
    assert np.array_equal(l0[both], l1[both])
    assert ((r1["flags"] & 0x200) != 0).any()
    # a second call reuses the context's staging slots and gives the same
    r2, _, _ = ix.query_stream(q, 333, mlp=m)
    assert np.array_equal(r1.view(np.uint8), r2.view(np.uint8))
    m.close()


def test_stream_rejects_bad_input(setup):
    p, db, q, ix = setup
    from hicops_gb300._lib import HcError
    with pytest.raises(HcError):
        ix.query_stream(q, 0)
