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
    import torch
    from hicops_gb300 import dslim
    p, db, q, ix = setup
    n = q.nspec
    d, args = _dev(q)
    ix.query_device(*args)
    m = dslim.MLP(ix, seed=3)
    dX = torch.zeros(n * 256, dtype=torch.float32, device="cuda")
    dY = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    m.features(d["hist"].data_ptr(), d["out"].data_ptr(), n, dX.data_ptr())
    m.targets(d["out"].data_ptr(), n, dY.data_ptr())
    torch.cuda.synchronize()
    m.train(dX.data_ptr(), dY.data_ptr(), n, batch=256, epochs=20, lr=1e-3)
    # device path: search, features, learned e-values on the whole batch
    learned = torch.zeros(n, dtype=torch.float32, device="cuda")
    nfb = torch.zeros(1, dtype=torch.int32, device="cuda")
    scratch = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    m.evalues(dX.data_ptr(), d["out"].data_ptr(), n, 0.1, learned.data_ptr(), nfb.data_ptr(), scratch.data_ptr())
    torch.cuda.synchronize()
    r0, _ = _results(d, n)
    # streamed in sub-batches with the same network
    r1, _, l1 = ix.query_stream(q, 333, mlp=m, thresh=0.1)
    assert np.array_equal(r0.view(np.uint8), r1.view(np.uint8)), "streamed learned results differ"
    l0 = learned.cpu().numpy()
    both = ~np.isnan(l0)
    assert np.array_equal(np.isnan(l0), np.isnan(l1))
    assert np.array_equal(l0[both], l1[both])
    assert ((r1["flags"] & 0x200) != 0).any()
    m.close()


def test_stream_rejects_bad_input(setup):
    p, db, q, ix = setup
    from hicops_gb300._lib import HcError
    with pytest.raises(HcError):
        ix.query_stream(q, 0)
