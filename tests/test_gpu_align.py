"""NeighborhoodAligner on the GPU (src/algos/alignment.rs:25-75, src/lib.rs:
3040-3167) through the C ABI, against the oracle's f32 restatement.

With a given alpha the arithmetic is the reference's, product by product,
so the rows must be bit-identical.  The adaptive alpha takes 1 / ln(deg + 1)
from the device's logf, which may differ from the host's log by an ulp:
those rows are compared within 2e-6 relative."""
import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import random_problem

pytestmark = pytest.mark.gpu


def _graph(seed, n, deg=(0, 12)):
    prob = random_problem(seed, n=n, n_feat=4, dims=4, deg=deg)
    rows, cols = prob["rows"], prob["cols"]
    rng = np.random.default_rng(seed + 1)
    w = rng.uniform(0.1, 5.0, len(cols)).astype(np.float32)
    cdf = np.zeros_like(w)
    for v in range(n):      # per-row CDF of the weights (graph.rs:664-691)
        s, e = int(rows[v]), int(rows[v + 1])
        if e > s:
            c = np.cumsum(w[s:e], dtype=np.float32)
            cdf[s:e] = c / c[-1]
    return rows, cols, cdf


@pytest.mark.parametrize("dims", [1, 33, 128, 512])
@pytest.mark.parametrize("max_neighbors", [None, 3])
def test_align_bit_exact_with_alpha(oracle, dims, max_neighbors):
    rows, cols, cdf = _graph(dims, 700)
    emb = np.random.default_rng(dims).standard_normal((700, dims)).astype(np.float32)
    got = _native.align(rows, cols, cdf, emb, alpha=0.35, max_neighbors=max_neighbors)
    want = oracle.align(rows, cols, cdf, emb, alpha=0.35, max_neighbors=max_neighbors)
    assert np.array_equal(got, want)
    assert (np.diff(rows) == 0).any()          # nodes without edges: alpha * own row
    z = np.nonzero(np.diff(rows) == 0)[0]
    assert np.array_equal(got[z], emb[z] * np.float32(0.35))


def test_align_adaptive_alpha(oracle):
    rows, cols, cdf = _graph(5, 900, deg=(0, 40))
    emb = np.random.default_rng(5).standard_normal((900, 64)).astype(np.float32)
    got = _native.align(rows, cols, cdf, emb)
    want = oracle.align(rows, cols, cdf, emb)
    scale = np.abs(want).max(axis=1, keepdims=True) + 1e-30
    assert (np.abs(got - want) / scale).max() < 2e-6
    one = np.nonzero(np.diff(rows) <= 1)[0]    # deg 0 and 1: alpha = 1, the own row
    assert np.array_equal(got[one], emb[one])


def test_align_extremes_and_errors(oracle):
    rows, cols, cdf = _graph(9, 300)
    emb = np.random.default_rng(9).standard_normal((300, 16)).astype(np.float32)
    assert np.array_equal(_native.align(rows, cols, cdf, emb, alpha=1.0), emb)
    full = _native.align(rows, cols, cdf, emb, alpha=0.0)
    assert np.array_equal(full, oracle.align(rows, cols, cdf, emb, alpha=0.0))
    with pytest.raises(_native.NativeError):
        _native.align(rows, cols, cdf, emb, alpha=1.5)
    bad = cols.copy()
    bad[0] = 300
    with pytest.raises(_native.NativeError):
        _native.align(rows, bad, cdf, emb, alpha=0.5)


def test_neighborhood_aligner_class(oracle, tmp_path):
    import cloverleaf_gb300 as cl
    rows, cols, cdf = _graph(13, 400)
    g = cl.Graph.from_csr(rows, cols, cdf, cdf=True)
    emb = cl.NodeEmbeddings(g.vocab_, np.random.default_rng(13).standard_normal((400, 24)).astype(np.float32))
    na = cl.NeighborhoodAligner(alpha=0.25, max_neighbors=5)
    out = na.align(emb, g)
    assert np.array_equal(out.table, oracle.align(rows, cols, cdf, emb.table, alpha=0.25, max_neighbors=5))
    assert out.vocab_ is emb.vocab_ and repr(na) == "NeighborhoodAligner<Alpha=Some(0.25), MaxNeighbors=Some(5)>"
    p = str(tmp_path / "aligned.emb")
    na.align_to_disk(p, emb, g)
    back = cl.NodeEmbeddings.load(p)
    assert np.array_equal(back.table, out.table)


def test_align_neighbour_cap_beyond_degree_and_zero_alpha(oracle):
    rows, cols, cdf = _graph(21, 200, deg=(0, 4))
    emb = np.random.default_rng(21).standard_normal((200, 32)).astype(np.float32)
    a = _native.align(rows, cols, cdf, emb, alpha=0.0, max_neighbors=1000)     # cap above every degree
    b = _native.align(rows, cols, cdf, emb, alpha=0.0)
    assert np.array_equal(a, b)
    z = np.nonzero(np.diff(rows) == 0)[0]
    assert len(z) and not a[z].any()                 # no edges and alpha 0: zero rows
