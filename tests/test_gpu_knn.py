"""GPU NodeEmbedder and exact cosine top-k (src/lib.rs:2092-2124,
src/algos/aggregator.rs:17-120, src/embeddings.rs:149-173) through the C ABI.

The embedder is compared bit for bit with a restatement of the reference's
f32 arithmetic.  The top-k rounds unit rows to BF16 (FP32 accumulation), so
it is checked against exact FP64 cosines up to that rounding: every returned
row's exact similarity is within 0.02 of the exact k-th best, returned
similarities within 0.02 of exact, and well separated neighbours exactly."""
import numpy as np
import pytest

from cloverleaf_gb300 import _native

pytestmark = pytest.mark.gpu
TOL_BF16 = 0.02


def _features(rng, n, n_feat, empty_every=7):
    k = rng.integers(1, 9, n)
    k[::empty_every] = 0
    fptr = np.zeros(n + 1, np.uint64)
    fptr[1:] = np.cumsum(k)
    fids = rng.integers(0, n_feat, int(fptr[-1])).astype(np.uint32)
    return fptr, fids


def _ref_embed(fptr, fids, table, w):
    n, d = len(fptr) - 1, table.shape[1]
    out = np.zeros((n, d), np.float32)
    for v in range(n):
        b, e = int(fptr[v]), int(fptr[v + 1])
        if b == e:
            continue
        acc = np.zeros(d, np.float32)
        ws = np.float32(0)
        for f in fids[b:e]:
            wf = np.float32(1) if w is None else np.float32(w[f])
            ws = np.float32(ws + wf)
            acc = acc + (table[f] if w is None else wf * table[f])
        out[v] = acc / ws
    return out


@pytest.mark.parametrize("dims", [64, 100])
@pytest.mark.parametrize("weighted", [False, True])
def test_embed_features_matches_reference_arithmetic(dims, weighted):
    rng = np.random.default_rng(dims + weighted)
    n, n_feat = 400, 250
    fptr, fids = _features(rng, n, n_feat)
    table = rng.standard_normal((n_feat, dims)).astype(np.float32)
    w = None
    if weighted:
        p = rng.random(n_feat).astype(np.float32)
        p /= p.sum()
        w = (np.float32(1e-3) / (np.float32(1e-3) + p)).astype(np.float32)
    got = _native.embed_features(fptr, fids, table, w)
    assert np.array_equal(got, _ref_embed(fptr, fids, table, w))


def _exact(db, q):
    dn = db / np.maximum(np.linalg.norm(db, axis=1, keepdims=True), 1e-300)
    qn = q / np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-300)
    return qn.astype(np.float64) @ dn.astype(np.float64).T


@pytest.mark.parametrize("dims,k", [(32, 10), (100, 16), (256, 10), (256, 32)])
def test_knn_cosine_matches_exact_up_to_bf16(dims, k):
    rng = np.random.default_rng(dims * 100 + k)
    n_db, n_q = 1000, 300
    db = rng.standard_normal((n_db, dims)).astype(np.float32)
    q = db[:n_q].copy()
    idx, sim = _native.knn_cosine(db, q, k, q_self=np.arange(n_q))
    S = _exact(db, q)
    S[np.arange(n_q), np.arange(n_q)] = -np.inf
    kth = -np.sort(-S, axis=1)[:, k - 1]
    assert (idx < n_db).all()
    assert (idx != np.arange(n_q)[:, None]).all()
    assert all(len(set(r)) == k for r in idx.tolist())
    assert (np.diff(sim, axis=1) <= 0).all()
    ex = S[np.arange(n_q)[:, None], idx.astype(np.int64)]
    assert (ex >= kth[:, None] - TOL_BF16).all()
    assert np.abs(ex - sim).max() < TOL_BF16
    top = np.argsort(-S, axis=1)[:, :k]
    overlap = np.mean([len(set(a) & set(b)) / k for a, b in zip(idx.tolist(), top.tolist())])
    assert overlap > 0.9, overlap


def test_knn_cosine_separated_clusters_exact():
    # 40 tight clusters of 25 points: each point's 24 cluster mates are its
    # 24 nearest rows by a wide margin
    rng = np.random.default_rng(7)
    c = rng.standard_normal((40, 64))
    db = (np.repeat(c, 25, axis=0) + 0.01 * rng.standard_normal((1000, 64))).astype(np.float32)
    idx, _ = _native.knn_cosine(db, db, 24, q_self=np.arange(1000))
    want = np.arange(1000) // 25
    assert (idx.astype(np.int64) // 25 == want[:, None]).all()


@pytest.mark.parametrize("k", [5, 20])
def test_knn_cosine_many_tiles_ragged(k):
    # 20000 rows = 78 full 256-row tiles + 32; 700 queries = 5 full query
    # tiles + 60; 192 dims = 3 K blocks, so copy stages wrap inside a tile
    rng = np.random.default_rng(31 + k)
    n_db, n_q, dims = 20000, 700, 192
    db = rng.standard_normal((n_db, dims)).astype(np.float32)
    q = rng.standard_normal((n_q, dims)).astype(np.float32)
    q[:50] = db[19950:20000]                 # some queries sit in the ragged last tile
    selfs = np.full(n_q, np.iinfo(np.uint64).max, np.uint64)
    selfs[:50] = np.arange(19950, 20000)
    idx, sim = _native.knn_cosine(db, q, k, q_self=selfs)
    S = _exact(db, q)
    S[np.arange(50), np.arange(19950, 20000)] = -np.inf
    kth = -np.sort(-S, axis=1)[:, k - 1]
    assert (idx < n_db).all()
    assert all(len(set(r)) == k for r in idx.tolist())
    assert (np.diff(sim, axis=1) <= 0).all()
    ex = S[np.arange(n_q)[:, None], idx.astype(np.int64)]
    assert np.isfinite(ex).all()             # the skipped row never comes back
    assert (ex >= kth[:, None] - TOL_BF16).all()
    assert np.abs(ex - sim).max() < TOL_BF16


def test_knn_cosine_fewer_rows_than_k():
    rng = np.random.default_rng(3)
    db = rng.standard_normal((5, 48)).astype(np.float32)
    q = rng.standard_normal((3, 48)).astype(np.float32)
    idx, sim = _native.knn_cosine(db, q, 8, q_self=np.array([0, 2**64 - 1, 4], np.uint64))
    S = _exact(db, q)
    for i, skip in enumerate([0, None, 4]):
        n_ok = 4 if skip is not None else 5
        assert sorted(idx[i, :n_ok].tolist()) == [j for j in range(5) if j != skip]
        assert (np.diff(sim[i, :n_ok]) <= 0).all()
        assert (idx[i, n_ok:] == 0xFFFFFFFF).all() and np.isneginf(sim[i, n_ok:]).all()
    e_idx, e_sim = _native.knn_cosine(np.zeros((0, 48), np.float32), q, 4)
    assert (e_idx == 0xFFFFFFFF).all() and np.isneginf(e_sim).all()


@pytest.mark.parametrize("weighted", [False, True])
def test_node_embedder_class_translates_vocabularies(weighted):
    # NodeEmbedder.embed_feature_set (lib.rs:2092-2124) through the Python
    # class: feature ids are translated into the embeddings' own vocabulary,
    # features it lacks are skipped, and SIF weights are looked up by the
    # translated row (aggregator.rs:103-110)
    import cloverleaf_gb300 as cl
    from tests._cases import random_problem
    prob = random_problem(8, n=500, n_feat=120, dims=4)
    g = cl.Graph.from_csr(prob["rows"], prob["cols"])
    fs = cl.FeatureSet.from_csr(g, prob["fptr"], prob["fids"], prob["n_feat"])
    rng = np.random.default_rng(9)
    order = rng.permutation(120)[:100]             # 20 features unknown to the embeddings
    ev = cl.Vocab()
    for f in order.tolist():
        ev.get_or_insert("feat", str(f))
    table = rng.standard_normal((100, 48)).astype(np.float32)
    femb = cl.NodeEmbeddings(ev, table)
    agg = cl.FeatureAggregator.Weighted(0.1, fs) if weighted else cl.FeatureAggregator.Averaged()
    out = cl.NodeEmbedder(agg).embed_feature_set(fs, femb)
    tr = np.full(120, -1, np.int64)
    tr[order] = np.arange(100)
    fptr, fids = prob["fptr"], prob["fids"]
    kept_ptr, kept = [0], []
    for v in range(500):
        t = [int(tr[f]) for f in fids[int(fptr[v]):int(fptr[v + 1])] if tr[f] >= 0]
        kept += t
        kept_ptr.append(len(kept))
    w = None
    if weighted:
        a = np.float32(0.1)
        w = a / (a + agg.unigrams[:100])
    want = _ref_embed(np.array(kept_ptr, np.uint64), np.array(kept, np.uint32), table, w)
    assert np.array_equal(out.table, want)
    assert out.vocab_ is fs.vocab_


def test_nearest_neighbors_batch_matches_exact():
    import cloverleaf_gb300 as cl
    rng = np.random.default_rng(21)
    table = rng.standard_normal((3000, 64)).astype(np.float32)
    e = cl.NodeEmbeddings(cl.Vocab.anonymous(3000), table)
    ids, dist = e.nearest_neighbors(table[:200], 5, exclude=np.arange(200))
    S = _exact(table, table[:200])
    S[np.arange(200), np.arange(200)] = -np.inf
    kth = -np.sort(-S, axis=1)[:, 4]
    ex = S[np.arange(200)[:, None], ids.astype(np.int64)]
    assert (ex >= kth[:, None] - TOL_BF16).all()
    assert np.abs((1 - ex) - dist).max() < TOL_BF16
    assert (np.diff(dist, axis=1) >= 0).all()
    with pytest.raises(cl.UnsupportedOption):
        cl.NodeEmbeddings(e.vocab_, table, cl.Distance.Euclidean).nearest_neighbors(table[:2], 3)


def test_knn_cosine_argument_limits():
    rng = np.random.default_rng(5)
    db = rng.standard_normal((300, 1)).astype(np.float32)        # one dimension: cosine is the sign
    q = np.array([[2.0], [-3.0]], np.float32)
    idx, sim = _native.knn_cosine(db, q, 4)
    assert (np.sign(db[idx[0].astype(np.int64), 0]) == 1).all() and np.allclose(sim[0], 1.0)
    assert (np.sign(db[idx[1].astype(np.int64), 0]) == -1).all() and np.allclose(sim[1], 1.0)
    for bad in (dict(k=0), dict(k=33)):
        with pytest.raises(_native.NativeError):
            _native.knn_cosine(db, q, bad["k"])
    with pytest.raises(_native.NativeError):
        _native.knn_cosine(np.zeros((4, 257), np.float32), np.zeros((1, 257), np.float32), 2)
    # zero rows have similarity 0 to everything and are still ranked
    z = np.zeros((3, 8), np.float32)
    idx, sim = _native.knn_cosine(z, rng.standard_normal((2, 8)).astype(np.float32), 3)
    assert sorted(idx[0].tolist()) == [0, 1, 2] and np.allclose(sim, 0.0)
