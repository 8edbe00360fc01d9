"""The Chung-Lu workloads end to end: held-out-edge recall@10
(scripts/evaluate.py:29-61) of both GPU forms within 1 point of the CPU
restatement of the reference loop after the same passes, and per-batch
parity of the plain FP32 form on the bipartite 1M-node workload with its
U[1, 5] edge weights turned into CDF rows (src/graph.rs:664-691).
"""
import numpy as np
import pytest

from cloverleaf_gb300 import _native, datagen, evaluate
from tests._cases import dense_from_sparse, rel_err

pytestmark = pytest.mark.gpu


def gpu_train(w, rows, cols, form, passes):
    ep = w["ep"]
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = ep["dims"], ep["negatives"], _native.LOSS_STARSPACE, ep["gamma"]
    cfg.batch_size, cfg.alpha, cfg.passes, cfg.valid_pct = w["batch"], ep["alpha"], passes, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.form = form
    ctx = _native.Context(cfg)
    ctx.upload_graph(rows, cols, None)
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    ctx.set_table(None)
    stats = ctx.train(passes)
    table = ctx.get_table(w["n_feat"], ep["dims"])
    ctx.close()
    return table, stats


def cpu_train(oracle, w, rows, cols, weights, passes):
    ep = w["ep"]
    table, st = oracle.train(rows, cols, weights, w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                             alpha=ep["alpha"], loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"],
                             negatives=ep["negatives"], batch_size=w["batch"], passes=passes,
                             max_nodes=(oracle.SAMPLE_FIXED, float(ep["max_nodes"])), threads=0)
    return table


@pytest.mark.parametrize("name,scale", [("cl10m", 0.05), ("cl1m", 0.2)])
def test_heldout_recall_matches_cpu_reference(oracle, name, scale):
    # A shrunken workload keeps the full one's batches per pass with a batch
    # shrunk in proportion (next power of two): the CPU restatement runs its
    # batches concurrently on every host core with hogwild writes, as the
    # reference does, and with the full batch size a 5% graph has so few
    # batches per pass that most of them would read a stale table.
    w = datagen.workload(name, scale=scale)
    w["batch"] = 1 << int(np.ceil(np.log2(w["ep"]["batch_size"] * scale)))
    passes = w["ep"]["passes"]
    rows, cols, wts, test = evaluate.holdout_edges(w["rows"], w["cols"], w["weights"], 0.01, seed=5, max_test=5000)
    assert len(test) >= 2000
    res, tables = {}, {}
    for form, fid in (("fused", _native.FORM_FUSED_BF16), ("plain", _native.FORM_PLAIN_FP32)):
        table, stats = gpu_train(w, rows, cols, fid, passes)
        assert np.isfinite(table).all() and stats[-1]["kept_anchors"] > 0
        tables[form] = table
        res[form] = evaluate.heldout_recall(w["fptr"], w["fids"], table, test)
    assert not np.array_equal(tables["fused"], tables["plain"])
    res["cpu"] = evaluate.heldout_recall(w["fptr"], w["fids"], cpu_train(oracle, w, rows, cols, wts, passes), test)
    print(name, {k: (round(v["recall"], 4), round(v["auc"], 4)) for k, v in res.items()},
          "max |fused - plain|", float(np.abs(tables["fused"] - tables["plain"]).max()))
    for form in ("fused", "plain"):
        assert abs(res[form]["recall"] - res["cpu"]["recall"]) <= 0.01, res
        # held-out edges vs random pairs: the CPU restatement's own spread
        # over seeds is about 0.003 at these sizes
        assert abs(res[form]["auc"] - res["cpu"]["auc"]) <= 0.02, res


@pytest.fixture(scope="module")
def cl1m():
    w = datagen.workload("cl1m")
    w["cdf"] = _native.cdf_convert(w["rows"], w["weights"].copy())
    return w


@pytest.mark.parametrize("weighted,chunk", [(False, "128"), (True, "128"), (False, "32")])
def test_cl1m_batches_plain_fp32_parity(oracle, monkeypatch, cl1m, weighted, chunk):
    monkeypatch.setenv("EP_REDUCE_CHUNK", chunk)
    w = cl1m
    ep = w["ep"]
    n = len(w["rows"]) - 1
    assert n == 1_000_000 and w["weights"].min() >= 1.0 and w["weights"].max() <= 5.0
    # bipartite: users [0, n/2) only link to items [n/2, n)
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(w["rows"]).astype(np.int64))
    assert ((src < n // 2) != (w["cols"] < n // 2)).all()
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = ep["dims"], ep["negatives"], _native.LOSS_STARSPACE, ep["gamma"]
    cfg.batch_size, cfg.alpha, cfg.passes, cfg.valid_pct = ep["batch_size"], ep["alpha"], 1, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.weighted_neighbor_averaging = int(weighted)
    cfg.weighted_neighbor_sampling = int(weighted)
    ctx = _native.Context(cfg)
    ctx.upload_graph(w["rows"], w["cols"], w["cdf"])
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    rng = np.random.default_rng(8)
    table = (rng.uniform(-1, 1, (w["n_feat"], ep["dims"]))).astype(np.float32)
    table /= np.linalg.norm(table, axis=1, keepdims=True)
    ctx.set_table(table)
    K = ep["max_nodes"]
    for step in (1, 2):
        anchors = rng.integers(0, n, ep["batch_size"]).astype(np.uint32)
        cnt, nbr, nw, neg = ctx.sample(anchors, step, K)
        deg = np.diff(w["rows"]).astype(np.int64)[anchors]
        assert (cnt == np.minimum(deg, K)).all()
        if weighted:
            # weights scale * p_j * deg (model.rs:373-375, graph.rs:630-661),
            # p_j the CDF differences of the chosen positions
            for a in range(len(anchors)):
                s, e = int(w["rows"][anchors[a]]), int(w["rows"][anchors[a] + 1])
                row = w["cols"][s:e]
                cdf = w["cdf"][s:e]
                p = np.diff(np.concatenate([[np.float32(0)], cdf])).astype(np.float32)
                r = int(cnt[a])
                sw = np.float32(deg[a]) / np.float32(r)
                pos = np.array([np.nonzero(row == x)[0][0] for x in nbr[a, :r]])
                np.testing.assert_allclose(nw[a, :r], sw * p[pos] * np.float32(deg[a]), rtol=1e-6)
        nbr_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint32)
        flat = np.concatenate([nbr[a, :cnt[a]] for a in range(len(anchors))])
        flw = np.concatenate([nw[a, :cnt[a]] for a in range(len(anchors))])
        s = _native.Context.samples(anchors, nbr_ptr, flat, flw, neg)
        gl, gst, ids, grow = ctx.batch_grad(s, w["n_feat"], ep["dims"])
        ol, ost, og, ot = oracle.batch(w["fptr"], w["fids"], w["n_feat"], table, w["rows"], anchors, nbr_ptr, flat,
                                       flw, neg, oracle.loss_cfg(loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"]),
                                       "f64")
        assert (gst == ost).all()
        kept = ost == 0
        assert kept.sum() > 0.5 * len(anchors)
        assert rel_err(gl[kept], ol[kept]) < 1e-4
        g, t = dense_from_sparse(ids, grow, w["n_feat"], ep["dims"])
        assert (t == ot).all()
        assert rel_err(g, og) < 1e-4
    ctx.close()
