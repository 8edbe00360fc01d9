"""End-to-end training on the GPU through the drop-in Python API, compared
with the oracle's CPU training loop (community recall@10 within 1 point)."""
import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import _native, datagen
from tests._eval import community_recall

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sbm10k():
    return datagen.workload("sbm10k")


def gpu_learn(w, loss, form, seed=20222022, passes=None, valid_pct=0.0, **extra):
    ep = w["ep"]
    g = cl.Graph.from_csr(w["rows"], w["cols"], w["weights"])
    fs = cl.FeatureSet.from_csr(g, w["fptr"], w["fids"], w["n_feat"])
    lossobj = cl.EPLoss.starspace(ep["gamma"], ep["negatives"]) if loss == "starspace" else \
        cl.EPLoss.margin(ep["gamma"], ep["negatives"])
    prop = cl.EmbeddingPropagator(alpha=ep["alpha"], loss=lossobj, batch_size=ep["batch_size"], dims=ep["dims"],
                                  passes=passes or ep["passes"], seed=seed, max_nodes=ep["max_nodes"],
                                  valid_pct=valid_pct, indicator=False, form=form, **extra)
    emb = prop.learn_features(g, fs)
    return emb, prop.last_stats


def oracle_learn(oracle, w, loss):
    ep = w["ep"]
    table, st = oracle.train(w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                             alpha=ep["alpha"], loss=oracle.LOSS_STARSPACE if loss == "starspace" else
                             oracle.LOSS_MARGIN, gamma=ep["gamma"], negatives=ep["negatives"],
                             batch_size=ep["batch_size"], passes=ep["passes"],
                             max_nodes=(oracle.SAMPLE_FIXED, ep["max_nodes"]), threads=0)
    return table


@pytest.mark.parametrize("form", ["plain", "fused"])
@pytest.mark.parametrize("loss", ["starspace", "margin"])
def test_recall_matches_cpu_reference(oracle, sbm10k, loss, form):
    w = sbm10k
    emb, stats = gpu_learn(w, loss, form)
    assert emb.table.shape == (w["n_feat"], w["ep"]["dims"])
    assert np.isfinite(emb.table).all()
    assert len(stats) == w["ep"]["passes"]
    assert stats[-1]["train_loss"] < stats[0]["train_loss"]
    r_gpu = community_recall(w["fptr"], w["fids"], emb.table, w["community"])
    r_cpu = community_recall(w["fptr"], w["fids"], oracle_learn(oracle, w, loss), w["community"])
    assert abs(r_gpu - r_cpu) <= 0.01, (r_gpu, r_cpu)


def test_training_is_deterministic(sbm10k):
    a, _ = gpu_learn(sbm10k, "starspace", "fused", passes=2)
    b, _ = gpu_learn(sbm10k, "starspace", "fused", passes=2)
    assert np.array_equal(a.table, b.table)
    c, _ = gpu_learn(sbm10k, "starspace", "plain", passes=2)
    d, _ = gpu_learn(sbm10k, "starspace", "plain", passes=2)
    assert np.array_equal(c.table, d.table)


def test_pass_stats_and_validation(sbm10k):
    w = sbm10k
    emb, stats = gpu_learn(w, "starspace", "fused", passes=2, valid_pct=0.1)
    n_train = w["rows"].shape[0] - 1 - int(np.float32(10_000) * np.float32(0.1))
    for s in stats:
        assert s["anchors"] == n_train
        assert s["batches"] == -(-n_train // w["ep"]["batch_size"])
        assert 0 < s["kept_anchors"] <= s["anchors"]
        assert s["gathered_rows"] <= s["items"]
        assert 0 < s["unique_rows"] <= w["n_feat"] * s["batches"]
        assert s["alg_bytes"] > 0 and s["ms"] > 0
        assert np.isfinite(s["valid_loss"]) and s["valid_loss"] > 0


def test_drop_in_api_strings():
    # the reference's own usage: GraphBuilder + FeatureSet with string ids
    b = cl.GraphBuilder()
    rng = np.random.default_rng(0)
    for i in range(200):
        for j in rng.integers(0, 200, 3):
            if i != j:
                b.add_edge(("user", str(i)), ("user", str(int(j))), 1.0, cl.EdgeType.Undirected)
    g = b.build_graph()
    fs = cl.FeatureSet.new_from_graph(g)
    for i in range(0, 200, 2):   # odd nodes stay featureless
        fs.set_features(("user", str(i)), [("feat", f"t{i % 7}"), ("feat", f"t{i % 11}")])
    ep = cl.EmbeddingPropagator(alpha=0.05, loss=cl.EPLoss.starspace(0.5, 3), batch_size=32, dims=16, passes=3,
                                max_nodes=5, indicator=False)
    emb = ep.learn_features(g, fs)
    # fill_missing_nodes gave every odd node its own ("node", id) feature
    assert fs.get_features(("user", "1"))[0][0] == "node"
    assert emb.len() == fs.num_features() and emb.dims() == 16
    assert emb.contains(("feat", "t3"))
    nn = emb.nearest_neighbor(emb.get_embedding(("feat", "t3")), 3)
    assert nn[0][0] == ("feat", "t3")


def test_warm_start_moves_table_out(sbm10k):
    w = sbm10k
    emb, _ = gpu_learn(w, "starspace", "plain", passes=1)
    init = emb.table.copy()
    ep = w["ep"]
    g = cl.Graph.from_csr(w["rows"], w["cols"], w["weights"])
    fs = cl.FeatureSet.from_csr(g, w["fptr"], w["fids"], w["n_feat"])
    prop = cl.EmbeddingPropagator(alpha=ep["alpha"], loss=cl.EPLoss.starspace(0.5, 5), batch_size=256, dims=64,
                                  passes=1, max_nodes=10, valid_pct=0.0, indicator=False)
    out = prop.learn_features(g, fs, emb)
    assert emb.dims() == 0                 # moved out, as lib.rs:1337-1341
    assert out.table.shape == init.shape
    assert not np.array_equal(out.table, init)


def test_unsupported_options_raise():
    with pytest.raises(NotImplementedError):
        cl.EmbeddingPropagator(attention=8)
    with pytest.raises(ValueError):
        cl.EmbeddingPropagator(max_features=-1.0)


def test_large_chung_lu_batches():
    # 2% of the 10M-node workload: same degree and feature distributions
    w = datagen.workload("cl10m", scale=0.02)
    cfg = _native.default_config()
    ep = w["ep"]
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = ep["dims"], ep["negatives"], _native.LOSS_STARSPACE, ep["gamma"]
    cfg.batch_size, cfg.alpha, cfg.passes, cfg.valid_pct = 2048, ep["alpha"], 1, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.form = _native.FORM_FUSED_BF16
    ctx = _native.Context(cfg)
    ctx.upload_graph(w["rows"], w["cols"], None)
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    ctx.set_table(None)
    s1 = ctx.train_batches(10)
    ctx.train_batches(150)
    s2 = ctx.train_batches(10)
    assert s1["kept_anchors"] > 0 and s1["nan_anchors"] == 0
    assert s2["train_loss"] < s1["train_loss"]
    t = ctx.get_table(w["n_feat"], ep["dims"])
    assert np.isfinite(t).all()


def _cl_ctx(w, form=_native.FORM_FUSED_BF16, autotune=0):
    return _cl_ctx_cfg(w, form=form, autotune=autotune)


def _cl_ctx_cfg(w, form=_native.FORM_FUSED_BF16, autotune=0, use_graphs=1):
    cfg = _native.default_config()
    cfg.use_graphs = use_graphs
    ep = w["ep"]
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = ep["dims"], ep["negatives"], _native.LOSS_STARSPACE, ep["gamma"]
    cfg.batch_size, cfg.alpha, cfg.passes, cfg.valid_pct = 2048, ep["alpha"], 1, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.form, cfg.autotune = form, autotune
    ctx = _native.Context(cfg)
    ctx.upload_graph(w["rows"], w["cols"], None)
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    ctx.set_table(None)
    return ctx


def test_multi_batch_graph_matches_single_batch_graphs(monkeypatch):
    # runs of 16 batches replay one graph; the result must equal one graph
    # replay per batch bit for bit (same kernels, same order)
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for gb in ("16", "1"):
        monkeypatch.setenv("EP_GRAPH_BATCHES", gb)
        ctx = _cl_ctx(w)
        assert ctx.tuning()[3] == int(gb)
        ctx.train_batches(37)
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("form", [_native.FORM_FUSED_BF16, _native.FORM_PLAIN_FP32])
@pytest.mark.parametrize("ctas", ["1", "608"])
def test_persistent_reducer_gives_the_same_table(monkeypatch, form, ctas):
    # warps taking reducer chunks from a work counter (down to a single CTA)
    # reduce every chunk as the one-warp-per-chunk grid does
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for r in ("0", ctas):
        monkeypatch.setenv("EP_RED_CTAS", r)
        ctx = _cl_ctx(w, form=form)
        st = ctx.train_batches(23)
        assert st["kept_anchors"] > 0
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("warps", ["1", "2"])
def test_sampler_cta_size_gives_the_same_table(monkeypatch, warps):
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for g in ("8", warps):
        monkeypatch.setenv("EP_SAMPLE_WARPS", g)
        ctx = _cl_ctx(w)
        ctx.train_batches(19)
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("warps", ["1", "2", "4"])
def test_gather_cta_size_gives_the_same_table(monkeypatch, warps):
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for g in ("8", warps):
        monkeypatch.setenv("EP_GATHER_WARPS", g)
        for graphs in (1, 0):
            ctx = _cl_ctx_cfg(w, use_graphs=graphs)
            ctx.train_batches(19)
            tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert all(np.array_equal(tables[0], t) for t in tables[1:])


def test_five_cta_queue_reducer_gives_the_same_table(monkeypatch):
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for q in ("4", "5"):
        monkeypatch.setenv("EP_QUEUE_CTAS", q)
        ctx = _cl_ctx(w)
        assert ctx.launch_shape()["queue_ctas_per_sm"] == int(q)
        ctx.train_batches(29)
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("mode", ["0", "1", "3"])
def test_adam_placements_give_the_same_table(monkeypatch, mode):
    # the fused form's Adam placements -- per row as each feature closes (0),
    # a separate kernel over dense gradient rows (1), the per-warp queue (2,
    # the reference point) and the warp-specialised ring with bulk copies (3)
    # -- apply the same update to the same reduced rows: equal tables, bit for bit
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for m in ("2", mode):
        monkeypatch.setenv("EP_FUSED_MODE", m)
        ctx = _cl_ctx(w)
        assert ctx.tuning()[2] == int(m)
        st = ctx.train_batches(37)
        assert st["kept_anchors"] > 0
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("ctas", ["1", "152", "608"])
def test_persistent_gather_gives_the_same_table(monkeypatch, ctas):
    # the staged gather as a persistent grid whose warps take anchors from a
    # work queue (any grid size, down to one CTA) computes every anchor as
    # the one-warp-per-anchor grid does
    w = datagen.workload("cl10m", scale=0.005)
    tables = []
    for g in ("0", ctas):
        monkeypatch.setenv("EP_GATHER_CTAS", g)
        for graphs in (1, 0):
            ctx = _cl_ctx_cfg(w, use_graphs=graphs)
            ctx.train_batches(19)
            tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert all(np.array_equal(tables[0], t) for t in tables[1:])


@pytest.mark.parametrize("shape", [("12", "4", "32"), ("6", "2", "4"), ("2", "14", "56"), ("1", "1", "2"),
                                   ("15", "1", "3")])
def test_ring_shapes_give_the_same_table(monkeypatch, shape):
    # reducing warps, Adam warps and slots per CTA of the ring change the
    # schedule only; tiny rings make every slot wrap many times
    w = datagen.workload("cl10m", scale=0.005)
    monkeypatch.setenv("EP_FUSED_MODE", "2")
    ref = _cl_ctx(w)
    ref.train_batches(21)
    want = ref.get_table(w["n_feat"], w["ep"]["dims"])
    monkeypatch.setenv("EP_FUSED_MODE", "3")
    for k, v in zip(("EP_RING_PW", "EP_RING_CW", "EP_RING_SLOTS"), shape):
        monkeypatch.setenv(k, v)
    ctx = _cl_ctx(w)
    ctx.train_batches(21)
    assert np.array_equal(ctx.get_table(w["n_feat"], w["ep"]["dims"]), want)


def test_graph_replays_match_stream_launches():
    # captured batches run k_batch_end on a side branch beside the sort and
    # reduction; the table and the pass statistics must equal those of the
    # same batches launched one kernel after another on one stream
    w = datagen.workload("cl10m", scale=0.005)
    out = []
    for graphs in (1, 0):
        ctx = _cl_ctx_cfg(w, use_graphs=graphs)
        st = ctx.train_batches(37)
        out.append((ctx.get_table(w["n_feat"], w["ep"]["dims"]), st))
    assert np.array_equal(out[0][0], out[1][0])
    same = ("pass", "batches", "train_loss", "lr_last", "anchors", "kept_anchors", "items", "gathered_rows",
            "unique_rows", "sampled_neighbors")
    assert {k: out[0][1][k] for k in same} == {k: out[1][1][k] for k in same}


def test_graph_replays_match_stream_launches_with_direct_gathers():
    # anchors too big for the staged gather's tables take the direct path,
    # in replayed graphs with their items from k_fwd_emit's direct walk
    from tests._cases import random_problem
    prob = random_problem(97, n=3000, n_feat=20000, dims=64, deg=(4, 30), feats=(10, 40))
    tables = []
    for graphs in (1, 0):
        cfg = _native.default_config()
        cfg.use_graphs = graphs
        cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = 64, 10, _native.LOSS_STARSPACE, 0.5
        cfg.batch_size, cfg.passes, cfg.valid_pct = 256, 1, 0.0
        cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, 25.0
        ctx = _native.Context(cfg)
        ctx.upload_graph(prob["rows"], prob["cols"], None)
        ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
        ctx.set_table(None)
        st = ctx.train_batches(20)
        assert st["kept_anchors"] > 0
        tables.append(ctx.get_table(prob["n_feat"], 64))
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("form", [_native.FORM_FUSED_BF16, _native.FORM_PLAIN_FP32])
@pytest.mark.parametrize("level", [1, 2])
def test_autotune_picks_a_candidate_and_trains(form, level):
    w = datagen.workload("cl10m", scale=0.01)
    ctx = _cl_ctx(w, form=form, autotune=level)
    assert ctx.tuning()[0] is False
    s1 = ctx.train_batches(260)          # the candidates' batches (200 at most), then more
    shape = ctx.launch_shape()
    tuned, chunk, mode, _ = ctx.tuning()
    assert tuned and shape["tuned"] and shape["autotune"] == level
    assert chunk == 128 if level == 1 else chunk in (64, 128, 256)
    if form == _native.FORM_FUSED_BF16:
        assert mode in ((2, 3) if level == 1 else (1, 2, 3))
    assert shape["gather_ctas"] in (0, 304, 456) and shape["gather_warps"] in (2, 4, 8)
    ctx.train_batches(120)
    s2 = ctx.train_batches(10)
    assert s2["train_loss"] < s1["train_loss"]
    assert np.isfinite(ctx.get_table(w["n_feat"], w["ep"]["dims"])).all()
    # a second context on the same workload starts with the remembered choice
    again = _cl_ctx(w, form=form, autotune=level)
    again.train_batches(1)
    assert again.launch_shape() == shape


def test_level_one_tuning_keeps_results_identical():
    # level 1 only chooses between launch shapes that give the same bits
    w = datagen.workload("cl10m", scale=0.01)
    tables = []
    for level in (0, 1):
        ctx = _cl_ctx(w, autotune=level)
        ctx.train_batches(110)
        tables.append(ctx.get_table(w["n_feat"], w["ep"]["dims"]))
    assert np.array_equal(tables[0], tables[1])
