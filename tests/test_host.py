"""Host-side logic and the C-ABI library, without a GPU."""
import glob
import os
import re

import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import _native, datagen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(ep_\w+|epg_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(native):
    names = declared_functions()
    assert {"ep_create", "ep_train", "ep_batch_grad", "ep_destroy", "epg_chung_lu"} <= names
    gen = datagen.lib()
    for n in names:
        assert hasattr(gen if n.startswith("epg_") else native, n), n
    bound = set(_native.SIGNATURES) | set(datagen.SIGNATURES)
    assert names == bound, names ^ bound


def test_generators_live_apart_from_the_trainer():
    # the generator library exports no trainer entry point, and loading it
    # does not load the trainer library
    import subprocess
    import sys

    code = ("import sys; sys.path.insert(0, %r); from cloverleaf_gb300 import datagen; "
            "w = datagen.workload('sbm1k'); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libep_datagen.so' in maps and 'libep_gb300.so' not in maps, 'trainer loaded'; "
            "assert not hasattr(datagen.lib(), 'ep_create')" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_config_defaults_match_reference(native):
    cfg = _native.default_config()
    # src/lib.rs:1262-1274
    assert cfg.abi_version == _native.ABI_VERSION
    assert cfg.alpha == pytest.approx(0.9) and cfg.batch_size == 50 and cfg.dims == 100 and cfg.passes == 100
    assert cfg.loss == _native.LOSS_MARGIN and cfg.gamma == 1.0 and cfg.negatives == 1
    assert cfg.valid_pct == pytest.approx(0.1) and cfg.seed == 20222022 and cfg.hard_negatives == 0


def test_create_rejects_bad_config(native):
    cfg = _native.default_config()
    cfg.dims = 0
    with pytest.raises(_native.NativeError) as e:
        _native.Context(cfg)
    assert e.value.code == -1
    cfg = _native.default_config()
    cfg.max_features_kind, cfg.max_features = _native.SAMPLE_PROB, 1.5
    with pytest.raises(_native.NativeError) as e:
        _native.Context(cfg)
    assert e.value.code == -1
    for loss, restart in ((_native.LOSS_PPR, 1.5), (_native.LOSS_PPR, -0.1), (9, 0.5)):
        cfg = _native.default_config()
        cfg.loss, cfg.ppr_restart_p = loss, restart
        with pytest.raises(_native.NativeError) as e:
            _native.Context(cfg)
        assert e.value.code == -1


def test_create_without_device_reports_it(native):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(_native.NativeError) as e:
        _native.Context(_native.default_config())
    assert e.value.code == -7


@pytest.mark.parametrize("dedup", [True, False])
def test_native_csr_builder_matches_oracle(oracle, dedup):
    rng = np.random.default_rng(4 + dedup)
    for trial in range(5):
        m = int(rng.integers(1, 400))
        src = rng.integers(0, 60, m)
        dst = rng.integers(0, 60, m)
        w = rng.uniform(0, 3, m).astype(np.float32)
        r1, c1, w1 = _native.csr_from_edges(src, dst, w, dedup)
        r2, c2, w2 = oracle.csr_from_edges(list(zip(src.tolist(), dst.tolist(), w.tolist())), dedup)
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2.astype(np.uint32))
        assert np.array_equal(w1, w2)
        assert np.array_equal(_native.cdf_convert(r1, w1), oracle.cdf_convert(r2, w2))


def test_graph_builder_reference_cases(native):
    # graph.rs:697-705 edges through the drop-in GraphBuilder
    b = cl.GraphBuilder()
    for f, t, w in [(0, 1, 1.0), (1, 1, 3.0), (1, 2, 2.0), (2, 0, 2.5), (1, 0, 10.0)]:
        b.add_edge(("n", str(f)), ("n", str(t)), w, cl.EdgeType.Directed)
    g = b.build_graph()
    assert g.nodes() == 3 and g.edges() == 5 and repr(g) == "Graph<Nodes=3, Edges=5>"
    names, w = g.get_edges(("n", "1"), normalized=True)
    assert names == [("n", "0"), ("n", "1"), ("n", "2")]
    np.testing.assert_allclose(w, [10 / 15, 3 / 15, 2 / 15], atol=1e-6)
    assert cl.GraphBuilder().build_graph() is None
    u = cl.GraphBuilder()
    u.add_edge(("a", "x"), ("a", "y"), 2.0, cl.EdgeType.Undirected)
    gu = u.build_graph()
    assert gu.edges() == 2 and gu.get_edges(("a", "y"))[0] == [("a", "x")]


def test_feature_set_semantics(native):
    b = cl.GraphBuilder()
    b.add_edge(("u", "a"), ("u", "b"), 1.0, cl.EdgeType.Undirected)
    b.add_edge(("u", "b"), ("u", "c"), 1.0, cl.EdgeType.Undirected)
    g = b.build_graph()
    fs = cl.FeatureSet.new_from_graph(g)
    fs.set_features(("u", "a"), [("feat", "x"), ("feat", "y")])
    fs.set_features(("u", "c"), [("feat", "y")])
    assert fs.num_features() == 2 and fs[0] == ("feat", "x") and fs[-1] == ("feat", "y")
    fs.fill_missing_nodes()           # feature_store.rs:83-89
    assert fs.get_features(("u", "b")) == [("node", "1")]
    fptr, fids = fs.to_csr()
    assert fptr.tolist() == [0, 2, 3, 4] and fids.tolist() == [0, 1, 2, 1]
    pruned = fs.prune_min_count(2)
    assert pruned.get_features(("u", "a")) == [("feat", "y")]
    with pytest.raises(KeyError):
        fs.get_features(("u", "zz"))
    with pytest.raises(IndexError):
        fs[10]


def test_sample_parsing():
    # Sample::new (utils.rs:173-184)
    from cloverleaf_gb300.ep import _sample

    assert _sample(None, "x") == (_native.SAMPLE_ALL, 0.0)
    assert _sample(0.25, "x") == (_native.SAMPLE_PROB, 0.25)
    assert _sample(10, "x") == (_native.SAMPLE_FIXED, 10.0)
    assert _sample(2.7, "x") == (_native.SAMPLE_FIXED, 2.0)
    with pytest.raises(ValueError):
        _sample(-1, "x")
    assert cl.EPLoss.starspace(0.5, 0).negatives == 1      # negatives.max(1), lib.rs:1034
    assert cl.EPLoss.margin(0.5).negatives == 1


def test_generators_are_deterministic(native):
    a = datagen.workload("sbm10k")
    b = datagen.workload("sbm10k")
    for k in ("rows", "cols", "fptr", "fids", "community"):
        assert np.array_equal(a[k], b[k])
    rows, cols = a["rows"], a["cols"]
    n = len(rows) - 1
    assert n == 10_000 and (np.diff(rows) > 0).all()            # no isolated nodes
    deg = np.diff(rows)
    assert 9.0 < deg.mean() < 11.0                              # 8 intra + 2 inter
    # symmetric, sorted, no self loops
    src = np.repeat(np.arange(n), deg.astype(np.int64))
    assert (src != cols).all()
    key = np.sort(src.astype(np.int64) * n + cols)
    rkey = np.sort(cols.astype(np.int64) * n + src)
    assert np.array_equal(key, rkey)
    comm = a["community"]
    intra = (comm[src] == comm[cols]).mean()
    assert 0.75 < intra < 0.85
    k = np.diff(a["fptr"])
    assert k.min() >= 4 and k.max() <= 8


def test_chung_lu_small(native):
    w = datagen.workload("cl10m", scale=0.005)
    rows, cols = w["rows"], w["cols"]
    deg = np.diff(rows)
    assert deg.min() >= 1 and deg.max() <= 1.2e4
    k = np.diff(w["fptr"])
    assert k.min() >= 1 and k.max() <= 32
    assert w["fids"].max() < w["n_feat"]
    # Zipf head: the most common slot is slot 0
    assert np.bincount(w["fids"]).argmax() == 0
    again = datagen.workload("cl10m", scale=0.005)
    assert np.array_equal(again["cols"], cols) and np.array_equal(again["fids"], w["fids"])


def test_embeddings_io_roundtrip(tmp_path):
    v = cl.Vocab()
    for i in range(5):
        v.get_or_insert("feat", f"f{i}")
    t = np.arange(15, dtype=np.float32).reshape(5, 3) / 7
    e = cl.NodeEmbeddings(v, t)
    p = str(tmp_path / "e.txt")
    e.save(p)
    e2 = cl.NodeEmbeddings.load(p, cl.Distance.Cosine)
    assert list(e2.vocab()) == list(e.vocab())
    np.testing.assert_array_equal(e2.table, e.table)
    nn = e.nearest_neighbor(t[2], 2)
    assert nn[0][0] == ("feat", "f2")
    assert cl.Distance.Euclidean.compute([1, 3], [3, 5]) == pytest.approx(8 ** 0.5)   # loss.rs:250-255


def test_evaluation_wrappers_check_shapes():
    # shape errors are caught before any host array is read past its end
    rows = np.array([0, 1, 2], np.uint64)
    cols = np.array([1, 0], np.uint32)
    cdf = np.ones(2, np.float32)
    with pytest.raises(ValueError):
        _native.align(rows, cols, cdf, np.zeros((3, 4), np.float32))
    with pytest.raises(ValueError):
        _native.align(rows, cols, cdf[:1], np.zeros((2, 4), np.float32))
    with pytest.raises(ValueError):
        _native.knn_cosine(np.zeros((5, 8), np.float32), np.zeros((2, 7), np.float32), 3)
    with pytest.raises(ValueError):
        _native.knn_cosine(np.zeros((5, 8), np.float32), np.zeros((2, 8), np.float32), 3, q_self=[0])
    with pytest.raises(ValueError):
        _native.embed_features(np.array([0, 3], np.uint64), np.array([0, 1], np.uint32), np.zeros((4, 8), np.float32))
