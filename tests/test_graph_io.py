"""Graph text files (GraphReader::load, src/io.rs:270-323; Graph::save,
src/lib.rs:414-430) through the native parser, vocabulary and writer.  No
GPU."""
import gzip

import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import _native
from cloverleaf_gb300.graph import NativeVocab


def _edges_tsv(path, lines, gz=False):
    opener = gzip.open if gz else open
    with opener(path, "wt", newline="") as f:
        f.write("".join(lines))


def _restated_load(lines, undirected, weighted):
    """GraphReader::load: ids in first-seen order (from, then to, per line),
    both directions for an undirected graph; CSR rows in source order with
    the edges of one source in input order; weights as per-row CDFs."""
    ids, names, edges = {}, [], []
    for ln in lines:
        p = ln.rstrip("\r\n").split("\t")
        a = ids.setdefault((p[0], p[1]), len(ids))
        if a == len(names):
            names.append((p[0], p[1]))
        b = ids.setdefault((p[2], p[3]), len(ids))
        if b == len(names):
            names.append((p[2], p[3]))
        w = np.float32(float(p[4])) if weighted else np.float32(1)
        edges.append((a, b, w))
        if undirected:
            edges.append((b, a, w))
    return names, edges


@pytest.mark.parametrize("undirected", [True, False])
@pytest.mark.parametrize("weighted", [True, False])
def test_load_matches_restatement(tmp_path, undirected, weighted):
    rng = np.random.default_rng(5)
    lines = []
    for _ in range(500):
        a, b = rng.integers(0, 60, 2)
        lines.append(f"{'ui'[a % 2]}\tn{a}\t{'ui'[b % 2]}\tn{b}\t{rng.uniform(0.5, 3):.4f}\n")
    p = str(tmp_path / "g.tsv")
    _edges_tsv(p, lines)
    et = cl.EdgeType.Undirected if undirected else cl.EdgeType.Directed
    g = cl.Graph.load(p, et, weighted=weighted)
    names, edges = _restated_load(lines, undirected, weighted)
    assert isinstance(g.vocab_, NativeVocab) and list(g.vocab_) == names
    src = np.array([e[0] for e in edges], np.uint32)
    dst = np.array([e[1] for e in edges], np.uint32)
    w = np.array([e[2] for e in edges], np.float32)
    rows, cols, wr = _native.csr_from_edges(src, dst, w, False)
    assert np.array_equal(g.rows, rows) and np.array_equal(g.cols, cols)
    assert np.array_equal(g.weights, _native.cdf_convert(rows, wr))


def test_load_skip_rows_gzip_crlf_blank_lines(tmp_path):
    p = str(tmp_path / "g.tsv.gz")
    _edges_tsv(p, ["from_type\tfrom\tto_type\tto\tweight\r\n", "a\t1\tb\t2\t2.5\r\n", "\r\n",
                   "b\t2\ta\t3\t+1e0\r\n"], gz=True)
    g = cl.Graph.load(p, cl.EdgeType.Directed, skip_rows=1)
    assert list(g.vocab_) == [("a", "1"), ("b", "2"), ("a", "3")]
    assert g.nodes() == 3 and g.edges() == 2
    assert g.vocab_.get_node_id("b", "2") == 1 and g.vocab_.get_node_id("b", "9") is None
    with pytest.raises(ValueError):
        cl.Graph.load(p, cl.EdgeType.Directed)        # the header's weight is not a number
    assert cl.Graph.load(p, cl.EdgeType.Directed, weighted=False).edges() == 3


@pytest.mark.parametrize("line", ["a\t1\tb\t2\n", "a\t1\tb\t2\t1.0\textra\n", "a\t1\tb\t2\tx\n", "a\t1\tb\t2\t\n"])
def test_load_rejects_malformed_lines(tmp_path, line):
    p = str(tmp_path / "bad.tsv")
    _edges_tsv(p, ["a\t0\tb\t0\t1\n", line])
    with pytest.raises(ValueError, match="Malformed graph file"):
        cl.Graph.load(p, cl.EdgeType.Directed)


def test_save_format_and_round_trip(tmp_path):
    b = cl.GraphBuilder()
    for f, t, w in [(("u", "x"), ("i", "y"), 1.0), (("u", "x"), ("i", "z"), 2.0), (("u", "w"), ("i", "y"), 3.0)]:
        b.add_edge(f, t, w, cl.EdgeType.Undirected)
    g = b.build_graph()
    p = str(tmp_path / "g.tsv")
    g.save(p)
    text = open(p).read().splitlines()
    # transition probabilities as Rust prints an f32: 1/3 -> 0.33333334, 1.0 -> 1
    assert "u\tx\ti\ty\t0.33333334" in text and "u\tx\ti\tz\t0.6666666" in text
    assert "i\tz\tu\tx\t1" in text and "u\tw\ti\ty\t1" in text
    g2 = cl.Graph.load(p, cl.EdgeType.Directed)
    assert g2.edges() == g.edges() and g2.nodes() == g.nodes()
    # same transition probabilities per (from, to) pair after the reload
    def probs(gr):
        out = {}
        for v in range(gr.nodes()):
            s, e = int(gr.rows[v]), int(gr.rows[v + 1])
            prev = np.float32(0)
            for j in range(s, e):
                out[(gr.vocab_.get_name(v), gr.vocab_.get_name(int(gr.cols[j])))] = np.float32(gr.weights[j] - prev)
                prev = gr.weights[j]
        return out
    a, c = probs(g), probs(g2)
    assert a.keys() == c.keys()
    assert all(abs(float(a[k]) - float(c[k])) <= 1e-6 for k in a)
    # the gzipped save holds the same text as the plain one
    p2, pz = str(tmp_path / "g2.tsv"), str(tmp_path / "g2.tsv.gz")
    g2.save(p2)
    g2.save(pz)
    with gzip.open(pz, "rt") as f:
        assert f.read() == open(p2).read()
    assert cl.Graph.load(pz, cl.EdgeType.Directed).edges() == g.edges()


def test_save_anonymous_graph(tmp_path):
    rows = np.array([0, 2, 3, 3], np.uint64)
    g = cl.Graph.from_csr(rows, np.array([1, 2, 0], np.uint32), np.array([1.0, 3.0, 1.0], np.float32))
    p = str(tmp_path / "a.tsv")
    g.save(p)
    assert open(p).read() == "node\t0\tnode\t1\t0.25\nnode\t0\tnode\t2\t0.75\nnode\t1\tnode\t0\t1\n"


def test_native_vocab_api():
    v = NativeVocab()
    assert v.get_or_insert("user", "a") == 0 and v.get_or_insert("item", "a") == 1
    assert v.get_or_insert("user", "a") == 0 and len(v) == 2
    assert v.get_node_id("item", "a") == 1 and v.get_node_id("item", "b") is None
    assert v.get_name(1) == ("item", "a") and v.get_node_type(0) == "user"
    assert v.get_or_insert("", "") == 2 and v.get_name(2) == ("", "")
    assert v.get_or_insert("é", "名前") == 3 and v.get_node_id("é", "名前") == 3
    with pytest.raises(IndexError):
        v.get_name(4)
    for i in range(5000):
        v.get_or_insert("t", str(i))
    assert len(v) == 5004 and v.get_node_id("t", "4321") == 4325
    assert list(v)[:4] == [("user", "a"), ("item", "a"), ("", ""), ("é", "名前")]


def test_features_and_embeddings_over_a_loaded_graph(tmp_path):
    p = str(tmp_path / "g.tsv")
    _edges_tsv(p, ["user\tu1\titem\ti1\t1\n", "user\tu2\titem\ti1\t1\n"])
    g = cl.Graph.load(p, cl.EdgeType.Undirected)
    fp = str(tmp_path / "f.tsv")
    with open(fp, "w") as f:
        f.write("user\tu1\tred\nitem\ti1\tblue big\nuser\tnobody\tx\n")
    fs = cl.FeatureSet.new_from_graph(g)
    fs.load_into(fp)
    assert fs.get_features(("item", "i1")) == [("feat", "blue"), ("feat", "big")]
    assert fs.get_features(("user", "u2")) == []
    e = cl.NodeEmbeddings(g.vocab_, np.arange(12, dtype=np.float32).reshape(3, 4))
    ep = str(tmp_path / "e.emb")
    e.save(ep)
    assert open(ep).read().splitlines()[1] == "item\ti1\t[4,5,6,7]"
    back = cl.NodeEmbeddings.load(ep)
    assert list(back.vocab_) == list(g.vocab_) and np.array_equal(back.table, e.table)


def test_load_deduplicate_merges_repeated_edges(tmp_path):
    p = str(tmp_path / "dup.tsv")
    _edges_tsv(p, ["a\t1\tb\t2\t1.0\n", "a\t1\tb\t2\t3.0\n", "a\t1\tc\t3\t2.0\n"])
    plain = cl.Graph.load(p, cl.EdgeType.Directed)
    merged = cl.Graph.load(p, cl.EdgeType.Directed, deduplicate=True)
    assert plain.edges() == 3 and merged.edges() == 2
    # the merged graph matches the native CSR builder's duplicate merge on the same edges
    rows, cols, w = _native.csr_from_edges(np.array([0, 0, 0]), np.array([1, 1, 2]),
                                           np.array([1.0, 3.0, 2.0], np.float32), True)
    assert np.array_equal(merged.rows, rows) and np.array_equal(merged.cols, cols)
    assert np.array_equal(merged.weights, _native.cdf_convert(rows, w))


def test_native_vocab_many_names_and_export_ranges():
    v = NativeVocab()
    names = [("t%d" % (i % 7), "n%d" % i) for i in range(70000)]
    for t, n in names:
        v.get_or_insert(t, n)
    assert len(v) == 70000
    assert v.names(65530, 65540) == names[65530:65540]
    assert v.get_node_id("t3", "n69999") is None and v.get_node_id("t6", "n69999") == 69999
    assert list(v) == names
