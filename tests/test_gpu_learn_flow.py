"""The sequence of package calls the reference's training script makes
(scripts/learn.py: load a TSV graph and a features file, train EP, save the
feature embeddings, build node embeddings with a weighted aggregator, align
them over the graph, save the aggregator), end to end on the GPU through this
package's drop-in API, on a small planted-community graph written as text."""
import gzip

import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import datagen

pytestmark = pytest.mark.gpu


def _write_inputs(tmp_path):
    w = datagen.workload("sbm1k")
    rows, cols, comm = w["rows"], w["cols"], w["community"]
    gp = str(tmp_path / "edges.tsv")
    with open(gp, "w") as f:
        f.write("from_type\tfrom\tto_type\tto\tweight\n")          # a header line, skipped
        for u in range(len(rows) - 1):
            for v in cols[int(rows[u]):int(rows[u + 1])].tolist():
                if u < v:
                    f.write(f"node\tn{u}\tnode\tn{v}\t1\n")
    fp = str(tmp_path / "features.tsv.gz")
    fptr, fids = w["fptr"], w["fids"]
    with gzip.open(fp, "wt") as f:
        for u in range(len(fptr) - 1):
            toks = " ".join(f"t{x}" for x in fids[int(fptr[u]):int(fptr[u + 1])].tolist())
            f.write(f"node\tn{u}\t{toks}\n")
    return w, gp, fp, comm


def test_training_script_call_sequence(tmp_path):
    w, gp, fp, comm = _write_inputs(tmp_path)
    graph = cl.Graph.load(gp, cl.EdgeType.Undirected, skip_rows=1, weighted=True)
    present = [u for u in range(len(w["rows"]) - 1) if graph.vocab_.get_node_id("node", f"n{u}") is not None]
    assert graph.nodes() == len(present) > 0
    features = cl.FeatureSet.new_from_graph(graph)
    features.load_into(fp)
    features = features.prune_min_count(1)
    assert features.num_features() > 0
    ep = w["ep"]
    prop = cl.EmbeddingPropagator(
        alpha=ep["alpha"], loss=cl.EPLoss.starspace(ep["gamma"], ep["negatives"]), batch_size=ep["batch_size"],
        dims=ep["dims"], passes=5, max_nodes=ep["max_nodes"], max_features=None, loss_weighting=None,
        weighted_neighbor_averaging=False, weighted_neighbor_sampling=False, attention=None, attention_heads=None,
        context_window=None, noise=None, hard_negatives=0, valid_pct=0.0)
    feature_embeddings = prop.learn_features(graph, features, None)
    out = str(tmp_path / "run")
    feature_embeddings.save(out + ".feature-embeddings.gz")
    back = cl.NodeEmbeddings.load(out + ".feature-embeddings.gz", cl.Distance.Cosine)
    assert np.array_equal(back.table, feature_embeddings.table)

    aggregator = cl.FeatureAggregator.Weighted(1e-3, features)
    embedder = cl.NodeEmbedder(aggregator)
    node_embeddings = embedder.embed_feature_set(features, feature_embeddings)
    assert node_embeddings.len() == graph.nodes()
    node_embeddings.save(out + ".node-embeddings.orig")
    cl.NeighborhoodAligner(0.5).align_to_disk(out + ".node-embeddings", node_embeddings, graph)
    aggregator.save(out + ".embedder")

    # the trained model separates the planted communities
    ids = [graph.vocab_.get_node_id("node", f"n{u}") for u in present]
    tab = node_embeddings.table[ids]
    comm = comm[present]
    un = tab / (np.linalg.norm(tab, axis=1, keepdims=True) + 1e-12)
    sim = un @ un.T
    np.fill_diagonal(sim, -np.inf)
    top = np.argsort(-sim, axis=1)[:, :10]
    recall = float(np.mean(comm[top] == comm[:, None]))
    assert recall > 2.0 / 8, recall          # 8 communities: chance is 1/8

    aligned = cl.NodeEmbeddings.load(out + ".node-embeddings")
    assert aligned.len() == graph.nodes() and aligned.dims() == ep["dims"]
    agg2 = cl.FeatureAggregator.load(out + ".embedder")
    assert repr(agg2) == repr(aggregator)
    again = cl.NodeEmbedder(agg2).embed_feature_set(features, back)
    assert np.allclose(again.table, node_embeddings.table, rtol=1e-5, atol=1e-6)
