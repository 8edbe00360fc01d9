"""Held-out-edge recall@k, the reference's evaluation of a trained model
(scripts/evaluate.py:29-61): for each test edge (u, v), the k nearest node
embeddings to u's by cosine (NodeEmbeddings.nearest_neighbor,
src/embeddings.rs:149-173; u itself is not excluded, as there) and a hit when
v is among them.  Node embeddings are the NodeEmbedder's averaged feature rows
(src/algos/aggregator.rs:34-48).

Both steps run on the GPU (ep_embed_features, ep_knn_cosine); the split of a
graph into training edges and held-out test edges is host code.
"""
from __future__ import annotations

import numpy as np

from . import _native


def holdout_edges(rows, cols, weights, frac: float, seed: int, max_test: int = 20000):
    """Removes a seeded fraction of the undirected edges of a symmetric CSR
    (both directions), never leaving a node without edges.

    Returns (rows, cols, weights, test) where test is an int64 [m, 2] array of
    up to max_test held-out (u, v) pairs, each in a random direction."""
    rows = np.asarray(rows, np.uint64)
    cols = np.asarray(cols, np.uint32)
    weights = np.asarray(weights, np.float32)
    n = len(rows) - 1
    deg = np.diff(rows).astype(np.int64)
    src = np.repeat(np.arange(n, dtype=np.uint32), deg)
    rng = np.random.default_rng(seed)
    pick = (src < cols) & (rng.random(len(cols)) < frac)
    # rows are sorted and so are the columns within a row: the key src*n+col
    # is globally sorted, and the reverse direction of an edge is found by
    # binary search
    key = src.astype(np.uint64) * np.uint64(n) + cols.astype(np.uint64)
    fwd = np.nonzero(pick)[0]
    rev = np.searchsorted(key, cols[fwd].astype(np.uint64) * np.uint64(n) + src[fwd].astype(np.uint64))
    ok = (rev < len(key))
    ok[ok] = key[rev[ok]] == cols[fwd[ok]].astype(np.uint64) * np.uint64(n) + src[fwd[ok]].astype(np.uint64)
    fwd, rev = fwd[ok], rev[ok]
    # keep every node at least one edge: give back the held-out edges of any
    # node that would lose them all
    for _ in range(4):
        lost = np.bincount(src[fwd], minlength=n) + np.bincount(src[rev], minlength=n)
        bare = (deg - lost) <= 0
        keep = ~(bare[src[fwd]] | bare[cols[fwd]])
        if keep.all():
            break
        fwd, rev = fwd[keep], rev[keep]
    drop = np.zeros(len(cols), bool)
    drop[fwd] = True
    drop[rev] = True
    new_deg = np.bincount(src[~drop], minlength=n)
    rows2 = np.zeros(n + 1, np.uint64)
    rows2[1:] = np.cumsum(new_deg)
    test = np.stack([src[fwd], cols[fwd]], axis=1).astype(np.int64)
    if len(test) > max_test:
        test = test[rng.choice(len(test), max_test, replace=False)]
    flip = rng.random(len(test)) < 0.5
    test[flip] = test[flip][:, ::-1]
    return rows2, cols[~drop], weights[~drop], test


def node_embeddings(fptr, fids, table, device: int = 0) -> np.ndarray:
    """The averaged feature rows of every node (GPU NodeEmbedder)."""
    return _native.embed_features(fptr, fids, table, device=device)


def heldout_recall(fptr, fids, table, test, k: int = 10, device: int = 0, block: int = 8192) -> dict:
    """Recall@k of the held-out test edges, and the share of test edges whose
    two nodes are more similar (cosine) than the query node and a uniform
    random node (an AUC-style score that stays informative where the top-k
    rarely holds the true neighbour)."""
    test = np.asarray(test, np.int64)
    emb = node_embeddings(fptr, fids, table, device)
    hits = 0
    for s in range(0, len(test), block):
        q = test[s:s + block]
        idx, _ = _native.knn_cosine(emb, emb[q[:, 0]], k, device=device)
        hits += int((idx.astype(np.int64) == q[:, 1:2]).any(axis=1).sum())
    rng = np.random.default_rng(len(test))
    other = rng.integers(0, len(emb), len(test))

    def cos(a, b):
        x, y = emb[a].astype(np.float64), emb[b].astype(np.float64)
        den = np.linalg.norm(x, axis=1) * np.linalg.norm(y, axis=1)
        return (x * y).sum(axis=1) / np.maximum(den, 1e-30)

    pos, neg = cos(test[:, 0], test[:, 1]), cos(test[:, 0], other)
    return {"recall": hits / max(len(test), 1), "k": k, "test_edges": int(len(test)),
            "auc": float(np.mean((pos > neg) + 0.5 * (pos == neg))) if len(test) else float("nan")}
