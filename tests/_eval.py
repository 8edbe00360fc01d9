"""Evaluation helpers for the end-to-end checks: node embeddings as the mean
of their feature rows (NodeEmbedder + FeatureAggregator.Averaged,
aggregator.rs:34-48) and community recall@k by exact cosine kNN."""
import numpy as np


def node_embeddings(fptr, fids, table):
    n = len(fptr) - 1
    node = np.repeat(np.arange(n), np.diff(fptr).astype(np.int64))
    out = np.zeros((n, table.shape[1]), np.float64)
    np.add.at(out, node, table[fids.astype(np.int64)].astype(np.float64))
    cnt = np.diff(fptr).astype(np.float64)
    out /= np.maximum(cnt, 1)[:, None]
    return out


def community_recall(fptr, fids, table, community, k=10, block=1024):
    """Mean over nodes of |top-k cosine neighbours (self excluded) in the
    node's community| / k."""
    E = node_embeddings(fptr, fids, table)
    nrm = np.linalg.norm(E, axis=1, keepdims=True)
    E = E / np.maximum(nrm, 1e-30)
    comm = np.asarray(community)
    n = len(E)
    hits = 0.0
    for s in range(0, n, block):
        S = E[s:s + block] @ E.T
        idx = np.arange(s, min(s + block, n))
        S[np.arange(len(idx)), idx] = -np.inf
        top = np.argpartition(-S, k, axis=1)[:, :k]
        hits += (comm[top] == comm[idx][:, None]).sum()
    return hits / (n * k)
