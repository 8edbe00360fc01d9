"""NeighborhoodAligner (src/algos/alignment.rs, Python class src/lib.rs:
3040-3167): shifts every node embedding toward the probability-weighted sum
of its neighbours' embeddings, on the GPU (``ep_align``)."""
from typing import Optional

import numpy as np

from . import _native
from .embeddings import NodeEmbeddings
from .graph import Graph


class NeighborhoodAligner:
    """alpha in [0, 1]: weight kept on the node's own embedding (None:
    min(1, 1 / ln(deg + 1)) per node); max_neighbors: the first K edges of
    each node (None: all)."""

    def __init__(self, alpha: Optional[float] = None, max_neighbors: Optional[int] = None):
        self.alpha = None if alpha is None else float(np.float32(alpha))
        self.max_neighbors = None if max_neighbors is None else int(max_neighbors)

    def __repr__(self) -> str:
        a = "None" if self.alpha is None else f"Some({self.alpha})"
        k = "None" if self.max_neighbors is None else f"Some({self.max_neighbors})"
        return f"NeighborhoodAligner<Alpha={a}, MaxNeighbors={k}>"

    def _aligned(self, embeddings: NodeEmbeddings, graph: Graph) -> np.ndarray:
        n = graph.nodes()
        if embeddings.len() < n:
            raise ValueError(f"embeddings hold {embeddings.len()} rows for a graph of {n} nodes")
        out = np.zeros_like(embeddings.table)    # rows past the graph's nodes stay zero (lib.rs:3119-3124)
        out[:n] = _native.align(graph.rows, graph.cols, graph.weights, embeddings.table[:n], self.alpha,
                                self.max_neighbors)
        return out

    def align(self, embeddings: NodeEmbeddings, graph: Graph) -> NodeEmbeddings:
        """A new NodeEmbeddings: node i of the graph is row i of embeddings."""
        return NodeEmbeddings(embeddings.vocab_, self._aligned(embeddings, graph), embeddings.distance)

    def align_to_disk(self, path: str, embeddings: NodeEmbeddings, graph: Graph, chunk_size: Optional[int] = None,
                      comp_level: Optional[int] = None) -> None:
        """align, written in NodeEmbeddings.save's format (lib.rs:3141-3167)."""
        del chunk_size      # the whole table is aligned in one device pass
        self.align(embeddings, graph).save(path, comp_level)
