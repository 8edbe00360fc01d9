"""cloverleaf_gb300 -- Embedding Propagation training on GB300 (sm_103a).

A drop-in for cloverleaf's ``EmbeddingPropagator.learn_features`` path: the
same Python classes and keyword arguments, with training executed by
hand-written CUDA kernels behind the C ABI in ``include/ep_gb300.h``.
"""
from ._native import NativeError, UnsupportedOption
from .alignment import NeighborhoodAligner
from .embeddings import Distance, FeatureAggregator, NodeEmbedder, NodeEmbeddings
from .ep import EmbeddingPropagator, EPLoss, LossWeighting
from .features import FeatureNamespace, FeaturePropagator, FeatureSet
from .graph import EdgeType, Graph, GraphBuilder, Vocab

__all__ = [
    "Distance", "EdgeType", "EmbeddingPropagator", "EPLoss", "FeatureAggregator", "FeatureNamespace", "FeaturePropagator", "FeatureSet",
    "Graph", "GraphBuilder", "LossWeighting", "NativeError", "NeighborhoodAligner", "NodeEmbedder", "NodeEmbeddings",
    "UnsupportedOption",
    "Vocab", "build",
]


def build(verbose: bool = False) -> str:
    """Compiles the native library in-tree (sm_103a) and returns its path."""
    from . import _build

    return _build.build(verbose=verbose)
