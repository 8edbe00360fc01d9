"""EPLoss, LossWeighting and EmbeddingPropagator: the drop-in for
``cloverleaf.EmbeddingPropagator`` (``src/lib.rs:939-1377``).

``learn_features`` keeps the reference's contract: it fills featureless nodes
in the caller's FeatureSet (``src/feature_store.rs:83-89``), moves a warm-start
table out of the caller's NodeEmbeddings, and returns new NodeEmbeddings keyed
by the feature vocabulary.  Training runs on the GPU through the C ABI.
"""
from __future__ import annotations

import copy
import sys
from typing import List, Optional

import numpy as np

from . import _native
from .embeddings import Distance, NodeEmbeddings
from .features import FeatureSet
from .graph import Graph

SEED = 20222022   # lib.rs:90


class EPLoss:
    """Loss choice (loss.rs:15-38): margin (Euclidean), starspace (cosine
    margin), contrastive, rank (softmax NLL of the positive with margin tau),
    rankspace (starspace + rank) and ppr (margin with random-walk
    positives)."""

    def __init__(self, kind: str, gamma: float, negatives: int, neg_margin: float = 0.0,
                 restart_p: Optional[float] = None):
        self.kind, self.gamma, self.negatives = kind, float(gamma), int(negatives)
        self.neg_margin, self.restart_p = float(neg_margin), restart_p

    @staticmethod
    def margin(gamma: float, negatives: Optional[int] = None) -> "EPLoss":
        return EPLoss("margin", gamma, 1 if negatives is None else negatives)

    @staticmethod
    def contrastive(positive_margin: float, negative_margin: float, negatives: int) -> "EPLoss":
        return EPLoss("contrastive", positive_margin, max(1, negatives), neg_margin=negative_margin)

    @staticmethod
    def starspace(gamma: float, negatives: int) -> "EPLoss":
        return EPLoss("starspace", gamma, max(1, negatives))

    @staticmethod
    def rank(tau: float, negatives: int) -> "EPLoss":
        return EPLoss("rank", tau, max(1, negatives))

    @staticmethod
    def rankspace(tau: float, negatives: int) -> "EPLoss":
        return EPLoss("rankspace", tau, max(1, negatives))

    @staticmethod
    def ppr(gamma: float, negatives: int, restart_p: float) -> "EPLoss":
        return EPLoss("ppr", gamma, max(1, negatives), restart_p=restart_p)

    def code(self) -> int:
        return {"margin": _native.LOSS_MARGIN, "starspace": _native.LOSS_STARSPACE,
                "contrastive": _native.LOSS_CONTRASTIVE, "rank": _native.LOSS_RANK,
                "rankspace": _native.LOSS_RANKSPACE, "ppr": _native.LOSS_PPR}[self.kind]

    def __repr__(self) -> str:
        return f"EPLoss<{self.kind}({self.gamma}, {self.negatives})>"


class LossWeighting:
    """Per-anchor loss divisor: ln(1+deg) or deg^w (mod.rs:190-200)."""

    def __init__(self, kind: int, weight: float = 1.0):
        self.kind, self.weight = kind, float(weight)

    @staticmethod
    def Log() -> "LossWeighting":
        return LossWeighting(_native.LW_LOG)

    @staticmethod
    def Exponential(weight: float) -> "LossWeighting":
        return LossWeighting(_native.LW_EXP, weight)


def _sample(value: Optional[float], what: str):
    """Sample::new (utils.rs:173-184): None -> All, (0,1) -> Probability,
    otherwise Fixed(int(value)); negative values are rejected."""
    if value is None:
        return _native.SAMPLE_ALL, 0.0
    v = float(value)
    if v < 0:
        raise ValueError(f"{what} must be either None, or (0, N)")
    if 0.0 < v < 1.0:
        return _native.SAMPLE_PROB, v
    return _native.SAMPLE_FIXED, float(int(v))


class EmbeddingPropagator:
    """Embedding Propagation trainer with the reference's keyword arguments.

    Extra keyword-only options: ``form`` ("plain" = FP32 table, one kernel per
    stage; "fused" = BF16 table with FP32 accumulation and Adam moments, fused
    reduction + Adam, CUDA-graph replay), ``grad_mode`` ("reference" =
    first-occurrence extraction as cloverleaf does, "true" = exact gradient)
    and ``device``.
    """

    def __init__(self, alpha=None, loss=None, batch_size=None, dims=None, passes=None, seed=None, max_nodes=None,
                 weighted_neighbor_sampling=None, weighted_neighbor_averaging=None, max_features=None,
                 loss_weighting=None, valid_pct=None, hard_negatives=None, indicator=None, attention=None,
                 attention_heads=None, context_window=None, noise=None, *, form: str = "plain",
                 grad_mode: str = "reference", device: int = 0, use_graphs: bool = True):
        self.alpha = 0.9 if alpha is None else float(alpha)
        self.loss = loss if loss is not None else EPLoss.margin(1.0, 1)
        self.batch_size = 50 if batch_size is None else int(batch_size)
        self.dims = 100 if dims is None else int(dims)
        self.passes = 100 if passes is None else int(passes)
        self.seed = SEED if seed is None else int(seed)
        self.max_nodes = _sample(max_nodes, "max_nodes")
        self.max_features = _sample(max_features, "max_features")
        self.weighted_neighbor_sampling = bool(weighted_neighbor_sampling)
        self.weighted_neighbor_averaging = bool(weighted_neighbor_averaging)
        self.loss_weighting = loss_weighting
        self.valid_pct = 0.1 if valid_pct is None else float(valid_pct)
        self.hard_negatives = 0 if hard_negatives is None else int(hard_negatives)
        self.indicator = True if indicator is None else bool(indicator)
        self.noise = 0.0 if noise is None else float(noise)
        if attention is not None:
            raise _native.UnsupportedOption(-6, "the attention feature model is not implemented on the GPU path")
        if form not in ("plain", "fused"):
            raise ValueError("form must be 'plain' or 'fused'")
        if grad_mode not in ("reference", "true"):
            raise ValueError("grad_mode must be 'reference' or 'true'")
        self.form, self.grad_mode, self.device, self.use_graphs = form, grad_mode, int(device), use_graphs
        self.last_stats: List[dict] = []

    def __repr__(self) -> str:
        return (f"EmbeddingPropagation {{ alpha: {self.alpha}, loss: {self.loss!r}, batch_size: {self.batch_size}, "
                f"d_model: {self.dims}, passes: {self.passes}, seed: {self.seed}, valid_pct: {self.valid_pct}, "
                f"form: {self.form} }}")

    def config(self) -> _native.EpConfig:
        cfg = _native.default_config()
        cfg.alpha = self.alpha
        cfg.loss = self.loss.code()
        cfg.gamma = self.loss.gamma
        cfg.neg_margin = self.loss.neg_margin
        if self.loss.restart_p is not None:
            cfg.ppr_restart_p = float(self.loss.restart_p)
        cfg.negatives = self.loss.negatives
        cfg.batch_size = self.batch_size
        cfg.dims = self.dims
        cfg.passes = self.passes
        cfg.seed = self.seed
        cfg.max_nodes_kind, cfg.max_nodes = self.max_nodes
        cfg.max_features_kind, cfg.max_features = self.max_features
        cfg.weighted_neighbor_sampling = int(self.weighted_neighbor_sampling)
        cfg.weighted_neighbor_averaging = int(self.weighted_neighbor_averaging)
        if self.loss_weighting is not None:
            cfg.loss_weighting = self.loss_weighting.kind
            cfg.loss_weighting_exp = self.loss_weighting.weight
        cfg.valid_pct = self.valid_pct
        cfg.hard_negatives = self.hard_negatives
        cfg.noise = self.noise
        cfg.form = _native.FORM_FUSED_BF16 if self.form == "fused" else _native.FORM_PLAIN_FP32
        cfg.grad_mode = _native.GRAD_TRUE if self.grad_mode == "true" else _native.GRAD_REFERENCE
        cfg.device = self.device
        cfg.use_graphs = int(self.use_graphs)
        return cfg

    def context(self, graph: Graph, features: FeatureSet) -> _native.Context:
        """Creates a device context with the graph and features uploaded."""
        ctx = _native.Context(self.config())
        ctx.upload_graph(graph.rows, graph.cols, graph.weights)
        fptr, fids = features.to_csr()
        ctx.upload_features(fptr, fids, features.num_features())
        return ctx

    def learn_features(self, graph: Graph, features: FeatureSet,
                       feature_embeddings: Optional[NodeEmbeddings] = None) -> NodeEmbeddings:
        features.fill_missing_nodes()
        if len(features.to_csr()[0]) - 1 != graph.nodes():
            raise ValueError("FeatureSet and Graph disagree on the number of nodes")
        n_feat = features.num_features()
        init = None
        if feature_embeddings is not None:
            init = feature_embeddings.table
            if init.shape != (n_feat, self.dims):
                raise ValueError(f"warm-start embeddings have shape {init.shape}, expected {(n_feat, self.dims)}")
            # the reference moves the store out, leaving the caller's object empty (lib.rs:1337-1341)
            feature_embeddings.table = np.zeros((len(feature_embeddings.vocab_), 0), np.float32)
        ctx = self.context(graph, features)
        try:
            ctx.set_table(init)
            self.last_stats = ctx.train(self.passes)
            table = ctx.get_table(n_feat, self.dims)
        finally:
            ctx.close()
        if self.indicator:
            for s in self.last_stats:
                print(f"Pass {s['pass']}/{self.passes}, Train: {s['train_loss']:.5f}, "
                      f"Valid: {s['valid_loss']:.5f}, LR: {s['lr_last']:.5f}", file=sys.stderr)
        return NodeEmbeddings(copy.deepcopy(features.feature_vocab), table, Distance.Cosine)

    # spec spelling: learn(graph, feature_set) -> NodeEmbeddings
    learn = learn_features
