"""FeatureSet: discrete features per node (``src/lib.rs:1433-1691``,
``src/feature_store.rs:19-139``).

Features are interned to dense feature ids in first-seen order; the per-node
lists are flattened to a CSR (fptr, fids) when uploaded to the GPU.
"""
from __future__ import annotations

from typing import Iterator, List, Optional, Sequence, Tuple

import numpy as np

from .graph import FQNode, Graph, Vocab, _node_id


class FeatureNamespace:
    """How a token becomes a (namespace, name) feature (lib.rs:1379-1428)."""

    def __init__(self, kind: str, arg: Optional[str] = None):
        self.kind, self.arg = kind, arg

    @staticmethod
    def single(ns: str) -> "FeatureNamespace":
        return FeatureNamespace("static", ns)

    @staticmethod
    def node_type() -> "FeatureNamespace":
        return FeatureNamespace("node_type")

    @staticmethod
    def prefix(delim: str) -> "FeatureNamespace":
        return FeatureNamespace("prefix", delim)

    def parse(self, node_type: str, token: str) -> Optional[Tuple[str, str]]:
        if self.kind == "static":
            return self.arg, token
        if self.kind == "node_type":
            return node_type, token
        idx = token.find(self.arg)
        if idx < 0:
            return None
        return token[:idx], token[idx + len(self.arg):]


class FeatureSet:
    """Node -> feature ids, with the feature vocabulary."""

    def __init__(self, vocab: Vocab, n_nodes: int):
        self.vocab_ = vocab                  # node vocabulary (shared with the graph)
        self.feature_vocab = Vocab()
        self._feats: List[List[int]] = [[] for _ in range(n_nodes)]
        self._csr: Optional[Tuple[np.ndarray, np.ndarray]] = None   # cache

    @staticmethod
    def new_from_graph(graph: Graph) -> "FeatureSet":
        return FeatureSet(graph.vocab_, graph.nodes())

    @staticmethod
    def new_from_file(path: str, namespace: Optional[FeatureNamespace] = None) -> "FeatureSet":
        """A FeatureSet over the nodes named in a features file, in file
        order (lib.rs:1440-1517), loaded with load_into."""
        import gzip

        v = Vocab()
        with (gzip.open(path, "rt") if path.endswith(".gz") else open(path)) as f:
            for line in f:
                pieces = line.rstrip("\n").split("\t")
                if len(pieces) != 3:
                    raise ValueError("Malformed feature line! Need node_type<TAB>name<TAB>f1 f2 ...")
                v.get_or_insert(pieces[0], pieces[1])
        fs = FeatureSet(v, len(v))
        fs.load_into(path, namespace)
        return fs

    @classmethod
    def from_csr(cls, graph: Graph, fptr, fids, n_feat: int, feature_vocab: Optional[Vocab] = None) -> "FeatureSet":
        """Builds a FeatureSet from CSR arrays (an extension for large
        synthetic workloads); feature names default to ("feat", str(id))."""
        fs = cls.__new__(cls)
        fs.vocab_ = graph.vocab_
        fs.feature_vocab = feature_vocab if feature_vocab is not None else Vocab.anonymous(n_feat, "feat")
        fs._feats = None
        fs._csr = (np.ascontiguousarray(fptr, np.uint64), np.ascontiguousarray(fids, np.uint32))
        return fs

    # -- internal representation ------------------------------------------
    def _lists(self) -> List[List[int]]:
        if self._feats is None:
            fptr, fids = self._csr
            self._feats = [fids[int(fptr[i]):int(fptr[i + 1])].tolist() for i in range(len(fptr) - 1)]
        return self._feats

    def to_csr(self) -> Tuple[np.ndarray, np.ndarray]:
        if self._csr is None:
            lists = self._feats
            counts = np.fromiter((len(x) for x in lists), np.uint64, len(lists))
            fptr = np.zeros(len(lists) + 1, np.uint64)
            np.cumsum(counts, out=fptr[1:])
            fids = np.fromiter((f for x in lists for f in x), np.uint32, int(fptr[-1]))
            self._csr = (fptr, fids)
        return self._csr

    def _touch(self):
        self._lists()
        self._csr = None

    # -- reference API ----------------------------------------------------
    def set_features(self, node: FQNode, features: Sequence[Tuple[str, str]]) -> None:
        i = _node_id(self.vocab_, node)
        self._touch()
        self._feats[i] = [self.feature_vocab.get_or_insert(t, n) for t, n in features]

    def get_features(self, node: FQNode) -> List[Tuple[str, str]]:
        i = _node_id(self.vocab_, node)
        return [self.feature_vocab.get_name(f) for f in self._lists()[i]]

    def load_into(self, path: str, f_ns: Optional[FeatureNamespace] = None) -> None:
        """``node_type\\tname\\tf1 f2 ...`` lines (lib.rs:1579-1606); unknown
        nodes are skipped."""
        import gzip

        ns = f_ns or FeatureNamespace.single("feat")
        opener = gzip.open if path.endswith(".gz") else open
        self._touch()
        with opener(path, "rt") as f:
            for i, line in enumerate(f):
                pieces = line.rstrip("\n").split("\t")
                if len(pieces) != 3:
                    raise ValueError(f"Line {i + 1}:Malformed feature line! Need node_type<TAB>name<TAB>f1 f2 ...")
                node = self.vocab_.get_node_id(pieces[0], pieces[1])
                if node is None:
                    continue
                bow = [ns.parse(pieces[0], tok) or ("feat", tok) for tok in pieces[2].split()]
                self._feats[node] = [self.feature_vocab.get_or_insert(t, n) for t, n in bow]

    def fill_missing_nodes(self) -> None:
        """Gives each featureless node the feature ("node", str(id))
        (feature_store.rs:83-89)."""
        if self._feats is None and np.all(np.diff(self._csr[0]) > 0):
            return  # CSR-backed and complete: nothing to fill
        lists = self._lists()
        changed = False
        for i, fl in enumerate(lists):
            if not fl:
                lists[i] = [self.feature_vocab.get_or_insert("node", str(i))]
                changed = True
        if changed:
            self._csr = None

    def nodes(self) -> int:
        return len(self.vocab_)

    def num_features(self) -> int:
        return len(self.feature_vocab)

    def vocab(self) -> Iterator[FQNode]:
        return iter(self.vocab_)

    def count_features(self) -> np.ndarray:
        fptr, fids = self.to_csr()
        return np.bincount(fids, minlength=self.num_features())

    def prune_min_count(self, count: int) -> "FeatureSet":
        """Drops features seen fewer than `count` times (feature_store.rs:118-136)."""
        counts = self.count_features()
        out = FeatureSet(self.vocab_, len(self._lists()))
        for i, fl in enumerate(self._lists()):
            out._feats[i] = [out.feature_vocab.get_or_insert(*self.feature_vocab.get_name(f))
                             for f in fl if counts[f] >= count]
        return out

    def __getitem__(self, idx: int) -> Tuple[str, str]:
        n = self.num_features()
        if idx < 0:
            idx += n
        if idx >= n or idx < 0:
            raise IndexError("Feature Index larger than FeatureSet!")
        return self.feature_vocab.get_name(idx)

    def __repr__(self) -> str:
        return f"FeatureSet<Nodes={self.nodes()},UniqueFeatures={self.num_features()}>"


class FeaturePropagator:
    """Fills featureless nodes from their neighbours' features
    (lib.rs:1695-1770; feat_propagation.rs:13-93), natively
    (``ep_propagate_features``)."""

    def __init__(self, k: int, threshold: Optional[float] = None, max_iters: Optional[int] = None):
        if k < 0 or (max_iters is not None and max_iters < 0):
            raise OverflowError("can't convert negative int to unsigned")
        self.k = int(k)
        self.threshold = 0.0 if threshold is None else float(threshold)
        self.max_iters = 20 if max_iters is None else int(max_iters)

    def __repr__(self) -> str:
        return f"FeaturePropagator<k={self.k},threshold={_rust_f32(self.threshold)},max_iters={self.max_iters}>"

    def propagate(self, graph: Graph, features: "FeatureSet") -> None:
        from . import _native

        fptr, fids = features.to_csr()
        fptr2, fids2 = _native.propagate_features(graph.rows, graph.cols, graph.weights, fptr, fids, self.max_iters,
                                                  self.k, self.threshold)
        features._feats = None
        features._csr = (fptr2, fids2)


def _rust_f32(x: float) -> str:
    """An f32 as Rust's Display writes it: the shortest round-trip digits,
    positional."""
    return np.format_float_positional(np.float32(x), unique=True, trim="-")
