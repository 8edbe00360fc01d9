"""Graph, GraphBuilder, EdgeType and the node vocabulary.

Mirrors cloverleaf's Python classes (``src/lib.rs:292-499``, ``:841-935``)
and its ``Vocab`` (``src/vocab.rs:12-80``).  The CSR itself is built by the
native library (``ep_csr_from_edges`` / ``ep_cdf_convert``, restating
``src/graph.rs:70-142, 414-422, 664-691``) and is uploaded to the GPU once per
training call.
"""
from __future__ import annotations

import enum
from typing import Iterator, List, Optional, Tuple

import numpy as np

from . import _native

FQNode = Tuple[str, str]


class EdgeType(enum.Enum):
    """``Undirected`` stores each edge in both directions (lib.rs:841-847)."""
    Directed = 0
    Undirected = 1


class Vocab:
    """(node_type, name) <-> dense id, ids assigned in first-seen order."""

    def __init__(self):
        self._ids = {}
        self._names: List[FQNode] = []

    def get_or_insert(self, node_type: str, name: str) -> int:
        key = (node_type, name)
        i = self._ids.get(key)
        if i is None:
            i = len(self._names)
            self._ids[key] = i
            self._names.append(key)
        return i

    def get_node_id(self, node_type: str, name: str) -> Optional[int]:
        return self._ids.get((node_type, name))

    def get_name(self, idx: int) -> FQNode:
        return self._names[idx]

    def get_node_type(self, idx: int) -> str:
        return self._names[idx][0]

    def __len__(self) -> int:
        return len(self._names)

    def __iter__(self) -> Iterator[FQNode]:
        return iter(self._names)

    @classmethod
    def anonymous(cls, n: int, node_type: str = "node") -> "Vocab":
        """The vocabulary (node_type, str(i)) for i in range(n), computed on
        demand so that large synthetic graphs need no per-node objects."""
        return RangeVocab(n, node_type)


class RangeVocab(Vocab):
    """(node_type, str(i)) <-> i for i < n; grows like Vocab for new names."""

    def __init__(self, n: int, node_type: str):
        super().__init__()
        self._n, self._type = n, node_type

    def _range_id(self, node_type, name):
        if node_type == self._type and name.isdigit() and (name == "0" or not name.startswith("0")):
            i = int(name)
            if i < self._n:
                return i
        return None

    def get_or_insert(self, node_type: str, name: str) -> int:
        i = self._range_id(node_type, name)
        if i is not None:
            return i
        j = self._ids.get((node_type, name))
        if j is None:
            j = self._n + len(self._names)
            self._ids[(node_type, name)] = j
            self._names.append((node_type, name))
        return j

    def get_node_id(self, node_type: str, name: str) -> Optional[int]:
        i = self._range_id(node_type, name)
        return i if i is not None else self._ids.get((node_type, name))

    def get_name(self, idx: int) -> FQNode:
        return (self._type, str(idx)) if idx < self._n else self._names[idx - self._n]

    def get_node_type(self, idx: int) -> str:
        return self.get_name(idx)[0]

    def __len__(self) -> int:
        return self._n + len(self._names)

    def __iter__(self) -> Iterator[FQNode]:
        for i in range(len(self)):
            yield self.get_name(i)


class NativeVocab(Vocab):
    """A Vocab held by the native library (``ep_vocab_*``): the vocabulary
    of graphs read by Graph.load, whose millions of names would otherwise be
    Python objects.  Same ids and lookups as Vocab."""

    def __init__(self, handle=None):
        from . import _native

        self._v = handle if handle is not None else _native.NativeVocabHandle()

    def get_or_insert(self, node_type: str, name: str) -> int:
        return self._v.intern(node_type, name)

    def get_node_id(self, node_type: str, name: str) -> Optional[int]:
        i = self._v.find(node_type, name)
        return None if i < 0 else i

    def get_name(self, idx: int) -> FQNode:
        if not 0 <= idx < len(self):
            raise IndexError(f"node id {idx} out of range")
        t, n = self._v.export(idx, idx + 1)
        return t[0], n[0]

    def get_node_type(self, idx: int) -> str:
        return self.get_name(idx)[0]

    def names(self, lo: int, hi: int) -> List[FQNode]:
        """The names of ids [lo, hi) in one native call."""
        t, n = self._v.export(lo, hi)
        return list(zip(t, n))

    def __len__(self) -> int:
        return len(self._v)

    def __iter__(self) -> Iterator[FQNode]:
        n = len(self)
        for lo in range(0, n, 65536):
            yield from self.names(lo, min(n, lo + 65536))


def _as_native_vocab(vocab: Vocab, n: int):
    """The vocabulary's first n names in a native handle (itself when it
    already is one), or the node type when every name is the decimal id."""
    from . import _native

    if isinstance(vocab, NativeVocab):
        return vocab._v
    if isinstance(vocab, RangeVocab) and vocab._n >= n:
        return vocab._type
    h = _native.NativeVocabHandle()
    for i in range(n):
        h.intern(*vocab.get_name(i))
    return h


def _node_id(vocab: Vocab, node: FQNode) -> int:
    i = vocab.get_node_id(node[0], node[1])
    if i is None:
        raise KeyError(f"Node {node} does not exist!")
    return i


class Graph:
    """Immutable CSR graph with per-row CDF weights (``CumCSR``, graph.rs:399)."""

    def __init__(self, rows: np.ndarray, cols: np.ndarray, weights_cdf: np.ndarray, vocab: Vocab):
        self.rows = np.ascontiguousarray(rows, np.uint64)
        self.cols = np.ascontiguousarray(cols, np.uint32)
        self.weights = np.ascontiguousarray(weights_cdf, np.float32)
        self.vocab_ = vocab

    @classmethod
    def from_csr(cls, rows, cols, weights=None, vocab: Optional[Vocab] = None, cdf: bool = False) -> "Graph":
        """Builds a Graph from CSR arrays (an extension for large synthetic
        graphs).  Raw weights are converted to per-row CDFs unless cdf=True."""
        rows = np.ascontiguousarray(rows, np.uint64)
        n = len(rows) - 1
        if weights is None:
            weights = np.ones(len(cols), np.float32)
        w = np.ascontiguousarray(weights, np.float32)
        if not cdf:
            w = _native.cdf_convert(rows, w)
        return cls(rows, cols, w, vocab if vocab is not None else Vocab.anonymous(n))

    def nodes(self) -> int:
        return len(self.rows) - 1

    def edges(self) -> int:
        return int(self.rows[-1])

    def degree(self, idx: int) -> int:
        return int(self.rows[idx + 1] - self.rows[idx])

    def contains_node(self, name: FQNode) -> bool:
        return self.vocab_.get_node_id(name[0], name[1]) is not None

    def get_edges(self, node: FQNode, normalized: Optional[bool] = None):
        """Outbound (nodes, weights); CDF weights unless normalized (lib.rs:374-388)."""
        i = _node_id(self.vocab_, node)
        s, e = int(self.rows[i]), int(self.rows[i + 1])
        names = [self.vocab_.get_name(int(c)) for c in self.cols[s:e]]
        w = self.weights[s:e]
        if normalized:
            w = np.diff(np.concatenate([[0.0], w.astype(np.float64)])).astype(np.float32)
        return names, [float(x) for x in w]

    def vocab(self) -> Iterator[FQNode]:
        return iter(self.vocab_)

    def __len__(self) -> int:
        return self.nodes()

    def __repr__(self) -> str:
        return f"Graph<Nodes={self.nodes()}, Edges={self.edges()}>"

    def save(self, path: str, comp_level: Optional[int] = None) -> None:
        """Writes ``from_type\\tfrom\\tto_type\\tto\\tweight`` lines, the
        weight each edge's transition probability written as Rust writes an
        f32 (Graph::save, lib.rs:414-430), gzipped (level comp_level,
        default 1) when the path ends with ``.gz``.  Rows are formatted
        natively in blocks (``ep_format_edges``)."""
        from . import _native

        n = self.nodes()
        h = _as_native_vocab(self.vocab_, n)
        if path.endswith(".gz"):
            import gzip
            f = gzip.open(path, "wb", compresslevel=1 if comp_level is None else int(comp_level))
        else:
            f = open(path, "wb")
        with f:
            lo = 0
            while lo < n:
                # blocks of about 1M edges
                hi = int(np.searchsorted(self.rows, self.rows[lo] + (1 << 20), side="right")) - 1
                hi = min(n, max(hi, lo + 1))
                f.write(_native.format_edges(h, self.rows, self.cols, self.weights, lo, hi))
                lo = hi

    @staticmethod
    def load(path: str, edge_type: EdgeType, chunk_size: Optional[int] = None, skip_rows: Optional[int] = None,
             weighted: Optional[bool] = None, deduplicate: Optional[bool] = None) -> "Graph":
        """Reads ``from_type\\tfrom\\tto_type\\tto\\tweight`` lines, optionally
        gzipped (GraphReader::load, io.rs:270-323): skip_rows leading lines
        skipped, weights read unless weighted is False, both directions of
        each line for an undirected graph, duplicate edges merged when
        deduplicate.  Lines are parsed and names interned natively
        (``ep_parse_edges``) into a NativeVocab; blank lines are skipped.
        chunk_size is accepted for API parity."""
        from . import _native
        from .embeddings import _line_blocks

        weighted = True if weighted is None else weighted
        v = NativeVocab()
        src, dst, w = [], [], []
        for buf in _line_blocks(path, skip_rows or 0):
            a, b, c = _native.parse_edges(v._v, buf, weighted)
            src.append(a)
            dst.append(b)
            w.append(c)
        if not src or not sum(len(x) for x in src):
            raise ValueError("graph file has no edges")
        src, dst, w = np.concatenate(src), np.concatenate(dst), np.concatenate(w)
        if edge_type == EdgeType.Undirected:
            # (f, t, w), (t, f, w) per line, as GraphReader::load pushes them
            s2 = np.empty(2 * len(src), np.uint32)
            d2 = np.empty(2 * len(src), np.uint32)
            s2[0::2], s2[1::2] = src, dst
            d2[0::2], d2[1::2] = dst, src
            src, dst, w = s2, d2, np.repeat(w, 2)
        n = len(v)
        rows, cols, wr = _native.csr_from_edges(src, dst, w, bool(deduplicate))
        if len(rows) - 1 < n:     # nodes past the largest edge endpoint id have no edges
            rows = np.concatenate([rows, np.full(n - (len(rows) - 1), rows[-1], np.uint64)])
        return Graph(rows, cols, _native.cdf_convert(rows, wr), v)


class GraphBuilder:
    """Incremental edge list -> Graph (lib.rs:851-935)."""

    def __init__(self):
        self._vocab = Vocab()
        self._src: List[int] = []
        self._dst: List[int] = []
        self._w: List[float] = []

    def __repr__(self) -> str:
        return f"GraphBuilder<Nodes={len(self._vocab)}, Edges={len(self._src)}>"

    def add_edge(self, from_node: FQNode, to_node: FQNode, weight: float, node_type: EdgeType) -> None:
        f = self._vocab.get_or_insert(from_node[0], from_node[1])
        t = self._vocab.get_or_insert(to_node[0], to_node[1])
        self._src.append(f)
        self._dst.append(t)
        self._w.append(float(weight))
        if node_type == EdgeType.Undirected:
            self._src.append(t)
            self._dst.append(f)
            self._w.append(float(weight))

    def build_graph(self, deduplicate: Optional[bool] = None) -> Optional[Graph]:
        """None when no edges were added; otherwise a CSR with CDF weights.
        The builder is emptied, as the reference swaps its buffers out."""
        if not self._src:
            return None
        dedup = True if deduplicate is None else bool(deduplicate)
        rows, cols, w = _native.csr_from_edges(np.array(self._src, np.uint32), np.array(self._dst, np.uint32),
                                               np.array(self._w, np.float32), dedup)
        vocab = self._vocab
        self._vocab, self._src, self._dst, self._w = Vocab(), [], [], []
        return Graph(rows, cols, _native.cdf_convert(rows, w), vocab)
