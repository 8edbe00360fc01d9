"""NodeEmbeddings, Distance, FeatureAggregator and NodeEmbedder.

Mirrors ``src/lib.rs:2009-2207`` (NodeEmbedder), ``:2536-2900``
(NodeEmbeddings), ``src/embeddings.rs:24-173`` (EmbeddingStore),
``src/distance.rs:132-198`` (distances) and ``src/algos/aggregator.rs:17-120``
(Averaged / Weighted aggregators).  NodeEmbedder.embed_feature_set and
NodeEmbeddings.nearest_neighbors (many queries) run on the GPU through the C
ABI; vocabularies, text I/O and single-query lookups stay on the host.
"""
from __future__ import annotations

import enum
from typing import Iterator, List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native
from .graph import FQNode, Graph, Vocab, _node_id


class Distance(enum.Enum):
    ALT = 0
    Cosine = 1
    Dot = 2
    Euclidean = 3
    Hamming = 4
    Jaccard = 5

    def compute(self, e1, e2) -> float:
        """distance.rs:132-198: zero means identical."""
        a = np.asarray(e1, np.float32)
        b = np.asarray(e2, np.float32)
        if self is Distance.Cosine:
            d = float(np.dot(a, b)) / (float(np.sqrt(np.dot(a, a))) * float(np.sqrt(np.dot(b, b))))
            return float("inf") if d != d else 1.0 - d
        if self is Distance.Euclidean:
            return float(np.sqrt(np.sum((a - b) ** 2)))
        if self is Distance.Dot:
            return -float(np.dot(a, b))
        if self is Distance.ALT:
            return float(np.max(np.abs(a - b))) if len(a) else 0.0
        if self is Distance.Hamming:
            return float(np.sum(a != b)) / len(a)
        # Jaccard over sorted non-negative ids
        i = j = m = 0
        while i < len(a) and j < len(b) and a[i] >= 0 and b[j] >= 0:
            if a[i] == b[j]:
                m += 1; i += 1; j += 1
            elif a[i] < b[j]:
                i += 1
            else:
                j += 1
        while i < len(a) and a[i] >= 0:
            i += 1
        while j < len(b) and b[j] >= 0:
            j += 1
        total = m + (i - m) + (j - m)
        return 1.0 - m / total

    def matrix(self, q: np.ndarray, X: np.ndarray) -> np.ndarray:
        """Distances from query q to every row of X (Cosine/Euclidean/Dot
        vectorised; others row by row)."""
        if self is Distance.Cosine:
            qn = np.sqrt(np.dot(q, q))
            xn = np.sqrt(np.einsum("ij,ij->i", X, X))
            with np.errstate(divide="ignore", invalid="ignore"):
                s = (X @ q) / (xn * qn)
            out = 1.0 - s
            out[~np.isfinite(out)] = np.inf
            return out
        if self is Distance.Euclidean:
            return np.sqrt(np.sum((X - q) ** 2, axis=1))
        if self is Distance.Dot:
            return -(X @ q)
        return np.array([self.compute(q, x) for x in X], np.float32)


class NodeEmbeddings:
    """Dense row-major embeddings keyed by a vocabulary."""

    def __init__(self, vocab: Vocab, table: np.ndarray, distance: Distance = Distance.Cosine):
        self.vocab_ = vocab
        self.table = np.ascontiguousarray(table, np.float32)
        self.distance = distance

    @classmethod
    def new(cls, graph: Graph, dims: int, distance: Distance) -> "NodeEmbeddings":
        return cls(graph.vocab_, np.zeros((graph.nodes(), dims), np.float32), distance)

    @staticmethod
    def new_from_list(lst: Sequence[Tuple[FQNode, Sequence[float]]], distance: Distance) -> "NodeEmbeddings":
        v = Vocab()
        rows = []
        for (nt, nn), emb in lst:
            v.get_or_insert(nt, nn)
            rows.append(list(emb))
        d = max((len(r) for r in rows), default=0)
        t = np.zeros((len(v), d), np.float32)
        for (nt, nn), emb in lst:
            t[v.get_node_id(nt, nn), : len(emb)] = emb
        return NodeEmbeddings(v, t, distance)

    def __repr__(self) -> str:
        return f"NodeEmbeddings<Nodes={self.len()}, Dims={self.dims()}, Distance={self.distance.name}>"

    def contains(self, node: FQNode) -> bool:
        return self.vocab_.get_node_id(node[0], node[1]) is not None

    def get_embedding(self, node: FQNode) -> List[float]:
        return self.table[_node_id(self.vocab_, node)].tolist()

    def set_embedding(self, node: FQNode, embedding: Sequence[float]) -> None:
        self.table[_node_id(self.vocab_, node), : len(embedding)] = embedding

    def vocab(self) -> Iterator[FQNode]:
        return iter(self.vocab_)

    def get_distance(self) -> Distance:
        return self.distance

    def dims(self) -> int:
        return self.table.shape[1]

    def len(self) -> int:
        return self.table.shape[0]

    def __len__(self) -> int:
        return self.len()

    def __getitem__(self, idx: int):
        n = self.len()
        if idx < 0:
            idx += n
        if idx < 0 or idx >= n:
            raise IndexError("Index larger than embedding store!")
        return self.vocab_.get_name(idx), self.table[idx].tolist()

    def l2norm(self) -> None:
        """Row-wise L2 normalisation; zero rows untouched (lib.rs:2804-2814)."""
        n = np.sqrt(np.einsum("ij,ij->i", self.table, self.table))
        nz = n > 0
        self.table[nz] /= n[nz, None]

    def compute_distance(self, e1, e2) -> float:
        def look(e):
            if isinstance(e, tuple) and len(e) == 2 and isinstance(e[0], str):
                return self.table[_node_id(self.vocab_, e)]
            return np.asarray(e, np.float32)
        return self.distance.compute(look(e1), look(e2))

    def nearest_neighbor(self, emb, k: int, filter_type: Optional[Union[str, Sequence[str]]] = None):
        """Brute-force top-k by the store's distance (embeddings.rs:149-173)."""
        q = np.asarray(emb, np.float32)
        d = self.distance.matrix(q, self.table).astype(np.float32)
        if filter_type is not None:
            types = {filter_type} if isinstance(filter_type, str) else set(filter_type)
            mask = np.array([self.vocab_.get_node_type(i) in types for i in range(self.len())])
            d = np.where(mask, d, np.float32(np.finfo(np.float32).max))
        k = min(k, len(d))
        idx = np.argpartition(d, k - 1)[:k] if k < len(d) else np.arange(len(d))
        idx = idx[np.argsort(d[idx], kind="stable")]
        return [(self.vocab_.get_name(int(i)), float(d[i])) for i in idx]

    def nearest_neighbors(self, queries, k: int, exclude=None, device: int = 0):
        """Exact cosine top-k of many query vectors at once on the tensor
        cores (``ep_knn_cosine``): (row ids [n_q, k], cosine distances
        1 - cos [n_q, k]) in increasing distance; exclude[i] names a row to
        skip for query i.  Rows are compared after rounding the unit vectors
        to BF16.  For a Cosine store, k <= 32, dims <= 256."""
        if self.distance is not Distance.Cosine:
            raise _native.UnsupportedOption(-6, "batched nearest neighbours are implemented for cosine distance")
        ids, sim = _native.knn_cosine(self.table, queries, k, exclude, device)
        return ids, (np.float32(1) - sim).astype(np.float32)

    def save(self, path: str, comp_level: Optional[int] = None) -> None:
        """``node_type\\tname\\t[v1,v2,...]`` lines (EmbeddingWriter,
        io.rs:44-76), gzipped when the path ends with ``.gz`` (level
        comp_level, default 1, io.rs:215-227).  Rows are formatted natively
        in blocks (``ep_format_embeddings``), each value the shortest decimal
        that reads back to the same f32."""
        from .graph import NativeVocab, RangeVocab

        v, n = self.vocab_, self.len()
        if path.endswith(".gz"):
            import gzip
            f = gzip.open(path, "wb", compresslevel=1 if comp_level is None else int(comp_level))
        else:
            f = open(path, "wb")
        step = max(1, (1 << 26) // (16 * max(self.table.shape[1], 1) + 32))
        with f:
            for lo in range(0, n, step):
                hi = min(n, lo + step)
                if isinstance(v, RangeVocab) and hi <= v._n:     # names are the decimal ids
                    f.write(_native.format_embeddings(self.table[lo:hi], v._type, None, lo))
                else:
                    names = v.names(lo, hi) if isinstance(v, NativeVocab) else [v.get_name(i) for i in range(lo, hi)]
                    f.write(_native.format_embeddings(self.table[lo:hi], [t for t, _ in names],
                                                      [x for _, x in names]))

    @staticmethod
    def load(path: str, distance: Optional[Distance] = None, filter_type=None, chunk_size=None,
             skip_rows=None) -> "NodeEmbeddings":
        """Reads the format written by save (EmbeddingReader::load,
        io.rs:134-198): skip_rows leading lines are skipped, filter_type keeps
        the rows of those node types, a node seen twice raises KeyError, rows
        of different widths raise ValueError.  Blocks of lines are parsed
        natively (``ep_parse_embeddings``) and their names interned into a
        NativeVocab (``ep_vocab_intern_tokens``); a file whose names are the
        decimal ids 0..n-1 of one node type gets a RangeVocab instead.
        chunk_size is accepted for API parity."""
        from .graph import NativeVocab, RangeVocab

        types = None if filter_type is None else ({filter_type} if isinstance(filter_type, str) else set(filter_type))
        tables, dims = [], None
        run_type, total = None, 0     # while every kept row so far is (run_type, str(its index))
        v = None                      # a NativeVocab once that stops
        for buf in _line_blocks(path, skip_rows or 0):
            vals, tok = _native.parse_embeddings(buf, dims)
            if not len(vals):
                continue
            dims = vals.shape[1]
            raw = np.frombuffer(buf, np.uint8)
            one = _one_type(raw, tok)
            if types is not None:
                if one is not None:
                    if one not in types:
                        continue
                else:
                    keep = np.array([buf[a:b].decode() in types for a, b in tok[:, :2].tolist()], bool)
                    vals, tok = vals[keep], tok[keep]
                    if not len(vals):
                        continue
            if v is None and one is not None and (run_type is None or one == run_type) and \
                    _decimal_run(raw, tok) == total:
                run_type = one
            else:
                if v is None:
                    v = NativeVocab()
                    for i in range(total):
                        v.get_or_insert(run_type, str(i))
                ids = v._v.intern_tokens(buf, tok)
                bad = np.nonzero(ids != np.arange(total, total + len(ids)))[0]
                if len(bad):
                    raise KeyError(f"found duplicate node at {total + int(bad[0])}!")
            tables.append(vals)
            total += len(vals)
        t = np.concatenate(tables) if tables else np.zeros((0, dims or 0), np.float32)
        if v is None:
            v = RangeVocab(total, run_type) if run_type is not None else Vocab()
        return NodeEmbeddings(v, t, distance or Distance.Cosine)


def _line_blocks(path: str, skip_rows: int, block: int = 1 << 24):
    """Blocks of whole lines of a (possibly gzipped) text file, after
    skip_rows leading lines."""
    import gzip

    with (gzip.open(path, "rb") if path.endswith(".gz") else open(path, "rb")) as f:
        for _ in range(skip_rows):
            if not f.readline():
                return
        rest = b""
        while True:
            chunk = f.read(block)
            if not chunk:
                break
            data = rest + chunk if rest else chunk
            cut = data.rfind(b"\n")
            if cut < 0:
                rest = data
                continue
            yield data[: cut + 1]
            rest = data[cut + 1:]
        if rest:
            yield rest


def _one_type(raw: np.ndarray, tok: np.ndarray) -> Optional[str]:
    """The node type when every row of the block has the same one."""
    tl = (tok[:, 1] - tok[:, 0]).astype(np.int64)
    if (tl != tl[0]).any():
        return None
    first = raw[int(tok[0, 0]): int(tok[0, 1])]
    if tl[0] and (raw[tok[:, :1].astype(np.int64) + np.arange(tl[0])] != first).any():
        return None
    return first.tobytes().decode()


def _decimal_run(raw: np.ndarray, tok: np.ndarray) -> Optional[int]:
    """f when the names of the block are the decimals f, f + 1, ... (no
    leading zeros), else None."""
    beg = tok[:, 2].astype(np.int64)
    ln = (tok[:, 3] - tok[:, 2]).astype(np.int64)
    if not 1 <= ln.min() <= ln.max() <= 18:
        return None
    cols = np.arange(int(ln.max()))
    m = cols < ln[:, None]
    dig = raw[np.minimum(beg[:, None] + cols, len(raw) - 1)].astype(np.int64) - 48
    if ((dig < 0) | (dig > 9))[m].any() or ((dig[:, 0] == 0) & (ln > 1)).any():
        return None
    val = np.zeros(len(beg), np.int64)
    for j in range(len(cols)):
        val = np.where(m[:, j], val * 10 + dig[:, j], val)
    f = int(val[0])
    return f if (val == f + np.arange(len(val))).all() else None


class FeatureAggregator:
    """How node embeddings are formed from feature embeddings
    (lib.rs:1772-2000): Averaged, Weighted (SIF) or Attention.  Attention
    aggregation is a separate model outside the EP training path: it can be
    built, printed, saved and loaded, but embedding with it raises
    UnsupportedOption."""

    def __init__(self, kind: str, alpha: float = 0.0, unigrams: Optional[np.ndarray] = None,
                 vocab: Optional[Vocab] = None, heads: int = 0, d_k: int = 0, window: Optional[int] = None):
        self.kind, self.alpha, self.unigrams, self.vocab = kind, alpha, unigrams, vocab
        self.heads, self.d_k, self.window = heads, d_k, window

    @staticmethod
    def Averaged() -> "FeatureAggregator":
        return FeatureAggregator("averaged")

    @staticmethod
    def Weighted(alpha: float, feature_set) -> "FeatureAggregator":
        """SIF weights alpha / (alpha + p(feature)) (aggregator.rs:50-120)."""
        counts = feature_set.count_features().astype(np.float64)
        p = (counts / max(counts.sum(), 1.0)).astype(np.float32)
        return FeatureAggregator("weighted", float(alpha), p, feature_set.feature_vocab)

    @staticmethod
    def Attention(num_heads: int, d_k: int, window: Optional[int] = None) -> "FeatureAggregator":
        return FeatureAggregator("attention", heads=int(num_heads), d_k=int(d_k), window=window)

    def __repr__(self) -> str:
        if self.kind == "weighted":
            t = f"Weighted<alpha={_rust_float(self.alpha, np.float32)}>"
        elif self.kind == "attention":
            w = "None" if self.window is None else f"Some({self.window})"
            t = f"Attention<num_heads={self.heads},d_k={self.d_k},window={w}"
        else:
            t = "Averaged"
        return f"FeatureAggregator<{t}>"

    def save(self, path: str) -> None:
        """The aggregator's text form (lib.rs:1876-1913): its kind, then
        alpha and one ``type\\tname\\tp`` line per feature (Weighted), or
        the head count, d_k and window (0 = none) (Attention)."""
        with open(path, "w") as f:
            if self.kind == "averaged":
                f.write("Averaged\n")
            elif self.kind == "attention":
                f.write(f"Attention\n{self.heads}\n{self.d_k}\n{self.window or 0}\n")
            else:
                f.write(f"Weighted\n{_rust_float(self.alpha, np.float32)}\n")
                for i, p in enumerate(np.asarray(self.unigrams, np.float32).tolist()):
                    if i >= len(self.vocab):
                        break
                    nt, nn = self.vocab.get_name(i)
                    f.write(f"{nt}\t{nn}\t{_rust_float(p, np.float64)}\n")

    @staticmethod
    def load(path: str) -> "FeatureAggregator":
        """Reads the form written by save (lib.rs:1928-2000)."""
        with open(path) as f:
            kind = f.readline().rstrip("\r\n")
            if kind == "Averaged":
                return FeatureAggregator.Averaged()
            if kind == "Attention":
                vals = []
                for _ in range(3):
                    line = f.readline().rstrip("\r\n")
                    if not line.isdigit():
                        raise ValueError(f"invalid dim! {line!r}")
                    vals.append(int(line))
                return FeatureAggregator.Attention(vals[0], vals[1], vals[2] or None)
            if kind != "Weighted":
                raise ValueError(f"Unknown aggregator type: {kind}")
            line = f.readline().rstrip("\r\n")
            try:
                alpha = float(np.float32(float(line)))
            except ValueError:
                raise ValueError(f"invalid dim! {line!r}") from None
            v, p = Vocab(), []
            for line in f:
                pieces = line.rstrip("\n").split("\t")
                if len(pieces) != 3:
                    raise ValueError("Malformed feature line! Need node_type<TAB>name<TAB>weight ...")
                try:
                    pw = float(pieces[2])
                except ValueError:
                    raise ValueError(f"Tried to parse weight and failed:{line!r}") from None
                if v.get_or_insert(pieces[0], pieces[1]) < len(p):
                    raise ValueError(f"Duplicate feature found:{pieces[0]} {pieces[1]}")
                p.append(pw)
            return FeatureAggregator("weighted", alpha, np.array(p, np.float32), v)


def _rust_float(x: float, ty) -> str:
    """x as Rust's Display writes an f32 / f64: shortest round-trip digits of
    that type, positional."""
    return np.format_float_positional(ty(x), unique=True, trim="-")


class NodeEmbedder:
    """Builds node embeddings from a FeatureSet and feature embeddings."""

    def __init__(self, feat_agg: FeatureAggregator):
        self.feat_agg = feat_agg

    def __repr__(self) -> str:
        return f"NodeEmbedder<aggregator={self.feat_agg!r}>"

    def _translate(self, feat_set, feature_embeddings: NodeEmbeddings) -> Tuple[np.ndarray, np.ndarray]:
        fptr, fids = feat_set.to_csr()
        fv, ev = feat_set.feature_vocab, feature_embeddings.vocab_
        if fv is ev:
            return fptr, fids.astype(np.int64)
        n = len(fv)
        tr = np.full(n, -1, np.int64)
        for i in range(n):
            j = ev.get_node_id(*fv.get_name(i))
            if j is not None:
                tr[i] = j
        return fptr, tr[fids]

    def embed_feature_set(self, feat_set, feature_embeddings: NodeEmbeddings, device: int = 0) -> NodeEmbeddings:
        """Mean (or SIF-weighted mean) of each node's known feature rows on the
        GPU (``ep_embed_features``); nodes without known features stay zero
        (lib.rs:2092-2124).  As the reference, the SIF weight of a feature is
        looked up by its row in feature_embeddings (aggregator.rs:103-110)."""
        if self.feat_agg.kind == "attention":
            raise _native.UnsupportedOption(-6, "attention aggregation is not implemented")
        fptr, ids = self._translate(feat_set, feature_embeddings)
        T = feature_embeddings.table
        n = len(fptr) - 1
        node = np.repeat(np.arange(n), np.diff(fptr).astype(np.int64))
        keep = ids >= 0
        kept = np.zeros(n + 1, np.uint64)
        kept[1:] = np.cumsum(np.bincount(node[keep], minlength=n))
        ids = ids[keep]
        fw = None
        if self.feat_agg.kind == "weighted":
            p = np.asarray(self.feat_agg.unigrams, np.float32)
            if len(ids) and ids.max() >= len(p):
                raise IndexError("a feature row beyond the aggregator's unigram table")
            a = np.float32(self.feat_agg.alpha)
            fw = np.ones(T.shape[0], np.float32)
            m = min(len(p), T.shape[0])
            fw[:m] = a / (a + p[:m])
        out = _native.embed_features(kept, ids.astype(np.uint32), T, fw, device)
        return NodeEmbeddings(feat_set.vocab_, out, Distance.Cosine)

    def embed_adhoc(self, features: Sequence[FQNode], feature_embeddings: NodeEmbeddings,
                    strict: Optional[bool] = None) -> List[float]:
        strict = True if strict is None else strict
        ids = []
        for nt, nn in features:
            i = feature_embeddings.vocab_.get_node_id(nt, nn)
            if i is not None:
                ids.append(i)
            elif strict:
                raise KeyError(f"Feature {nt} {nn} does not exist!")
        out = np.zeros(feature_embeddings.dims(), np.float32)
        if ids:
            out = feature_embeddings.table[ids].mean(0)
        return out.tolist()

    def bulk_embed_adhoc(self, features_set, feature_embeddings: NodeEmbeddings, strict=None):
        return [self.embed_adhoc(f, feature_embeddings, strict) for f in features_set]
