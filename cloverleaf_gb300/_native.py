"""ctypes binding of ``include/ep_gb300.h``.

The shared library is the product path: every training call goes through it,
and loading fails loudly (``NativeError``) when it cannot be built or loaded;
there is no Python fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

ABI_VERSION = 2

EP_OK = 0
_STATUS = {
    -1: "invalid argument", -2: "CUDA error", -3: "out of device memory", -4: "bad call order",
    -5: "device error flag", -6: "unsupported option", -7: "no CUDA device",
}
LOSS_MARGIN, LOSS_STARSPACE, LOSS_CONTRASTIVE, LOSS_RANK, LOSS_RANKSPACE, LOSS_PPR = 0, 1, 2, 3, 4, 5
SAMPLE_ALL, SAMPLE_FIXED, SAMPLE_PROB = 0, 1, 2
LW_NONE, LW_LOG, LW_EXP = 0, 1, 2
FORM_PLAIN_FP32, FORM_FUSED_BF16 = 0, 1
GRAD_REFERENCE, GRAD_TRUE = 0, 1


class NativeError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} ({_STATUS.get(code, 'error')} {code})")
        self.code = code


class UnsupportedOption(NativeError, NotImplementedError):
    pass


class EpConfig(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_uint32),
        ("alpha", ctypes.c_float),
        ("loss", ctypes.c_int32),
        ("gamma", ctypes.c_float),
        ("neg_margin", ctypes.c_float),
        ("negatives", ctypes.c_uint32),
        ("batch_size", ctypes.c_uint32),
        ("dims", ctypes.c_uint32),
        ("passes", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
        ("max_nodes_kind", ctypes.c_int32),
        ("max_nodes", ctypes.c_float),
        ("max_features_kind", ctypes.c_int32),
        ("max_features", ctypes.c_float),
        ("weighted_neighbor_sampling", ctypes.c_int32),
        ("weighted_neighbor_averaging", ctypes.c_int32),
        ("loss_weighting", ctypes.c_int32),
        ("loss_weighting_exp", ctypes.c_float),
        ("valid_pct", ctypes.c_float),
        ("hard_negatives", ctypes.c_uint32),
        ("noise", ctypes.c_float),
        ("form", ctypes.c_int32),
        ("grad_mode", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("use_graphs", ctypes.c_int32),
        ("autotune", ctypes.c_int32),
        ("ppr_restart_p", ctypes.c_float),
    ]


class EpPassStats(ctypes.Structure):
    _fields_ = [
        ("pass_", ctypes.c_uint32),
        ("batches", ctypes.c_uint32),
        ("train_loss", ctypes.c_float),
        ("valid_loss", ctypes.c_float),
        ("lr_last", ctypes.c_float),
        ("noise_last", ctypes.c_float),
        ("anchors", ctypes.c_uint64),
        ("kept_anchors", ctypes.c_uint64),
        ("nan_anchors", ctypes.c_uint64),
        ("items", ctypes.c_uint64),
        ("gathered_rows", ctypes.c_uint64),
        ("unique_rows", ctypes.c_uint64),
        ("sampled_neighbors", ctypes.c_uint64),
        ("ms", ctypes.c_double),
        ("alg_bytes", ctypes.c_double),
        ("launches", ctypes.c_uint64),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["pass"] = d.pop("pass_")
        return d


class EpLaunchShape(ctypes.Structure):
    _fields_ = [("chunk", ctypes.c_uint32), ("fused_mode", ctypes.c_int32), ("graph_batches", ctypes.c_uint32),
                ("gather_ctas", ctypes.c_uint32), ("ring_reduce_warps", ctypes.c_uint32),
                ("ring_adam_warps", ctypes.c_uint32), ("ring_slots", ctypes.c_uint32), ("ring_active", ctypes.c_int32),
                ("queue_ctas_per_sm", ctypes.c_uint32), ("gather_warps", ctypes.c_uint32), ("tuned", ctypes.c_int32), ("autotune", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class EpBatchSamples(ctypes.Structure):
    _fields_ = [
        ("n_anchors", ctypes.c_uint32),
        ("anchors", ctypes.c_void_p),
        ("nbr_ptr", ctypes.c_void_p),
        ("nbr", ctypes.c_void_p),
        ("nbr_w", ctypes.c_void_p),
        ("negatives", ctypes.c_void_p),
    ]


class EpSparseGrad(ctypes.Structure):
    _fields_ = [
        ("capacity", ctypes.c_uint32),
        ("n_rows", ctypes.c_uint32),
        ("feat_ids", ctypes.c_void_p),
        ("rows", ctypes.c_void_p),
        ("loss", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
    ]


_lock = threading.Lock()
_lib = None

# name -> (restype, argtypes)
_P = ctypes.c_void_p
_U32, _U64, _I32, _F32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float
SIGNATURES = {
    "ep_config_default": (None, [ctypes.POINTER(EpConfig)]),
    "ep_create": (ctypes.c_int, [ctypes.POINTER(EpConfig), ctypes.POINTER(_P)]),
    "ep_upload_graph": (ctypes.c_int, [_P, _U64, _P, _P, _P]),
    "ep_upload_features": (ctypes.c_int, [_P, _U64, _P, _P, _U32]),
    "ep_set_table": (ctypes.c_int, [_P, _P]),
    "ep_train": (ctypes.c_int, [_P, ctypes.POINTER(EpPassStats), _U32]),
    "ep_train_batches": (ctypes.c_int, [_P, _U32, ctypes.POINTER(EpPassStats)]),
    "ep_profile_batches": (ctypes.c_int, [_P, _U32, _P, ctypes.POINTER(EpPassStats)]),
    "ep_batch_grad": (ctypes.c_int, [_P, ctypes.POINTER(EpBatchSamples), ctypes.POINTER(EpSparseGrad)]),
    "ep_batch_step": (ctypes.c_int, [_P, ctypes.POINTER(EpBatchSamples), _F32, _U32]),
    "ep_get_table": (ctypes.c_int, [_P, _P]),
    "ep_get_table_static": (ctypes.c_int, [_P, _U64, _U64, _P]),
    "ep_get_tuning": (ctypes.c_int, [_P, _P, _P, _P]),
    "ep_sample": (ctypes.c_int, [_P, _P, _U32, _U32, _U32, _P, _P, _P, _P]),
    "ep_embed_features": (ctypes.c_int, [ctypes.c_int, _U64, _P, _P, _P, _U32, _U32, _P, _P]),
    "ep_knn_cosine": (ctypes.c_int, [ctypes.c_int, _U64, _U32, _P, _U64, _P, _P, _U32, _P, _P]),
    "ep_align": (ctypes.c_int, [ctypes.c_int, _U64, _P, _P, _P, _U32, _P, ctypes.c_float, _U64, _P]),
    "ep_knn_last_error": (ctypes.c_char_p, []),
    "ep_knn_last_kernel_ms": (ctypes.c_float, []),
    "ep_ag_forward": (ctypes.c_int, [_P, ctypes.POINTER(EpBatchSamples), ctypes.c_int, _P, _P, _P]),
    "ep_ag_backward": (ctypes.c_int, [_P, _P, _P, _P]),
    "ep_get_split": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
    "ep_get_launch_shape": (ctypes.c_int, [_P, _P]),
    "ep_sample_validation": (ctypes.c_int, [_P, _U32, _U32, _U32, _P, _P, _P, _P, _P]),
    "ep_selftest_stochastic_rounding": (ctypes.c_int, [ctypes.c_int, _U64, _U64, ctypes.POINTER(_U64)]),
    "ep_synchronize": (ctypes.c_int, [_P]),
    "ep_last_error": (ctypes.c_char_p, [_P]),
    "ep_destroy": (None, [_P]),
    "ep_csr_from_edges": (ctypes.c_int, [_U64, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P, _P]),
    "ep_cdf_convert": (ctypes.c_int, [_U64, _P, _P]),
    "ep_format_embeddings": (ctypes.c_int64, [_U64, _U32, _P, _P, _P, _P, _P, _U64, _P, _U64]),
    "ep_parse_embeddings": (ctypes.c_int64, [_P, _U64, ctypes.POINTER(_U32), _P, _P, ctypes.POINTER(_U64)]),
    "ep_propagate_features": (ctypes.c_int64, [_U64, _P, _P, _P, _P, _P, _U32, _U32, _F32, _P, _P, _U64]),
    "ep_vocab_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "ep_vocab_destroy": (None, [_P]),
    "ep_vocab_len": (_U64, [_P]),
    "ep_vocab_max_key": (_U64, [_P]),
    "ep_vocab_intern": (ctypes.c_int64, [_P, ctypes.c_char_p, _U64, ctypes.c_char_p, _U64]),
    "ep_vocab_find": (ctypes.c_int64, [_P, ctypes.c_char_p, _U64, ctypes.c_char_p, _U64]),
    "ep_vocab_intern_tokens": (ctypes.c_int, [_P, _P, _P, _U64, _P]),
    "ep_vocab_range_bytes": (ctypes.c_int, [_P, _U64, _U64, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "ep_vocab_export": (ctypes.c_int, [_P, _U64, _U64, _P, _P, _P, _P]),
    "ep_parse_edges": (ctypes.c_int64, [_P, _P, _U64, ctypes.c_int, _P, _P, _P, _U64, ctypes.POINTER(_U64)]),
    "ep_format_edges": (ctypes.c_int64, [_P, ctypes.c_char_p, _U64, _P, _P, _P, _U64, _U64, _P, _U64]),
}


def lib():
    """Loads (building first when needed) the native library."""
    global _lib
    with _lock:
        if _lib is None:
            try:
                path = _build.build()
            except Exception as e:  # no toolchain / compile error
                if not os.path.exists(_build.LIB_PATH):
                    raise NativeError(-2, f"cannot build libep_gb300.so: {e}") from e
                path = _build.LIB_PATH
            handle = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


def check(rc: int, ctx=None, what: str = ""):
    if rc == EP_OK:
        return
    msg = lib().ep_last_error(ctx).decode(errors="replace")
    cls = UnsupportedOption if rc == -6 else NativeError
    raise cls(rc, f"{what}: {msg}" if what else msg)


def default_config() -> EpConfig:
    cfg = EpConfig()
    lib().ep_config_default(ctypes.byref(cfg))
    return cfg


class Context:
    """Owns one ``ep_ctx``; thin RAII wrapper used by the Python API."""

    def __init__(self, cfg: EpConfig):
        self._h = ctypes.c_void_p()
        check(lib().ep_create(ctypes.byref(cfg), ctypes.byref(self._h)), None, "ep_create")
        self.cfg = cfg

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().ep_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_graph(self, rows, cols, wcdf=None):
        rows = np.ascontiguousarray(rows, np.uint64)
        cols = np.ascontiguousarray(cols, np.uint32)
        w = None if wcdf is None else np.ascontiguousarray(wcdf, np.float32)
        check(lib().ep_upload_graph(self._h, len(rows) - 1, ptr(rows), ptr(cols), ptr(w)), self._h, "ep_upload_graph")

    def upload_features(self, fptr, fids, n_feat):
        fptr = np.ascontiguousarray(fptr, np.uint64)
        fids = np.ascontiguousarray(fids, np.uint32)
        check(lib().ep_upload_features(self._h, len(fptr) - 1, ptr(fptr), ptr(fids), int(n_feat)), self._h,
              "ep_upload_features")

    def set_table(self, table=None):
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        check(lib().ep_set_table(self._h, ptr(t)), self._h, "ep_set_table")

    def sample(self, anchors, step, stride):
        """Device sampler output for given anchors: (nbr_cnt, nbr[n, stride],
        nbr_w[n, stride], neg[n, R])."""
        anchors = np.ascontiguousarray(anchors, np.uint32)
        n = len(anchors)
        cnt = np.zeros(n, np.uint32)
        nbr = np.zeros((n, stride), np.uint32)
        w = np.zeros((n, stride), np.float32)
        neg = np.zeros((n, self.cfg.negatives), np.uint32)
        check(lib().ep_sample(self._h, ptr(anchors), n, int(step), int(stride), ptr(cnt), ptr(nbr), ptr(w), ptr(neg)),
              self._h, "ep_sample")
        return cnt, nbr, w, neg

    def split(self):
        """(train ids, validation ids in validation order) of this context's
        seeded train/validation split."""
        nt, nv = ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().ep_get_split(self._h, None, None, ctypes.byref(nt), ctypes.byref(nv)), self._h, "ep_get_split")
        tr = np.zeros(max(nt.value, 1), np.uint32)
        va = np.zeros(max(nv.value, 1), np.uint32)
        check(lib().ep_get_split(self._h, ptr(tr), ptr(va), ctypes.byref(nt), ctypes.byref(nv)), self._h,
              "ep_get_split")
        return tr[: nt.value], va[: nv.value]

    def sample_validation(self, first, n, stride):
        """The validation pass's samples at validation positions [first,
        first + n): (anchors, nbr_cnt, nbr[n, stride], nbr_w[n, stride],
        neg[n, R])."""
        anchors = np.zeros(n, np.uint32)
        cnt = np.zeros(n, np.uint32)
        nbr = np.zeros((n, stride), np.uint32)
        w = np.zeros((n, stride), np.float32)
        neg = np.zeros((n, self.cfg.negatives), np.uint32)
        check(lib().ep_sample_validation(self._h, int(first), int(n), int(stride), ptr(anchors), ptr(cnt), ptr(nbr),
                                         ptr(w), ptr(neg)), self._h, "ep_sample_validation")
        return anchors, cnt, nbr, w, neg

    def launch_shape(self):
        """Every launch shape in use (ep_get_launch_shape) as a dict."""
        out = EpLaunchShape()
        check(lib().ep_get_launch_shape(self._h, ctypes.byref(out)), self._h, "ep_get_launch_shape")
        return out.as_dict()

    def tuning(self):
        """(tuned, chunk, fused_mode, graph_batches) of this context."""
        ch, fm, gb = ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_uint32()
        rc = lib().ep_get_tuning(self._h, ctypes.byref(ch), ctypes.byref(fm), ctypes.byref(gb))
        if rc < 0:
            check(rc, self._h, "ep_get_tuning")
        return rc == 0, ch.value, fm.value, gb.value

    def get_table(self, n_feat, dims, out=None):
        """The table as FP32 [n_feat, dims], into `out` when given (a
        contiguous float32 array, e.g. in pinned memory)."""
        if out is None:
            out = np.empty((n_feat, dims), np.float32)
        elif out.dtype != np.float32 or out.shape != (n_feat, dims) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous float32 array of shape (n_feat, dims)")
        check(lib().ep_get_table(self._h, ptr(out)), self._h, "ep_get_table")
        return out

    def train(self, passes):
        stats = (EpPassStats * max(passes, 1))()
        check(lib().ep_train(self._h, stats, passes), self._h, "ep_train")
        return [s.as_dict() for s in stats[:passes]]

    def train_batches(self, n):
        st = EpPassStats()
        check(lib().ep_train_batches(self._h, n, ctypes.byref(st)), self._h, "ep_train_batches")
        return st.as_dict()

    STAGES = ("sample", "forward", "sort", "reduce", "fixup", "adam", "end")

    def profile_batches(self, n):
        ms = (ctypes.c_double * len(self.STAGES))()
        st = EpPassStats()
        check(lib().ep_profile_batches(self._h, n, ms, ctypes.byref(st)), self._h, "ep_profile_batches")
        return dict(zip(self.STAGES, list(ms))), st.as_dict()

    @staticmethod
    def samples(anchors, nbr_ptr, nbr, nbr_w, negatives):
        arrs = dict(anchors=np.ascontiguousarray(anchors, np.uint32),
                    nbr_ptr=np.ascontiguousarray(nbr_ptr, np.uint32),
                    nbr=np.ascontiguousarray(nbr if len(nbr) else [0], np.uint32),
                    nbr_w=np.ascontiguousarray(nbr_w if len(nbr_w) else [0], np.float32),
                    negatives=np.ascontiguousarray(negatives, np.uint32).reshape(-1))
        s = EpBatchSamples(len(arrs["anchors"]), ptr(arrs["anchors"]), ptr(arrs["nbr_ptr"]), ptr(arrs["nbr"]),
                           ptr(arrs["nbr_w"]), ptr(arrs["negatives"]))
        return s, arrs   # keep arrays alive with the struct

    def batch_grad(self, samples, n_feat, dims):
        s, keep = samples
        B = s.n_anchors
        ids = np.zeros(n_feat, np.uint32)
        rows = np.zeros((n_feat, dims), np.float32)
        loss = np.zeros(B, np.float32)
        status = np.zeros(B, np.int32)
        g = EpSparseGrad(n_feat, 0, ptr(ids), ptr(rows), ptr(loss), ptr(status))
        check(lib().ep_batch_grad(self._h, ctypes.byref(s), ctypes.byref(g)), self._h, "ep_batch_grad")
        n = g.n_rows
        return loss, status, ids[:n].copy(), rows[:n].copy()

    def batch_step(self, samples, lr, pass_idx):
        s, keep = samples
        check(lib().ep_batch_step(self._h, ctypes.byref(s), float(lr), int(pass_idx)), self._h, "ep_batch_step")

    def ag_forward(self, samples, precision, table_ptr, loss_ptr, stream):
        s, keep = samples
        check(lib().ep_ag_forward(self._h, ctypes.byref(s), precision, ctypes.c_void_p(table_ptr),
                                  ctypes.c_void_p(loss_ptr), ctypes.c_void_p(stream)), self._h, "ep_ag_forward")

    def ag_backward(self, dloss_ptr, grad_ptr, stream):
        check(lib().ep_ag_backward(self._h, ctypes.c_void_p(dloss_ptr), ctypes.c_void_p(grad_ptr),
                                   ctypes.c_void_p(stream)), self._h, "ep_ag_backward")


def csr_from_edges(src, dst, w, dedup=True):
    """graph.rs:70-142 through the C ABI.  Returns (rows u64, cols u32, w f32)."""
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    w = np.ascontiguousarray(w, np.float32)
    n = len(src)
    max_node = int(max(src.max(initial=0), dst.max(initial=0)))
    rows = np.zeros(max_node + 2, np.uint64)
    cols = np.zeros(max(n, 1), np.uint32)
    wo = np.zeros(max(n, 1), np.float32)
    nn, ne = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().ep_csr_from_edges(n, ptr(src), ptr(dst), ptr(w), int(dedup), ptr(rows), ptr(cols), ptr(wo),
                                  ctypes.byref(nn), ctypes.byref(ne)), None, "ep_csr_from_edges")
    return rows[: nn.value + 1], cols[: ne.value], wo[: ne.value]


def cdf_convert(rows, w):
    rows = np.ascontiguousarray(rows, np.uint64)
    w = np.ascontiguousarray(w, np.float32).copy()
    check(lib().ep_cdf_convert(len(rows) - 1, ptr(rows), ptr(w)), None, "ep_cdf_convert")
    return w


def _strings(strs):
    """A list of str as (utf-8 bytes as uint8, n+1 uint64 offsets)."""
    enc = [x.encode() for x in strs]
    off = np.zeros(len(enc) + 1, np.uint64)
    np.cumsum([len(x) for x in enc], out=off[1:])
    return np.frombuffer(b"".join(enc), np.uint8) if off[-1] else np.zeros(1, np.uint8), off


def format_embeddings(table, types, names=None, first_id=0) -> bytes:
    """EmbeddingWriter::stream (io.rs:44-76) for the rows of table: types is
    one str for every row or a list of str; names a list of str, or None for
    the decimal ids first_id, first_id + 1, ...  (``ep_format_embeddings``)."""
    table = np.ascontiguousarray(table, np.float32)
    n, dims = table.shape
    if isinstance(types, str):
        tbuf, toff = np.frombuffer(types.encode() + b"\0", np.uint8), None
    else:
        if len(types) != n:
            raise ValueError(f"{len(types)} types for {n} rows")
        tbuf, toff = _strings(types)
    nbuf = noff = None
    if names is not None:
        if len(names) != n:
            raise ValueError(f"{len(names)} names for {n} rows")
        nbuf, noff = _strings(names)
    cap = n * (16 * dims + 25) + (int(toff[-1]) if toff is not None else n * len(tbuf))
    cap += int(noff[-1]) if noff is not None else 0
    out = np.empty(max(cap, 1), np.uint8)
    rc = lib().ep_format_embeddings(n, dims, ptr(table), ptr(tbuf), ptr(toff), ptr(nbuf), ptr(noff), int(first_id),
                                    ptr(out), cap)
    if rc < 0:
        check(int(rc), None, "ep_format_embeddings")
    return out[:rc].tobytes()


def parse_embeddings(buf: bytes, dims=None):
    """line_to_embedding (io.rs:246-262) over a block of whole lines:
    (values [rows, dims] f32, token offsets [rows, 4] u64 as type begin/end,
    name begin/end).  dims, when given, is the width every row must have.
    Raises ValueError naming the first bad line.  (``ep_parse_embeddings``)"""
    arr = np.frombuffer(buf, np.uint8)
    d = _U32(0)
    bad = _U64(0)
    rows = int(lib().ep_parse_embeddings(ptr(arr), len(arr), ctypes.byref(d), None, None, ctypes.byref(bad)))
    if rows < 0:
        check(rows, None, "ep_parse_embeddings")
    if rows and d.value == 0:
        raise ValueError(f"Error parsing line: {_line(buf, 1)[:200]!r}")
    if dims is not None:
        d = _U32(int(dims))
    vals = np.empty((max(rows, 1), d.value), np.float32)
    tok = np.empty((max(rows, 1), 4), np.uint64)
    got = lib().ep_parse_embeddings(ptr(arr), len(arr), ctypes.byref(d), ptr(vals), ptr(tok), ctypes.byref(bad))
    if got < 0:
        if not bad.value:
            check(int(got), None, "ep_parse_embeddings")
        line = _line(buf, bad.value)
        alone = _U32(0)
        one = np.frombuffer(line, np.uint8)
        if lib().ep_parse_embeddings(ptr(one), len(one), ctypes.byref(alone), None, None, None) == 1 and alone.value:
            raise ValueError(f"Embeddings have different sizes! ({alone.value} values, expected {d.value}, "
                             f"line: {line[:200]!r})")
        raise ValueError(f"Error parsing line: {line[:200]!r}")
    return vals[:got], tok[:got]


class NativeVocabHandle:
    """Owns an ``ep_vocab``."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().ep_vocab_create(ctypes.byref(h)), None, "ep_vocab_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ep_vocab_destroy(self.h)
            self.h = None

    def __len__(self) -> int:
        return int(lib().ep_vocab_len(self.h))

    def intern(self, node_type: str, name: str) -> int:
        t, n = node_type.encode(), name.encode()
        r = int(lib().ep_vocab_intern(self.h, t, len(t), n, len(n)))
        if r < 0:
            check(r, None, "ep_vocab_intern")
        return r

    def find(self, node_type: str, name: str) -> int:
        t, n = node_type.encode(), name.encode()
        return int(lib().ep_vocab_find(self.h, t, len(t), n, len(n)))

    def intern_tokens(self, buf: bytes, tok: np.ndarray) -> np.ndarray:
        """Ids of the keys of buf at the (type, name) byte ranges tok [n, 4]."""
        arr = np.frombuffer(buf, np.uint8)
        tok = np.ascontiguousarray(tok, np.uint64)
        ids = np.empty(max(len(tok), 1), np.uint32)
        check(lib().ep_vocab_intern_tokens(self.h, ptr(arr), ptr(tok), len(tok), ptr(ids)), None,
              "ep_vocab_intern_tokens")
        return ids[:len(tok)]

    def export(self, lo: int, hi: int):
        """(types, names) of ids [lo, hi) as lists of str."""
        tb, nb = _U64(0), _U64(0)
        check(lib().ep_vocab_range_bytes(self.h, lo, hi, ctypes.byref(tb), ctypes.byref(nb)), None, "ep_vocab_export")
        types = np.empty(max(tb.value, 1), np.uint8)
        names = np.empty(max(nb.value, 1), np.uint8)
        toff = np.empty(hi - lo + 1, np.uint64)
        noff = np.empty(hi - lo + 1, np.uint64)
        check(lib().ep_vocab_export(self.h, lo, hi, ptr(types), ptr(toff), ptr(names), ptr(noff)), None,
              "ep_vocab_export")
        tbytes, nbytes = types.tobytes(), names.tobytes()
        to, no = toff.tolist(), noff.tolist()
        return ([tbytes[to[i]:to[i + 1]].decode() for i in range(hi - lo)],
                [nbytes[no[i]:no[i + 1]].decode() for i in range(hi - lo)])


def parse_edges(vocab: NativeVocabHandle, buf: bytes, weighted: bool):
    """GraphReader::load's line step (io.rs:270-323) through
    ``ep_parse_edges``: (src ids, dst ids, weights) of the block's lines."""
    arr = np.frombuffer(buf, np.uint8)
    cap = buf.count(b"\n") + 1
    src = np.empty(cap, np.uint32)
    dst = np.empty(cap, np.uint32)
    w = np.empty(cap, np.float32)
    bad = _U64(0)
    n = int(lib().ep_parse_edges(vocab.h, ptr(arr), len(arr), int(bool(weighted)), ptr(src), ptr(dst), ptr(w), cap,
                                 ctypes.byref(bad)))
    if n < 0:
        if bad.value:
            raise ValueError(f"Malformed graph file: expected 5 fields with a numeric weight, got "
                             f"{_line(buf, bad.value)[:200]!r}")
        check(n, None, "ep_parse_edges")
    return src[:n], dst[:n], w[:n]


def format_edges(vocab, rows, cols, cdf, lo: int, hi: int) -> bytes:
    """Graph::save (lib.rs:414-430) lines of the rows of nodes [lo, hi)
    (``ep_format_edges``).  vocab: a NativeVocabHandle, or a str naming the
    node type of a vocabulary whose names are the decimal ids."""
    rows = np.ascontiguousarray(rows, np.uint64)
    cols = np.ascontiguousarray(cols, np.uint32)
    cdf = np.ascontiguousarray(cdf, np.float32)
    n = len(rows) - 1
    ne = int(rows[hi] - rows[lo])
    if isinstance(vocab, str):
        h, anon = None, vocab.encode()
        longest = len(anon) + 20
    else:
        h, anon = vocab.h, None
        longest = int(lib().ep_vocab_max_key(vocab.h))
    cap = ne * (2 * longest + 54) + 1
    out = np.empty(cap, np.uint8)
    r = int(lib().ep_format_edges(h, anon, n, ptr(rows), ptr(cols), ptr(cdf), lo, hi, ptr(out), cap))
    if r < 0:
        check(r, None, "ep_format_edges")
    return out[:r].tobytes()


def propagate_features(rows, cols, cdf, fptr, fids, max_iters: int, k: int, threshold: float):
    """propagate_features (feat_propagation.rs:13-93) through
    ``ep_propagate_features``: the new (fptr, fids)."""
    rows = np.ascontiguousarray(rows, np.uint64)
    cols = np.ascontiguousarray(cols, np.uint32)
    cdf = np.ascontiguousarray(cdf, np.float32)
    fptr = np.ascontiguousarray(fptr, np.uint64)
    fids = np.ascontiguousarray(fids, np.uint32)
    n = len(fptr) - 1
    if len(rows) != n + 1:
        raise ValueError(f"graph has {len(rows) - 1} nodes, feature set {n}")
    missing = int((np.diff(fptr) == 0).sum())
    cap = int(fptr[-1]) + missing * int(k)
    fptr_out = np.zeros(n + 1, np.uint64)
    fids_out = np.zeros(max(cap, 1), np.uint32)
    rc = lib().ep_propagate_features(n, ptr(rows), ptr(cols), ptr(cdf), ptr(fptr), ptr(fids), int(max_iters), int(k),
                                     float(threshold), ptr(fptr_out), ptr(fids_out), cap)
    if rc < 0:
        check(int(rc), None, "ep_propagate_features")
    return fptr_out, fids_out[:rc]


def _line(buf: bytes, k: int) -> bytes:
    """The k-th (1-based) non-blank line of buf."""
    for line in buf.split(b"\n"):
        if line and line != b"\r":
            k -= 1
            if k == 0:
                return line.rstrip(b"\r")
    return b""


def selftest_stochastic_rounding(n=1 << 24, seed=1, device=0) -> int:
    """Pairs (of n) whose hardware stochastic rounding to BF16 differs from
    the bit rule it stands for (ep_selftest_stochastic_rounding); 0 expected."""
    out = _U64(0)
    check(lib().ep_selftest_stochastic_rounding(int(device), int(n), int(seed), ctypes.byref(out)), None,
          "ep_selftest_stochastic_rounding")
    return int(out.value)


def _knn_check(rc, what):
    if rc != EP_OK:
        msg = lib().ep_knn_last_error().decode(errors="replace")
        raise NativeError(rc, f"{what}: {msg}")


def embed_features(fptr, fids, table, weights=None, device=0):
    """GPU NodeEmbedder: weighted mean of each node's feature rows
    (``ep_embed_features``)."""
    fptr = np.ascontiguousarray(fptr, np.uint64)
    fids = np.ascontiguousarray(fids, np.uint32)
    table = np.ascontiguousarray(table, np.float32)
    w = None if weights is None else np.ascontiguousarray(weights, np.float32)
    n = len(fptr) - 1
    if table.ndim != 2 or (n and int(fptr[-1]) != len(fids)) or (w is not None and len(w) != table.shape[0]):
        raise ValueError("fptr / fids / table / weights shapes disagree")
    out = np.zeros((n, table.shape[1]), np.float32)
    _knn_check(lib().ep_embed_features(int(device), n, ptr(fptr), ptr(fids), ptr(w), table.shape[0], table.shape[1],
                                       ptr(table), ptr(out)), "ep_embed_features")
    return out


def align(row_ptr, cols, w_cdf, emb, alpha=None, max_neighbors=None, device=0):
    """GPU NeighborhoodAligner (``ep_align``): each node blended with the
    probability-weighted sum of its first max_neighbors neighbours' rows;
    alpha None = adaptive."""
    rp = np.ascontiguousarray(row_ptr, np.uint64)
    c = np.ascontiguousarray(cols, np.uint32)
    w = np.ascontiguousarray(w_cdf, np.float32)
    e = np.ascontiguousarray(emb, np.float32)
    n = len(rp) - 1
    if e.ndim != 2 or e.shape[0] != n:
        raise ValueError(f"emb must hold one row per node: shape {e.shape} for {n} nodes")
    if len(w) != len(c) or (n and int(rp[-1]) != len(c)):
        raise ValueError("row_ptr, cols and w_cdf disagree on the edge count")
    out = np.zeros((n, e.shape[1]), np.float32)
    _knn_check(lib().ep_align(int(device), n, ptr(rp), ptr(c), ptr(w), e.shape[1], ptr(e),
                              -1.0 if alpha is None else float(alpha), int(max_neighbors or 0), ptr(out)), "ep_align")
    return out


def knn_cosine(db, queries, k, q_self=None, device=0):
    """Exact cosine top-k on the tensor cores (``ep_knn_cosine``):
    (ids[n_q, k], similarities[n_q, k]) in decreasing similarity."""
    db = np.ascontiguousarray(db, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    if db.ndim != 2 or q.ndim != 2 or db.shape[1] != q.shape[1]:
        raise ValueError(f"db {db.shape} and queries {q.shape} must be 2-D with the same width")
    qs = None if q_self is None else np.ascontiguousarray(q_self, np.uint64)
    if qs is not None and qs.shape != (len(q),):
        raise ValueError("q_self must hold one entry per query")
    idx = np.zeros((len(q), k), np.uint32)
    sim = np.zeros((len(q), k), np.float32)
    _knn_check(lib().ep_knn_cosine(int(device), len(db), db.shape[1], ptr(db), len(q), ptr(q), ptr(qs), int(k),
                                   ptr(idx), ptr(sim)), "ep_knn_cosine")
    return idx, sim
