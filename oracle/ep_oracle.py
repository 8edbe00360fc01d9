"""CPU oracle for the Embedding Propagation training path -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline
use this module, and only as the checker.  Nothing in ``cloverleaf_gb300``
imports it.

Two independent restatements of cloverleaf's EP batch live here:

* ``batch()`` wraps the C restatement (``ep_oracle.c``): closed-form
  gradients, FP32 or FP64, first-occurrence extraction
  (``src/algos/ep/mod.rs:361-378``).
* ``batch_autograd()`` rebuilds the reference's expression graph with torch
  FP64 autograd the way ``simple_grad`` builds it: one leaf variable per
  distinct feature per role (``src/algos/ep/model.rs:254-278``), the means of
  ``model.rs:448-463``, the losses of ``src/algos/ep/loss.rs:56-129`` written
  with ``pow(2).sum().pow(0.5)`` (``loss.rs:229-243``), then the reference's
  extraction rule over the leaves' gradients.

Parity status: CSR/CDF construction is pinned by the reference's own tests
(``src/graph.rs:697-787``) and the distance helpers by
``src/algos/ep/loss.rs:250-263``; EP loss/gradient/Adam values are unpinned
(the Rust reference cannot be built here and no reference test asserts them).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libep_oracle.so")
_SOURCES = ("ep_oracle.c", "ep_oracle_batch.inc", "ep_oracle.h", "Makefile")
_lock = threading.Lock()
_lib = None

LOSS_MARGIN, LOSS_STARSPACE, LOSS_CONTRASTIVE, LOSS_RANK, LOSS_RANKSPACE, LOSS_PPR = 0, 1, 2, 3, 4, 5
LW_NONE, LW_LOG, LW_EXP = 0, 1, 2
GRAD_REFERENCE, GRAD_TRUE = 0, 1
SAMPLE_ALL, SAMPLE_FIXED, SAMPLE_PROB = 0, 1, 2


def build() -> str:
    """Compiles the C oracle with its Makefile when missing or stale."""
    newest = max(os.path.getmtime(os.path.join(_HERE, s)) for s in _SOURCES)
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < newest:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class LossCfg(ctypes.Structure):
    _fields_ = [
        ("loss", ctypes.c_int32),
        ("gamma", ctypes.c_float),
        ("neg_margin", ctypes.c_float),
        ("grad_mode", ctypes.c_int32),
        ("loss_weighting", ctypes.c_int32),
        ("lw_exp", ctypes.c_float),
        ("feat_scalar", ctypes.c_float),
    ]


class TrainCfg(ctypes.Structure):
    _fields_ = [
        ("alpha", ctypes.c_float),
        ("loss", LossCfg),
        ("negatives", ctypes.c_uint32),
        ("batch_size", ctypes.c_uint32),
        ("dims", ctypes.c_uint32),
        ("passes", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
        ("max_nodes_kind", ctypes.c_int32),
        ("max_nodes", ctypes.c_float),
        ("max_features_kind", ctypes.c_int32),
        ("max_features", ctypes.c_float),
        ("valid_pct", ctypes.c_float),
        ("threads", ctypes.c_int32),
        ("max_batches", ctypes.c_uint64),
        ("hard_negatives", ctypes.c_uint32),
        ("ppr_restart_p", ctypes.c_float),
    ]


class TrainStats(ctypes.Structure):
    _fields_ = [
        ("seconds", ctypes.c_double),
        ("anchors", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("last_train_loss", ctypes.c_float),
        ("last_valid_loss", ctypes.c_float),
        ("shuffle_seconds", ctypes.c_double),
        ("steps_per_pass", ctypes.c_uint64),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            P = ctypes.c_void_p
            _lib.orc_csr_from_edges.argtypes = [ctypes.c_uint64, P, P, P, ctypes.c_int, P, P, P, P, P]
            _lib.orc_cdf_convert.argtypes = [ctypes.c_uint64, P, P]
            for name in ("orc_batch_f32", "orc_batch_f64"):
                getattr(_lib, name).argtypes = [P, P, ctypes.c_uint32, P, ctypes.c_uint32, P,
                                                ctypes.c_uint32, P, P, P, P, ctypes.c_uint32, P,
                                                ctypes.POINTER(LossCfg), P, P, P, P]
                getattr(_lib, name).restype = ctypes.c_int
            _lib.orc_adam.argtypes = [P, P, P, ctypes.c_uint32, ctypes.c_uint32, P, P,
                                      ctypes.c_float, ctypes.c_uint32]
            _lib.orc_lr_cos_decay.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_uint64,
                                              ctypes.c_uint64, ctypes.c_uint64]
            _lib.orc_lr_cos_decay.restype = ctypes.c_float
            _lib.orc_train.argtypes = [P, P, P, ctypes.c_uint64, P, P, ctypes.c_uint32,
                                       ctypes.POINTER(TrainCfg), P, ctypes.c_int,
                                       ctypes.POINTER(TrainStats)]
        return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def csr_from_edges(edges, dedup=True):
    """graph.rs:70-142.  edges: iterable of (from, to, weight)."""
    e = list(edges)
    n = len(e)
    f = _c([x[0] for x in e], np.uint64)
    t = _c([x[1] for x in e], np.uint64)
    w = _c([x[2] for x in e], np.float32)
    max_node = int(max(f.max(initial=0), t.max(initial=0)))
    rows = np.zeros(max_node + 2, np.uint64)
    cols = np.zeros(max(n, 1), np.uint64)
    wo = np.zeros(max(n, 1), np.float32)
    nn = ctypes.c_uint64()
    ne = ctypes.c_uint64()
    lib().orc_csr_from_edges(n, _p(f), _p(t), _p(w), int(dedup), _p(rows), _p(cols), _p(wo),
                             ctypes.byref(nn), ctypes.byref(ne))
    return rows[: nn.value + 1], cols[: ne.value], wo[: ne.value]


def cdf_convert(rows, weights):
    """graph.rs:414-422 + 664-691, in place on a copy."""
    rows = _c(rows, np.uint64)
    w = _c(weights, np.float32).copy()
    lib().orc_cdf_convert(len(rows) - 1, _p(rows), _p(w))
    return w


def lr_cos_decay(min_alpha, alpha, warmup, max_steps, cur_step):
    return lib().orc_lr_cos_decay(min_alpha, alpha, warmup, max_steps, cur_step)


def loss_cfg(loss=LOSS_STARSPACE, gamma=0.5, neg_margin=0.0, grad_mode=GRAD_REFERENCE,
             loss_weighting=LW_NONE, lw_exp=1.0, feat_scalar=1.0):
    return LossCfg(loss, gamma, neg_margin, grad_mode, loss_weighting, lw_exp, feat_scalar)


def batch(fptr, fids, n_feat, table, graph_rows, anchors, nbr_ptr, nbr, nbr_w, neg, cfg: LossCfg,
          precision="f32"):
    """One EP batch from explicit samples.  Returns (loss[B], status[B],
    grad[n_feat, d], touched[n_feat]) in the requested precision."""
    table = _c(table, np.float32)
    d = table.shape[1]
    fptr = _c(fptr, np.uint64)
    fids = _c(fids, np.uint32)
    graph_rows = _c(graph_rows, np.uint64)
    anchors = _c(anchors, np.uint32)
    nbr_ptr = _c(nbr_ptr, np.uint32)
    nbr = _c(nbr if len(nbr) else [0], np.uint32)
    nbr_w = _c(nbr_w if len(nbr_w) else [0], np.float32)
    B = len(anchors)
    neg = _c(neg, np.uint32).reshape(B, -1) if B else np.zeros((0, 0), np.uint32)
    R = neg.shape[1]
    neg = _c(neg.reshape(-1) if neg.size else [0], np.uint32)
    dt = np.float32 if precision == "f32" else np.float64
    loss = np.zeros(B, dt)
    status = np.zeros(B, np.int32)
    grad = np.zeros((n_feat, d), dt)
    touched = np.zeros(n_feat, np.uint8)
    fn = lib().orc_batch_f32 if precision == "f32" else lib().orc_batch_f64
    rc = fn(_p(fptr), _p(fids), n_feat, _p(table), d, _p(graph_rows), B, _p(anchors), _p(nbr_ptr),
            _p(nbr), _p(nbr_w), R, _p(neg), ctypes.byref(cfg), _p(loss), _p(status), _p(grad),
            _p(touched))
    if rc < 0:
        raise ValueError("oracle batch rejected its inputs")
    return loss, status, grad, touched.astype(bool)


def adam(table, m, v, grad, touched, lr, pass_idx):
    """optimizer.rs:43-81 on copies; returns (table, m, v)."""
    table = _c(table, np.float32).copy()
    m = _c(m, np.float32).copy()
    v = _c(v, np.float32).copy()
    grad = _c(grad, np.float32)
    touched = _c(touched, np.uint8)
    n, d = table.shape
    lib().orc_adam(_p(table), _p(m), _p(v), d, n, _p(grad), _p(touched), lr, pass_idx)
    return table, m, v


def train(rows, cols, wcdf, fptr, fids, n_feat, *, dims, alpha, loss=LOSS_STARSPACE, gamma=0.5,
          neg_margin=0.0, negatives=5, batch_size=256, passes=5, seed=20222022,
          max_nodes=(SAMPLE_ALL, 0.0), max_features=(SAMPLE_ALL, 0.0), valid_pct=0.0,
          loss_weighting=LW_NONE, lw_exp=1.0, threads=0, max_batches=0, init_table=None, hard_negatives=0,
          ppr_restart_p=0.5):
    """The whole reference training loop (mod.rs:92-287) on host cores.
    Returns (table[n_feat, dims], TrainStats)."""
    rows = _c(rows, np.uint64)
    cols = _c(cols, np.uint32)
    wcdf = _c(wcdf, np.float32)
    fptr = _c(fptr, np.uint64)
    fids = _c(fids, np.uint32)
    cfg = TrainCfg()
    cfg.alpha = alpha
    cfg.loss = loss_cfg(loss, gamma, neg_margin, GRAD_REFERENCE, loss_weighting, lw_exp, 0.0)
    cfg.negatives = negatives
    cfg.batch_size = batch_size
    cfg.dims = dims
    cfg.passes = passes
    cfg.seed = seed
    cfg.max_nodes_kind, cfg.max_nodes = max_nodes
    cfg.max_features_kind, cfg.max_features = max_features
    cfg.valid_pct = valid_pct
    cfg.threads = threads
    cfg.max_batches = max_batches
    cfg.hard_negatives = hard_negatives
    cfg.ppr_restart_p = ppr_restart_p
    if init_table is not None:
        table = _c(init_table, np.float32).copy()
        given = 1
    else:
        table = np.zeros((n_feat, dims), np.float32)
        given = 0
    st = TrainStats()
    rc = lib().orc_train(_p(rows), _p(cols), _p(wcdf), len(rows) - 1, _p(fptr), _p(fids), n_feat,
                         ctypes.byref(cfg), _p(table), given, ctypes.byref(st))
    if rc != 0:
        raise ValueError("oracle train rejected its config")
    return table, st


# ---------------------------------------------------------------------------
# Autograd restatement (torch FP64), mirroring simple_grad's expression graph
# ---------------------------------------------------------------------------
def batch_autograd(fptr, fids, n_feat, table, graph_rows, anchors, nbr_ptr, nbr, nbr_w, neg,
                   loss=LOSS_STARSPACE, gamma=0.5, neg_margin=0.0, grad_mode=GRAD_REFERENCE,
                   loss_weighting=LW_NONE, lw_exp=1.0, feat_scalar=1.0, dtype=None):
    """Returns (loss[B], status[B], grad[n_feat, d], touched[n_feat]) computed
    with torch autograd in FP64 (default) for small cases."""
    import torch

    dtype = dtype or torch.float64
    # the reference holds its loss parameters as f32 (loss.rs:15-38)
    gamma, neg_margin, lw_exp = (float(np.float32(x)) for x in (gamma, neg_margin, lw_exp))
    table = np.asarray(table, np.float32)
    d = table.shape[1]
    B = len(anchors)
    neg = np.asarray(neg).reshape(B, -1) if B else np.zeros((0, 0), np.int64)
    R = neg.shape[1] if B else 0
    grad = np.zeros((n_feat, d), np.float64)
    touched = np.zeros(n_feat, bool)
    losses = np.zeros(B, np.float64)
    status = np.zeros(B, np.int32)

    def feats(v):
        return [int(x) for x in fids[int(fptr[v]):int(fptr[v + 1])]]

    def role(nodes_weights):
        # NodeCounts: feature -> (leaf Variable, count), first-seen order
        # counts accumulate in f32 like the reference's (model.rs:268-271)
        m = {}
        for v, w in nodes_weights:
            wc = np.float32(np.float32(w) + np.float32(feat_scalar))
            for f in feats(v):
                if f in m:
                    m[f][1] = np.float32(m[f][1] + wc)
                else:
                    leaf = torch.tensor(table[f], dtype=dtype, requires_grad=True)
                    m[f] = [leaf, wc]
        return {f: [leaf, float(c)] for f, (leaf, c) in m.items()}

    def mean(m):
        vs = []
        n = 0.0
        for leaf, c in m.values():
            vs.append(leaf if abs(c - 1.0) < 1e-6 else leaf * c)
            n += c
        return torch.stack(vs).sum(0) / n

    def l2(x):
        return x.pow(2).sum().pow(0.5)

    for a in range(B):
        v = int(anchors[a])
        maps = [role([(v, 1.0)]),
                role([(int(nbr[j]), float(nbr_w[j])) for j in range(int(nbr_ptr[a]), int(nbr_ptr[a + 1]))])]
        maps += [role([(int(neg[a, i]), 1.0)]) for i in range(R)]
        hv, thv = mean(maps[0]), mean(maps[1])
        hus = [mean(m) for m in maps[2:]]
        if loss in (LOSS_MARGIN, LOSS_PPR):
            d1 = gamma + l2(thv - hv)
            terms = [d1 - l2(thv - hu) for hu in hus]
            terms = [t for t in terms if t.item() > 0]
        elif loss in (LOSS_STARSPACE, LOSS_RANKSPACE):
            tn, hn = thv / l2(thv), hv / l2(hv)
            rd = tn.dot(hn)
            terms = [torch.clamp(gamma - (rd - hn.dot(hu / l2(hu))), min=0.0) for hu in hus]
            terms = [t for t in terms if t.item() > 0]
        elif loss == LOSS_RANK:
            terms = []
        else:
            tn, hn = thv / l2(thv), hv / l2(hv)
            pos = torch.clamp(gamma - tn.dot(hn), min=0.0)
            terms = [torch.clamp(hn.dot(hu / l2(hu)) - neg_margin, min=0.0) for hu in hus]
            terms = [t for t in terms if t.item() > 0]
            if pos.item() > 0:
                terms.append(pos)
        L = torch.stack(terms).sum() / len(terms) if terms else torch.zeros((), dtype=dtype)
        if loss in (LOSS_RANK, LOSS_RANKSPACE):
            # RankLoss (loss.rs:130-155) with the exact softmax; the max is a
            # constant outside the graph, as in attention.rs:283-296
            ds = torch.stack([hu.dot(hv) for hu in hus] + [hv.dot(thv)])
            n = torch.exp(ds - ds.max().detach())
            pr = (n / n.sum())[-1]
            if pr.item() < gamma:
                L = L - torch.log(pr)
        if loss_weighting != LW_NONE:
            deg = float(graph_rows[v + 1] - graph_rows[v])
            L = L / (np.log(1.0 + deg) if loss_weighting == LW_LOG else deg ** lw_exp)
        lv = float(L.item())
        losses[a] = lv
        if lv != lv:
            status[a] = 2
            continue
        if not lv > 0:
            status[a] = 1
            continue
        L.backward()
        seen = set()
        for m in maps:
            for f, (leaf, _c0) in m.items():
                g = leaf.grad
                if g is None:
                    continue
                g = g.detach().cpu().numpy()
                if grad_mode == GRAD_REFERENCE and f in seen:
                    continue
                if not np.all(np.isfinite(g)):
                    continue
                if grad_mode == GRAD_REFERENCE:
                    seen.add(f)
                grad[f] += g
                touched[f] = True
    return losses, status, grad, touched


# ---------------------------------------------------------------------------
# Neighbourhood alignment (src/algos/alignment.rs:25-75), f32 as the reference
# ---------------------------------------------------------------------------
def align(rows, cols, wcdf, emb, alpha=None, max_neighbors=None):
    """out[v] = (1 - a) * sum_j p_j emb[cols[j]] + a * emb[v] over the first
    max_neighbors edges of v in CSR order; p_j = w_0, w_j - w_{j-1} from the
    CDF weights; a = alpha or min(1, 1 / ln(deg + 1)).  Every product is
    rounded to f32 before it is added, element by element in edge order.  A
    node without edges gets a * emb[v] (the reference indexes the empty
    weight list there)."""
    rows = np.asarray(rows, np.uint64)
    cols = np.asarray(cols, np.int64)
    wcdf = np.asarray(wcdf, np.float32)
    emb = np.asarray(emb, np.float32)
    n, d = emb.shape
    out = np.zeros_like(emb)
    one = np.float32(1)
    for v in range(len(rows) - 1):
        s, e = int(rows[v]), int(rows[v + 1])
        deg = e - s
        m = deg if max_neighbors is None else min(deg, int(max_neighbors))
        acc = np.zeros(d, np.float32)
        for j in range(m):
            p = wcdf[s] if j == 0 else np.float32(wcdf[s + j] - wcdf[s + j - 1])
            acc = acc + p * emb[cols[s + j]]
        if alpha is None:
            with np.errstate(divide="ignore"):
                a = np.float32(min(np.float32(one / np.log(np.float32(deg) + one)), one))
        else:
            a = np.float32(alpha)
        out[v] = acc * (one - a) + emb[v] * a
    return out
