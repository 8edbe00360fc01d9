"""Seeded synthetic EP workloads (native generators of include/ep_datagen.h).

Named workloads restate the five benchmark configurations as generators:

* ``sbm10k``  -- SBM, 10,000 nodes, 32 communities, intra-degree 8, inter-degree
  2; 4-8 tokens per node (80% from the community's 256-token sub-vocabulary,
  20% from a global 8,192-token vocabulary) hashed into 2^16 slots; dims 64,
  max_neighbors 10, 5 negatives, margin 0.5 cosine (starspace), batch 256,
  lr 0.01, 5 passes.
* ``cl1m``    -- bipartite Chung-Lu, 1M nodes, exponent 2.1, mean degree 20,
  weights U[1,5]; 1-16 features Zipf(1.1) over 100k tokens; dims 128,
  max_neighbors 25, 10 negatives, batch 1024, 3 passes.
* ``sbm1k``   -- SBM, 1,000 nodes, 8 communities, mean degree 12; 2-6
  features from a 4,096-slot space; dims 32, batches of 128 anchors, 5
  negatives (differentiation checks).
* ``cl10m``   -- Chung-Lu, 10M nodes, exponent 2.0, degrees clipped to
  [1, 10^4], mean degree 16; Poisson(6) features clipped to [1, 32], Zipf(1.05)
  over 2M slots; dims 256, max_neighbors 25, 10 negatives, batch 8192.
* ``cl50m``   -- Chung-Lu, 50M nodes, ~1B directed edges, exponent 2.1;
  Poisson(8) features clipped to [1, 64], Zipf(1.1) over 5M slots; dims 256,
  max_neighbors 32, 16 negatives, batch 32768, 1 pass.
"""
from __future__ import annotations

import ctypes
import threading
from typing import Dict

import numpy as np

from . import _build

_P, _U32, _U64, _F32, _D = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_double
# include/ep_datagen.h, exported by libep_datagen.so (host code only: loading
# it loads none of the trainer's library)
SIGNATURES = {
    "epg_sbm": (ctypes.c_int, [_U64, _U32, _D, _D, _U64, _P, _P, _P, _P, _P]),
    "epg_sbm_tokens": (ctypes.c_int, [_U64, _P, _U32, _U32, _U32, _U32, _D, _U32, _U64, _P, _P, _P, _P, _P]),
    "epg_chung_lu": (ctypes.c_int, [_U64, _D, _D, _D, ctypes.c_int, _F32, _F32, _U64, _P, _P, _P, _P]),
    "epg_zipf_features": (ctypes.c_int, [_U64, _D, _U32, _U32, _D, _U32, _U64, _P, _P, _P]),
}
_lib = None
_lock = threading.Lock()


def lib():
    """Loads (building first when needed) libep_datagen.so."""
    global _lib
    with _lock:
        if _lib is None:
            handle = ctypes.CDLL(_build.build_datagen())
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


def check(rc: int, _ctx, what: str):
    if rc != 0:
        raise ValueError(f"{what}: invalid argument (status {rc})")


def sbm(n: int, blocks: int, k_in: float, k_out: float, seed: int):
    """Returns (rows, cols, weights, community)."""
    ne = ctypes.c_uint64()
    check(lib().epg_sbm(n, blocks, k_in, k_out, seed, None, None, None, None, ctypes.byref(ne)), None, "epg_sbm")
    rows = np.zeros(n + 1, np.uint64)
    cols = np.zeros(max(ne.value, 1), np.uint32)
    w = np.zeros(max(ne.value, 1), np.float32)
    comm = np.zeros(n, np.uint32)
    check(lib().epg_sbm(n, blocks, k_in, k_out, seed, ptr(rows), ptr(cols), ptr(w), ptr(comm), ctypes.byref(ne)),
          None, "epg_sbm")
    return rows, cols[: ne.value], w[: ne.value], comm


def sbm_tokens(community, tok_min, tok_max, sub_vocab, global_vocab, p_local, slot_bits, seed):
    """Returns (fptr, fids, n_feat, slot_of_feature)."""
    community = np.ascontiguousarray(community, np.uint32)
    n = len(community)
    nf, nfe = ctypes.c_uint64(), ctypes.c_uint32()
    args = (n, ptr(community), tok_min, tok_max, sub_vocab, global_vocab, p_local, slot_bits, seed)
    check(lib().epg_sbm_tokens(*args, None, None, None, ctypes.byref(nf), ctypes.byref(nfe)), None, "epg_sbm_tokens")
    fptr = np.zeros(n + 1, np.uint64)
    fids = np.zeros(max(nf.value, 1), np.uint32)
    slots = np.zeros(max(nfe.value, 1), np.uint32)
    check(lib().epg_sbm_tokens(*args, ptr(fptr), ptr(fids), ptr(slots), ctypes.byref(nf), ctypes.byref(nfe)), None,
          "epg_sbm_tokens")
    return fptr, fids[: nf.value], nfe.value, slots[: nfe.value]


def chung_lu(n, exponent, mean_degree, max_degree, bipartite=False, w_lo=1.0, w_hi=1.0, seed=1):
    """Returns (rows, cols, weights)."""
    ne = ctypes.c_uint64()
    args = (n, exponent, mean_degree, max_degree, int(bipartite), w_lo, w_hi, seed)
    check(lib().epg_chung_lu(*args, None, None, None, ctypes.byref(ne)), None, "epg_chung_lu")
    rows = np.zeros(n + 1, np.uint64)
    cols = np.zeros(max(ne.value, 1), np.uint32)
    w = np.zeros(max(ne.value, 1), np.float32)
    check(lib().epg_chung_lu(*args, ptr(rows), ptr(cols), ptr(w), ctypes.byref(ne)), None, "epg_chung_lu")
    return rows, cols[: ne.value], w[: ne.value]


def zipf_features(n, lam, cmin, cmax, s, n_slots, seed):
    """Returns (fptr, fids)."""
    nf = ctypes.c_uint64()
    check(lib().epg_zipf_features(n, lam, cmin, cmax, s, n_slots, seed, None, None, ctypes.byref(nf)), None,
          "epg_zipf_features")
    fptr = np.zeros(n + 1, np.uint64)
    fids = np.zeros(max(nf.value, 1), np.uint32)
    check(lib().epg_zipf_features(n, lam, cmin, cmax, s, n_slots, seed, ptr(fptr), ptr(fids), ctypes.byref(nf)),
          None, "epg_zipf_features")
    return fptr, fids[: nf.value]


# EP settings per workload (EmbeddingPropagator keyword arguments)
EP_SETTINGS: Dict[str, dict] = {
    "sbm10k": dict(dims=64, max_nodes=10, negatives=5, gamma=0.5, batch_size=256, alpha=0.01, passes=5),
    "cl1m": dict(dims=128, max_nodes=25, negatives=10, gamma=0.5, batch_size=1024, alpha=0.01, passes=3),
    "sbm1k": dict(dims=32, max_nodes=10, negatives=5, gamma=0.5, batch_size=128, alpha=0.01, passes=1),
    "cl10m": dict(dims=256, max_nodes=25, negatives=10, gamma=0.5, batch_size=8192, alpha=0.01, passes=1),
    "cl50m": dict(dims=256, max_nodes=32, negatives=16, gamma=0.5, batch_size=32768, alpha=0.01, passes=1),
}


def workload(name: str, seed: int = 20222022, scale: float = 1.0) -> dict:
    """Generates a named workload.  scale < 1 shrinks the node count of the
    Chung-Lu workloads (same distributions) for quick tests.  Returns a dict
    with rows, cols, weights, fptr, fids, n_feat, optional community, and the
    EP settings under "ep"."""
    out = {"name": name, "ep": dict(EP_SETTINGS[name])}
    if name in ("sbm10k", "sbm1k"):
        if name == "sbm10k":
            n, blocks, k_in, k_out = 10_000, 32, 8.0, 2.0
            tok = dict(tok_min=4, tok_max=8, sub_vocab=256, global_vocab=8192, p_local=0.8, slot_bits=16)
        else:
            n, blocks, k_in, k_out = 1_000, 8, 9.6, 2.4
            tok = dict(tok_min=2, tok_max=6, sub_vocab=256, global_vocab=2048, p_local=0.8, slot_bits=12)
        rows, cols, w, comm = sbm(n, blocks, k_in, k_out, seed)
        fptr, fids, n_feat, slots = sbm_tokens(comm, seed=seed + 1, **tok)
        out.update(rows=rows, cols=cols, weights=w, community=comm, fptr=fptr, fids=fids, n_feat=n_feat)
        return out
    params = {
        "cl1m": dict(n=1_000_000, exponent=2.1, mean_degree=20.0, max_degree=1e9, bipartite=True, w_lo=1.0, w_hi=5.0,
                     feat=(0.0, 1, 16, 1.1, 100_000)),
        "cl10m": dict(n=10_000_000, exponent=2.0, mean_degree=16.0, max_degree=1e4, bipartite=False, w_lo=1.0,
                      w_hi=1.0, feat=(6.0, 1, 32, 1.05, 2_000_000)),
        "cl50m": dict(n=50_000_000, exponent=2.1, mean_degree=20.0, max_degree=1e5, bipartite=False, w_lo=1.0,
                      w_hi=1.0, feat=(8.0, 1, 64, 1.1, 5_000_000)),
    }[name]
    n = max(1000, int(params["n"] * scale))
    rows, cols, w = chung_lu(n, params["exponent"], params["mean_degree"], params["max_degree"], params["bipartite"],
                             params["w_lo"], params["w_hi"], seed)
    lam, cmin, cmax, s, slots = params["feat"]
    slots = max(1000, int(slots * scale)) if scale < 1.0 else slots
    fptr, fids = zipf_features(n, lam, cmin, cmax, s, slots, seed + 1)
    out.update(rows=rows, cols=cols, weights=w, fptr=fptr, fids=fids, n_feat=slots)
    return out
