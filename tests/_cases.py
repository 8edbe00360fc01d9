"""Shared builders for the parity tests: small random graphs, feature CSRs,
tables and explicit sample batches (anchor, sampled neighbours with their
reconstruction weights, negatives)."""
import numpy as np


def random_problem(seed, n=200, n_feat=150, dims=16, deg=(1, 8), feats=(1, 6), scale=1.0):
    rng = np.random.default_rng(seed)
    d = rng.integers(deg[0], deg[1] + 1, n)
    rows = np.zeros(n + 1, np.uint64)
    rows[1:] = np.cumsum(d)
    cols = rng.integers(0, n, int(rows[-1])).astype(np.uint32)
    k = rng.integers(feats[0], feats[1] + 1, n)
    fptr = np.zeros(n + 1, np.uint64)
    fptr[1:] = np.cumsum(k)
    fids = rng.integers(0, n_feat, int(fptr[-1])).astype(np.uint32)
    table = (rng.standard_normal((n_feat, dims)) * scale).astype(np.float32)
    return dict(rows=rows, cols=cols, fptr=fptr, fids=fids, table=table, n=n, n_feat=n_feat, dims=dims)


def sample_batch(seed, prob, B, K, R, weighted=False):
    """Anchors uniform over nodes; min(K, deg) neighbours without replacement
    with weight deg/r (Sample::Fixed, utils.rs:200-203); R negatives."""
    rng = np.random.default_rng(seed)
    rows, cols = prob["rows"], prob["cols"]
    anchors = rng.integers(0, prob["n"], B).astype(np.uint32)
    nbr_ptr, nbr, nbr_w = [0], [], []
    for a in anchors:
        s, e = int(rows[a]), int(rows[a + 1])
        deg = e - s
        r = min(K, deg)
        pick = rng.choice(deg, r, replace=False) if r < deg else np.arange(deg)
        for p in pick:
            nbr.append(int(cols[s + p]))
            nbr_w.append(float(rng.uniform(0.5, 2.0)) if weighted else float(deg) / float(r))
        nbr_ptr.append(len(nbr))
    neg = rng.integers(0, prob["n"], (B, R)).astype(np.uint32)
    if weighted:
        # A negative equal to an anchor's only neighbour gives t and u the same
        # features under different count weights: |t - u| is rounding noise and
        # the gradient direction (t - u)/|t - u| is not reproducible in any
        # precision.  Redraw such negatives.
        for a in range(B):
            if nbr_ptr[a + 1] - nbr_ptr[a] == 1:
                only = nbr[nbr_ptr[a]]
                for i in range(R):
                    while neg[a, i] == only:
                        neg[a, i] = rng.integers(0, prob["n"])
    return dict(anchors=anchors, nbr_ptr=np.array(nbr_ptr, np.uint32), nbr=np.array(nbr, np.uint32),
                nbr_w=np.array(nbr_w, np.float32), neg=neg)


def dense_from_sparse(ids, rows, n_feat, dims):
    g = np.zeros((n_feat, dims), np.float64)
    t = np.zeros(n_feat, bool)
    g[ids] = rows
    t[ids] = True
    return g, t


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.abs(b).max(initial=0.0), 1e-30)
    return float(np.abs(a - b).max(initial=0.0) / den)
