"""Parity of the CUDA path with the oracle, through the C ABI.

Per-batch checks use explicit samples (the reference's trajectory is
nondeterministic, so parity is per batch from a frozen table).  Tolerances:
FP32 loss and gradient within 1e-4 relative (max |diff| / max |oracle|) of
the FP64 oracle.  The BF16 form is compared on the BF16-rounded table: its
loss (FP32 arithmetic) within the same 1e-4; its gradient within 1e-2,
because that form stores each role's gradient direction in BF16 (relative
rounding 2^-9 per element) before the FP32 per-feature sums.
"""
import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import dense_from_sparse, random_problem, rel_err, sample_batch

pytestmark = pytest.mark.gpu

TOL = 1e-4
TOL_GRAD_BF16 = 1e-2


def make_ctx(prob, *, loss=1, gamma=0.5, R=4, form=0, grad_mode=0, weighting=0, lw_exp=0.5, neg_margin=0.1,
             dims=None, table=None):
    cfg = _native.default_config()
    cfg.dims = dims or prob["dims"]
    cfg.loss, cfg.gamma, cfg.neg_margin, cfg.negatives = loss, gamma, neg_margin, R
    cfg.form, cfg.grad_mode = form, grad_mode
    cfg.loss_weighting, cfg.loss_weighting_exp = weighting, lw_exp
    cfg.batch_size = 64
    cfg.passes = 1
    cfg.valid_pct = 0.0
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    ctx.set_table(prob["table"] if table is None else table)
    return ctx


def oracle_batch(oracle, prob, smp, table, *, loss=1, gamma=0.5, grad_mode=0, weighting=0, lw_exp=0.5,
                 neg_margin=0.1):
    cfg = oracle.loss_cfg(loss=loss, gamma=gamma, neg_margin=neg_margin, grad_mode=grad_mode,
                          loss_weighting=weighting, lw_exp=lw_exp)
    return oracle.batch(prob["fptr"], prob["fids"], prob["n_feat"], table, prob["rows"], smp["anchors"],
                        smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"], cfg, "f64")


def gpu_batch(ctx, prob, smp, dims=None):
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    return ctx.batch_grad(s, prob["n_feat"], dims or prob["dims"])


def check_parity(oracle, prob, smp, ctx, table, grad_tol=TOL, **kw):
    ol, ost, og, ot = oracle_batch(oracle, prob, smp, table, **kw)
    gl, gst, ids, rows = gpu_batch(ctx, prob, smp)
    assert (gst == ost).all(), (gst, ost)
    kept = ost == 0
    assert rel_err(gl[kept], ol[kept]) < TOL
    g, t = dense_from_sparse(ids, rows, prob["n_feat"], prob["dims"])
    assert (t == ot).all(), np.nonzero(t != ot)
    assert np.isfinite(rows).all()
    assert rel_err(g, og) < grad_tol, rel_err(g, og)
    return ids, rows


@pytest.mark.parametrize("dims", [16, 64, 100, 256])
@pytest.mark.parametrize("loss", [0, 1, 2])
def test_batch_grad_plain_fp32(oracle, loss, dims):
    prob = random_problem(100 + dims, n=300, n_feat=200, dims=dims)
    smp = sample_batch(5 + loss, prob, B=96, K=5, R=4)
    gamma = 1.0 if loss == 0 else 0.5
    ctx = make_ctx(prob, loss=loss, gamma=gamma)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=loss, gamma=gamma)


def zipf_problem(seed):
    """Zipf(1.1) feature ids over 2,000 slots: many features whose items span
    several reducer chunks, ending at every offset within a chunk."""
    prob = random_problem(seed, n=3000, n_feat=2000, dims=16, deg=(1, 12), feats=(1, 16))
    rng = np.random.default_rng(seed + 1)
    p = 1.0 / np.arange(1, prob["n_feat"] + 1) ** 1.1
    prob["fids"] = rng.choice(prob["n_feat"], len(prob["fids"]), p=p / p.sum()).astype(np.uint32)
    return prob


@pytest.mark.parametrize("chunk", ["32", "64", "128"])
@pytest.mark.parametrize("form", [0, 1])
def test_batch_grad_multi_chunk_spans(oracle, monkeypatch, chunk, form):
    # the fix-ups locate the last chunk of each feature spanning three or more
    # chunks by a 32-ary search; every such feature's last partial sum must
    # be included (about ten features per case here end where a search
    # that clipped its bound after 32 inside probes would stop one chunk early)
    monkeypatch.setenv("EP_REDUCE_CHUNK", chunk)
    prob = zipf_problem(3)
    smp = sample_batch(3, prob, B=1024, K=10, R=5)
    ctx = make_ctx(prob, loss=1, gamma=0.5, R=5, form=form)
    table = ctx.get_table(prob["n_feat"], prob["dims"]) if form else prob["table"]   # BF16-rounded when fused
    check_parity(oracle, prob, smp, ctx, table, grad_tol=TOL if form == 0 else TOL_GRAD_BF16, loss=1, gamma=0.5)


@pytest.mark.parametrize("name", ["margin", "starspace", "contrastive"])
@pytest.mark.parametrize("form", [0, 1])
def test_default_losses_known_answers(name, form):
    # the hand-derived Margin, StarSpace and Contrastive answers of
    # tests/test_oracle.py, straight through the C ABI (the tables are exact
    # in BF16)
    from tests.test_oracle import KATS

    k, lid = KATS[name]
    n = len(k["fptr"]) - 1
    prob = dict(rows=np.arange(n + 1, dtype=np.uint64), cols=((np.arange(n) + 1) % n).astype(np.uint32),
                fptr=np.array(k["fptr"], np.uint64), fids=np.array(k["fids"], np.uint32),
                table=np.array(k["table"], np.float32), n=n, n_feat=len(k["table"]), dims=2)
    smp = dict(anchors=np.array([0], np.uint32), nbr_ptr=np.array(k["nbr_ptr"], np.uint32),
               nbr=np.array(k["nbr"], np.uint32), nbr_w=np.array(k["nbr_w"], np.float32),
               neg=np.array(k["neg"], np.uint32))
    R = smp["neg"].shape[1]
    ctx = make_ctx(prob, loss=lid, gamma=k["gamma"], neg_margin=k.get("neg_margin", 0.1), R=R, form=form)
    gl, gst, ids, rows = gpu_batch(ctx, prob, smp)
    assert gst.tolist() == [0]
    assert abs(gl[0] - k["loss"]) < 1e-6
    assert sorted(ids.tolist()) == sorted(k["grad"])
    tol = 1e-6 if form == 0 else TOL_GRAD_BF16       # fused form: BF16 directions
    for f, row in zip(ids.tolist(), rows):
        np.testing.assert_allclose(row, k["grad"][f], atol=tol, rtol=0)


@pytest.mark.parametrize("grad_mode", [0, 1])
@pytest.mark.parametrize("weighting", [0, 1, 2])
def test_batch_grad_modes_and_weighting(oracle, grad_mode, weighting):
    prob = random_problem(31, n=150, n_feat=60, dims=32, feats=(1, 8))   # many shared features
    smp = sample_batch(41, prob, B=128, K=6, R=5, weighted=True)
    ctx = make_ctx(prob, loss=0, gamma=1.0, R=5, grad_mode=grad_mode, weighting=weighting)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=0, gamma=1.0, grad_mode=grad_mode,
                 weighting=weighting)


def test_batch_grad_hot_feature_spans_chunks(oracle):
    # one feature on every node: its items span many reducer chunks, which
    # exercises the carry/fix-up path and the look-back for the first role
    prob = random_problem(5, n=400, n_feat=40, dims=32, feats=(2, 6))
    fptr, fids = prob["fptr"].copy(), prob["fids"].copy()
    fids[fptr[:-1].astype(np.int64)] = 0
    prob.update(fids=fids)
    smp = sample_batch(6, prob, B=256, K=8, R=6)
    for grad_mode in (0, 1):
        ctx = make_ctx(prob, loss=1, gamma=0.5, R=6, grad_mode=grad_mode)
        check_parity(oracle, prob, smp, ctx, prob["table"], loss=1, gamma=0.5, grad_mode=grad_mode)


def test_nan_and_empty_roles(oracle):
    # t == h for some anchors (anchor and neighbour share their only
    # feature), empty neighbour lists, a negative equal to the reconstruction
    prob = random_problem(9, n=50, n_feat=30, dims=8, feats=(1, 1))
    smp = sample_batch(10, prob, B=40, K=1, R=3)
    # unit neighbour weights: every role then counts its single feature 2x, so
    # equal feature sets give bit-identical means (an exact zero distance,
    # NaN direction, dropped), not means that differ by rounding
    smp["nbr_w"] = np.ones_like(smp["nbr_w"])
    fids = prob["fids"].copy()
    for a in range(0, 40, 3):
        j = smp["nbr_ptr"][a]
        if smp["nbr_ptr"][a + 1] > j:
            fids[int(prob["fptr"][smp["nbr"][j]])] = fids[int(prob["fptr"][smp["anchors"][a]])]
    prob.update(fids=fids)
    # an anchor without neighbours: ~h(v) is NaN, every margin term is
    # filtered, so the loss is the constant 0 and the anchor is skipped
    # (loss.rs:60-72, mod.rs:209-213): status 1
    smp["nbr_ptr"] = smp["nbr_ptr"].copy()
    cut = int(smp["nbr_ptr"][1] - smp["nbr_ptr"][0])
    smp["nbr"] = smp["nbr"][cut:]
    smp["nbr_w"] = smp["nbr_w"][cut:]
    smp["nbr_ptr"] = np.concatenate([[0], smp["nbr_ptr"][1:] - cut]).astype(np.uint32)
    ctx = make_ctx(prob, loss=0, gamma=1.0, R=3)
    ol, ost, og, ot = oracle_batch(oracle, prob, smp, prob["table"], loss=0, gamma=1.0)
    assert ost[0] == 1
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=0, gamma=1.0)


def test_batch_grad_fused_bf16(oracle):
    prob = random_problem(77, n=300, n_feat=200, dims=128)
    smp = sample_batch(78, prob, B=128, K=5, R=4)
    ctx = make_ctx(prob, loss=1, gamma=0.5, form=1)
    table_bf16 = ctx.get_table(prob["n_feat"], prob["dims"])     # BF16-rounded values
    assert not np.array_equal(table_bf16, prob["table"])
    check_parity(oracle, prob, smp, ctx, table_bf16, grad_tol=TOL_GRAD_BF16, loss=1, gamma=0.5)


def test_batch_grad_deterministic(oracle):
    prob = random_problem(3, n=400, n_feat=100, dims=64)
    smp = sample_batch(4, prob, B=256, K=10, R=5)
    ctx = make_ctx(prob, loss=1, gamma=0.5, R=5)
    a = gpu_batch(ctx, prob, smp)
    b = gpu_batch(ctx, prob, smp)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_batch_step_adam_plain(oracle):
    prob = random_problem(12, n=200, n_feat=120, dims=32)
    smp = sample_batch(13, prob, B=64, K=5, R=4)
    ctx = make_ctx(prob, loss=1, gamma=0.5)
    lr, pass_idx = 0.05, 1
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    ctx.batch_step(s, lr, pass_idx)
    got = ctx.get_table(prob["n_feat"], prob["dims"])
    _, _, og, ot = oracle_batch(oracle, prob, smp, prob["table"], loss=1, gamma=0.5)
    z = np.zeros_like(prob["table"])
    exp, _, _ = oracle.adam(prob["table"], z, z, og.astype(np.float32), ot.astype(np.uint8), lr, pass_idx)
    # Adam maps a tiny gradient to an update of about +-lr (m/sqrt(v) ~ sign(g)),
    # so entries whose gradient is at rounding level may differ by up to 2*lr
    big = np.abs(og) > 1e-3 * np.abs(og).max()
    diff = np.abs(got - exp)
    assert diff[big].max() < 1e-5 + 1e-4 * np.abs(exp[big]).max()
    assert diff.max() <= 2 * lr + 1e-5
    assert np.array_equal(got[~ot], prob["table"][~ot])     # untouched rows unchanged


def test_bad_inputs_fail_cleanly():
    prob = random_problem(1, n=20, n_feat=10, dims=8)
    ctx = make_ctx(prob)
    smp = sample_batch(2, prob, B=4, K=2, R=4)
    smp["anchors"] = smp["anchors"].copy()
    smp["anchors"][0] = 10_000
    with pytest.raises(_native.NativeError) as e:
        gpu_batch(ctx, prob, smp)
    assert e.value.code == -1
    bad = dict(prob)
    bad["cols"] = prob["cols"].copy()
    bad["cols"][0] = 999
    cfg = _native.default_config()
    cfg.dims = 8
    c2 = _native.Context(cfg)
    with pytest.raises(_native.NativeError) as e:
        c2.upload_graph(bad["rows"], bad["cols"], None)
    assert "out of range" in str(e.value)
    rows = prob["rows"].copy()
    rows[6] = rows[5] - 1              # every row has an edge, so rows[5] >= 5
    with pytest.raises(_native.NativeError) as e:
        c2.upload_graph(rows, prob["cols"], None)
    assert "decrease at row 5" in str(e.value)
    fids = prob["fids"].copy()
    fids[-1] = prob["n_feat"]
    with pytest.raises(_native.NativeError) as e:
        c2.upload_features(prob["fptr"], fids, prob["n_feat"])
    assert "out of range" in str(e.value)
    with pytest.raises(_native.NativeError):
        c2.train(1)         # nothing valid uploaded
    # a context recovers from a rejected upload
    c2.upload_graph(prob["rows"], prob["cols"], None)
    c2.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    c2.set_table(prob["table"])
    assert c2.train(1)[0]["anchors"] > 0


@pytest.mark.parametrize("n_feat", [600_000, (1 << 21) + 7])
def test_batch_grad_wide_feature_ids(oracle, n_feat):
    # 20- and 22-bit feature ids: three digit passes of the radix sort, the
    # last one partial; a few hot features share many items
    prob = random_problem(77, n=400, n_feat=n_feat, dims=8)
    rng = np.random.default_rng(78)
    hot = rng.random(len(prob["fids"])) < 0.5
    prob["fids"][hot] = rng.integers(n_feat - 40, n_feat, int(hot.sum())).astype(np.uint32)
    smp = sample_batch(79, prob, B=128, K=6, R=5)
    ctx = make_ctx(prob, loss=1, gamma=0.5, R=5)
    ids, _ = check_parity(oracle, prob, smp, ctx, prob["table"], loss=1, gamma=0.5)
    assert ids.max() >= n_feat - 40 and ids.min() < n_feat // 2


@pytest.mark.parametrize("chunk", ["32", "48", "128"])
@pytest.mark.parametrize("grad_mode", [0, 1])
def test_batch_grad_chunk_boundaries(oracle, monkeypatch, chunk, grad_mode):
    # features of at most one chunk of items are reduced whole by the warp of
    # the chunk they start in; longer ones are split into partial sums that
    # the fix-up kernels add: small chunks make both kinds common
    monkeypatch.setenv("EP_REDUCE_CHUNK", chunk)
    prob = random_problem(91, n=400, n_feat=3000, dims=64)
    rng = np.random.default_rng(92)
    hot = rng.random(len(prob["fids"])) < 0.4
    prob["fids"][hot] = rng.integers(0, 12, int(hot.sum())).astype(np.uint32)
    smp = sample_batch(93, prob, B=128, K=6, R=5)
    ctx = make_ctx(prob, loss=1, gamma=0.5, R=5, grad_mode=grad_mode)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=1, gamma=0.5, grad_mode=grad_mode)


@pytest.mark.parametrize("R", [5, 40])
def test_batch_grad_anchors_past_the_staging_tables(oracle, R):
    # anchors whose roles hold more than 512 feature occurrences (or more
    # than 32 negatives) skip the staged gather's shared-memory tables and
    # take the direct path
    prob = random_problem(95, n=300, n_feat=4000, dims=32, deg=(4, 14), feats=(20, 60))
    smp = sample_batch(96, prob, B=64, K=10, R=R)
    occ = np.diff(prob["fptr"]).astype(np.int64)
    per_anchor = [occ[a] + sum(occ[smp["nbr"][int(smp["nbr_ptr"][i]):int(smp["nbr_ptr"][i + 1])]]) + occ[smp["neg"][i]].sum()
                  for i, a in enumerate(smp["anchors"])]
    assert max(per_anchor) > 512 and min(per_anchor) <= 512 or R > 32
    ctx = make_ctx(prob, loss=1, gamma=0.5, R=R)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=1, gamma=0.5)
