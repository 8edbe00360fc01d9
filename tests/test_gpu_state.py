"""Device-side schedule, initialisation and validation, against the oracle.

* learning rate: the cos-decay schedule with warm-up (LRScheduler::CosDecay,
  src/algos/grad_utils/scheduler.rs:120-137, built at
  src/algos/ep/mod.rs:133-137) that each batch computes on the device;
* table initialisation: rows U(-1, 1)^d, L2-normalised
  (src/algos/ep/mod.rs:100-110, 381-392);
* the validation loss: the mean over the validation ids of the forward loss
  with the validation pass's samples (src/algos/ep/mod.rs:267-283);
* the FUSED form's BF16 rounding of updated table rows: the hardware
  stochastic-rounding conversion equals the bit rule it stands for.
"""
import math

import numpy as np
import pytest
from scipy import stats

from cloverleaf_gb300 import _native, datagen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sbm10k():
    return datagen.workload("sbm10k")


def make_ctx(w, form, passes=5, valid_pct=0.0, table=None):
    ep = w["ep"]
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = ep["dims"], ep["negatives"], _native.LOSS_STARSPACE, ep["gamma"]
    cfg.batch_size, cfg.alpha, cfg.passes, cfg.valid_pct = ep["batch_size"], ep["alpha"], passes, valid_pct
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.form = form
    ctx = _native.Context(cfg)
    ctx.upload_graph(w["rows"], w["cols"], w["weights"])
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    ctx.set_table(table)
    return ctx


@pytest.mark.parametrize("form", [_native.FORM_PLAIN_FP32, _native.FORM_FUSED_BF16])
def test_learning_rate_follows_cos_decay(oracle, sbm10k, form):
    w = sbm10k
    ep = w["ep"]
    passes = 5
    ctx = make_ctx(w, form, passes=passes)
    n = len(w["rows"]) - 1
    steps_per_pass = math.ceil(n / ep["batch_size"])
    total = int(np.float32(math.ceil(np.float32(n) / np.float32(ep["batch_size"])))) * passes   # mod.rs:125
    warmup = int(np.float32(total) / np.float32(5.0))                                           # mod.rs:134
    done = 0
    # ends inside the warm-up, at its last step, inside the decay, and at the end
    for upto in (7, warmup, warmup + 1, 3 * steps_per_pass + 5, total):
        st = ctx.train_batches(upto - done)
        done = upto
        want = oracle.lr_cos_decay(ep["alpha"] / 100.0, ep["alpha"], warmup, total, done)
        assert st["lr_last"] == pytest.approx(want, rel=2e-6, abs=1e-9), (done, st["lr_last"], want)


@pytest.mark.parametrize("form", [_native.FORM_PLAIN_FP32, _native.FORM_FUSED_BF16])
def test_initial_table_rows_are_unit_and_uniform(sbm10k, form):
    w = sbm10k
    ctx = make_ctx(w, form)
    t = ctx.get_table(w["n_feat"], w["ep"]["dims"]).astype(np.float64)
    norms = np.linalg.norm(t, axis=1)
    # BF16 rows: each element rounded to 8 significant bits
    tol = 1e-6 if form == _native.FORM_PLAIN_FP32 else 4e-3
    assert np.abs(norms - 1.0).max() < tol
    # components distributed as those of a normalised U(-1, 1)^d vector
    rng = np.random.default_rng(3)
    u = rng.uniform(-1.0, 1.0, (t.shape[0], t.shape[1]))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    x = t[:4000].reshape(-1)
    assert stats.ks_2samp(x, u[:4000].reshape(-1)).pvalue > 1e-4
    # and not as those of a normalised Gaussian vector (the test can tell)
    g = rng.standard_normal(u.shape)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    assert stats.ks_2samp(u[:4000].reshape(-1), g[:4000].reshape(-1)).pvalue < 1e-4
    # rows differ, and the same seed gives the same table
    assert len(np.unique(t, axis=0)) == t.shape[0]
    assert np.array_equal(t, make_ctx(w, form).get_table(w["n_feat"], w["ep"]["dims"]))


@pytest.mark.parametrize("form", [_native.FORM_PLAIN_FP32, _native.FORM_FUSED_BF16])
def test_validation_loss_matches_oracle(oracle, sbm10k, form):
    w = sbm10k
    ep = w["ep"]
    ctx = make_ctx(w, form, passes=1, valid_pct=0.1)
    st = ctx.train(1)[0]
    table = ctx.get_table(w["n_feat"], ep["dims"])      # the table the validation pass read
    train, valid = ctx.split()
    assert len(valid) == int(np.float32(10_000) * np.float32(0.1))
    K, R, B = ep["max_nodes"], ep["negatives"], ep["batch_size"]
    losses = []
    for first in range(0, len(valid), B):
        n = min(B, len(valid) - first)
        anchors, cnt, nbr, nw, neg = ctx.sample_validation(first, n, K)
        assert (anchors == valid[first:first + n]).all()
        assert np.isin(neg, valid).all()                # validation negatives come from the validation ids
        nbr_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint32)
        flat = np.concatenate([nbr[a, :cnt[a]] for a in range(n)])
        flw = np.concatenate([nw[a, :cnt[a]] for a in range(n)])
        cfg = oracle.loss_cfg(loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"])
        l, _, _, _ = oracle.batch(w["fptr"], w["fids"], w["n_feat"], table, w["rows"], anchors, nbr_ptr, flat, flw,
                                  neg, cfg, "f64")
        losses.append(l)
    want = float(np.concatenate(losses).sum() / len(valid))
    assert np.isfinite(st["valid_loss"]) and want > 0
    assert abs(st["valid_loss"] - want) <= 1e-4 * abs(want), (st["valid_loss"], want)


def test_hardware_stochastic_rounding_matches_the_bit_rule():
    # 16M element pairs, every 16th from special values (zeros, infinities,
    # NaNs, subnormals, the largest finite values, BF16 carry boundaries)
    assert _native.selftest_stochastic_rounding(n=1 << 24, seed=7) == 0
    assert _native.selftest_stochastic_rounding(n=1 << 20, seed=12345) == 0


@pytest.mark.parametrize("form,dims", [(_native.FORM_FUSED_BF16, 64), (_native.FORM_PLAIN_FP32, 64),
                                       (_native.FORM_FUSED_BF16, 30)])
def test_table_download_into_page_locked_memory(sbm10k, form, dims):
    # page-locked output memory is written by the device directly; the rows
    # must equal the staged download into ordinary memory bit for bit
    # (dims 30: not a multiple of 4, the staged path in both cases)
    torch = pytest.importorskip("torch")
    w = dict(sbm10k, ep=dict(sbm10k["ep"], dims=dims))
    ctx = make_ctx(w, form, passes=1)
    ctx.train(1)
    n = w["n_feat"]
    ref = ctx.get_table(n, dims)
    pin = torch.empty((n, dims), dtype=torch.float32, pin_memory=True).numpy()
    pin[...] = np.nan
    got = ctx.get_table(n, dims, out=pin)
    ctx.close()
    assert got is pin
    assert np.array_equal(ref.view(np.uint32), pin.view(np.uint32))
