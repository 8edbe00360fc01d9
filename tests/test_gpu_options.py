"""Reference options off the default path, on the GPU: gradient noise
(src/algos/ep/mod.rs:140-146, 239-247)."""
import math

import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import random_problem, sample_batch

pytestmark = pytest.mark.gpu


def _ctx(prob, form=_native.FORM_PLAIN_FP32, noise=0.0, passes=1, batch_size=64):
    cfg = _native.default_config()
    cfg.dims, cfg.loss, cfg.gamma, cfg.negatives = prob["dims"], _native.LOSS_STARSPACE, 0.5, 4
    cfg.form, cfg.noise, cfg.passes, cfg.batch_size, cfg.valid_pct = form, noise, passes, batch_size, 0.0
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    ctx.set_table(prob["table"])
    return ctx


def test_noise_schedule_matches_reference():
    # sigma(step) = noise * decay^step, decay = exp((ln 1e-9 - ln noise) / total_updates)
    prob = random_problem(3, n=1000, n_feat=300, dims=32)
    noise, passes, B = 0.05, 3, 64
    ctx = _ctx(prob, noise=noise, passes=passes, batch_size=B)
    stats = ctx.train(passes)
    steps = -(-1000 // B)
    total = steps * passes
    decay = math.exp((math.log(1e-9) - math.log(noise)) / total)
    for p, s in enumerate(stats, start=1):
        want = noise * decay ** (p * steps)     # the last step of pass p
        assert s["noise_last"] == pytest.approx(want, rel=1e-4), (p, s["noise_last"], want)
    off = _ctx(prob).train(1)
    assert off[0]["noise_last"] == 0.0


def test_noise_is_applied_to_the_update():
    # First Adam step from zero moments moves each touched element by about
    # lr * 0.74 * sign(g + sigma * z): with sigma far above |g| about half of
    # the signs disagree with the noiseless step; with sigma = 0 none do.
    prob = random_problem(12, n=200, n_feat=120, dims=32)
    smp = sample_batch(13, prob, B=64, K=5, R=4)
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    lr, t0 = 0.05, prob["table"]
    clean = _ctx(prob)
    clean.batch_step(s, lr, 1)
    d_clean = clean.get_table(prob["n_feat"], prob["dims"]) - t0
    noisy = _ctx(prob, noise=1e3)
    noisy.batch_step(s, lr, 1)
    t_noisy = noisy.get_table(prob["n_feat"], prob["dims"])
    d_noisy = t_noisy - t0
    touched = np.abs(d_clean) > 0.5 * lr * 0.74
    assert touched.sum() > 500
    flips = np.mean(np.sign(d_noisy[touched]) != np.sign(d_clean[touched]))
    assert 0.4 < flips < 0.6, flips
    assert np.array_equal(d_noisy[~touched.any(axis=1)], d_clean[~touched.any(axis=1)])
    again = _ctx(prob, noise=1e3)
    again.batch_step(s, lr, 1)
    assert np.array_equal(again.get_table(prob["n_feat"], prob["dims"]), t_noisy)   # same stream, same result
