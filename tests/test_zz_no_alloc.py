"""ep_get_table_static -- the row download that allocates no device memory --
called through the C ABI and checked against ep_get_table.

Both read the table through the same conversion kernel, so the rows must be
identical (tolerance 0), on two sweeps in a row.  The table (20000 x 200
FP32, 16 MB dense) is larger than the 8 MiB static scratch, so a full sweep
takes several windows.
"""
import ctypes

import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import random_problem

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 8 << 20


def static_rows(ctx, first, n, dims):
    out = np.full((n, dims), np.nan, np.float32)
    rc = _native.lib().ep_get_table_static(ctx.handle, first, n, ctypes.c_void_p(out.ctypes.data if n else 0))
    _native.check(rc, ctx.handle, "ep_get_table_static")
    return out


def trained_ctx(form, n_feat, dims):
    prob = random_problem(2024 + form, n=3000, n_feat=n_feat, dims=dims, feats=(1, 4))
    cfg = _native.default_config()
    cfg.dims, cfg.form, cfg.batch_size, cfg.negatives = dims, form, 256, 3
    cfg.loss, cfg.gamma, cfg.valid_pct, cfg.passes = _native.LOSS_STARSPACE, 0.5, 0.0, 1
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], n_feat)
    ctx.set_table(prob["table"])
    ctx.train_batches(4)
    return ctx


@pytest.mark.parametrize("form", [_native.FORM_PLAIN_FP32, _native.FORM_FUSED_BF16])
def test_static_download_matches_get_table(form):
    n_feat, dims = 20000, 200
    ctx = trained_ctx(form, n_feat, dims)
    want = ctx.get_table(n_feat, dims)
    window = SCRATCH_BYTES // (4 * dims)
    assert window < n_feat
    for _ in range(2):          # two sweeps in a row through the same scratch
        got = np.concatenate([static_rows(ctx, r, min(window, n_feat - r), dims)
                              for r in range(0, n_feat, window)])
        assert np.array_equal(got, want)
    # two single calls in a row on an inner window
    a = static_rows(ctx, 1234, 777, dims)
    b = static_rows(ctx, 1234, 777, dims)
    assert np.array_equal(a, want[1234:2011]) and np.array_equal(b, a)


def test_static_download_limits():
    n_feat, dims = 20000, 200
    ctx = trained_ctx(_native.FORM_PLAIN_FP32, n_feat, dims)
    window = SCRATCH_BYTES // (4 * dims)
    with pytest.raises(_native.NativeError) as e:
        static_rows(ctx, 0, window + 1, dims)
    assert e.value.code == -1 and "static scratch" in str(e.value)
    with pytest.raises(_native.NativeError) as e:
        static_rows(ctx, n_feat - 1, 2, dims)
    assert e.value.code == -1
    assert static_rows(ctx, n_feat, 0, dims).shape == (0, dims)
    assert np.array_equal(static_rows(ctx, n_feat - window, window, dims), ctx.get_table(n_feat, dims)[-window:])
