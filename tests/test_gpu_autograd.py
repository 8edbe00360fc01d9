"""The torch.autograd.Function binding with the hand-written backward:
central finite differences (FP64, eps 1e-6) and the oracle's per-batch
gradient (FP32 within 1e-4 relative) on 64 fixed seeded batches of 128
anchors of the 1,000-node SBM workload (dims 32, 5 negatives)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import datagen
from cloverleaf_gb300.autograd import EPBatchLoss
from tests._cases import rel_err, sample_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sbm1k():
    w = datagen.workload("sbm1k")
    rng = np.random.default_rng(3)
    w["table"] = (rng.standard_normal((w["n_feat"], w["ep"]["dims"])) / 4).astype(np.float32)
    w["n"] = len(w["rows"]) - 1
    return w


def batches(w, count, seed0=1000):
    prob = dict(rows=w["rows"], cols=w["cols"], n=w["n"])
    return [sample_batch(seed0 + i, prob, B=128, K=w["ep"]["max_nodes"], R=w["ep"]["negatives"]) for i in range(count)]


def args(s):
    return s["anchors"], s["nbr_ptr"], s["nbr"], s["nbr_w"], s["neg"]


@pytest.mark.parametrize("loss", ["margin", "starspace"])
def test_fp32_backward_matches_reference_gradient(oracle, sbm1k, loss):
    w = sbm1k
    lo = cl.EPLoss.margin(1.0, 5) if loss == "margin" else cl.EPLoss.starspace(0.5, 5)
    f = EPBatchLoss(w["rows"], w["cols"], w["fptr"], w["fids"], w["n_feat"], 32, lo, grad_mode="reference")
    worst = 0.0
    for s in batches(w, 64):
        t = torch.tensor(w["table"], device="cuda", requires_grad=True)
        lv = f(t, *args(s))
        st_ok = torch.isfinite(lv) & (lv > 0)
        lv.sum().backward()
        cfg = oracle.loss_cfg(loss=0 if loss == "margin" else 1, gamma=lo.gamma, grad_mode=0)
        ol, ost, og, ot = oracle.batch(w["fptr"], w["fids"], w["n_feat"], w["table"], w["rows"], *args(s), cfg, "f64")
        assert np.array_equal(st_ok.cpu().numpy(), ost == 0)
        assert rel_err(lv.detach().cpu().numpy()[ost == 0], ol[ost == 0]) < 1e-4
        worst = max(worst, rel_err(t.grad.cpu().numpy(), og))
    assert worst < 1e-4, worst


@pytest.mark.parametrize("loss", ["margin", "starspace"])
def test_fp64_backward_matches_finite_differences(sbm1k, loss):
    w = sbm1k
    lo = cl.EPLoss.margin(1.0, 5) if loss == "margin" else cl.EPLoss.starspace(0.5, 5)
    f = EPBatchLoss(w["rows"], w["cols"], w["fptr"], w["fids"], w["n_feat"], 32, lo, grad_mode="true")
    rng = np.random.default_rng(5)
    worst = 0.0
    for s in batches(w, 4, seed0=77):
        base = torch.tensor(w["table"], dtype=torch.float64, device="cuda")
        t = base.clone().requires_grad_(True)
        f(t, *args(s)).sum().backward()
        g = t.grad.cpu().numpy()
        rows_touched = np.nonzero(np.abs(g).sum(1) > 0)[0]
        picks = [(int(r), int(rng.integers(0, 32))) for r in rng.choice(rows_touched, 40, replace=False)]
        eps = 1e-6
        for r, k in picks:
            tp, tm = base.clone(), base.clone()
            tp[r, k] += eps
            tm[r, k] -= eps
            fd = (f(tp, *args(s)).sum().item() - f(tm, *args(s)).sum().item()) / (2 * eps)
            # gradcheck-style bound: FD rounding noise is ~ulp(sum of 128 losses)/eps ~ 1e-8
            worst = max(worst, abs(fd - g[r, k]) / (1e-6 + 1e-4 * abs(g[r, k])))
    assert worst < 1.0, worst


def test_fp64_matches_oracle_fp64(oracle, sbm1k):
    w = sbm1k
    lo = cl.EPLoss.starspace(0.5, 5)
    f = EPBatchLoss(w["rows"], w["cols"], w["fptr"], w["fids"], w["n_feat"], 32, lo, grad_mode="reference")
    for s in batches(w, 4, seed0=500):
        t = torch.tensor(w["table"], dtype=torch.float64, device="cuda", requires_grad=True)
        f(t, *args(s)).sum().backward()
        cfg = oracle.loss_cfg(loss=1, gamma=0.5, grad_mode=0)
        _, _, og, _ = oracle.batch(w["fptr"], w["fids"], w["n_feat"], w["table"], w["rows"], *args(s), cfg, "f64")
        # the reference (and the oracle) accumulate feature counts in f32
        # (model.rs:268-271), the FP64 kernels in double: agreement ~1e-7
        assert rel_err(t.grad.cpu().numpy(), og) < 1e-6
