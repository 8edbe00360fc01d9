"""The oracle itself, pinned against the reference's own unit tests and
cross-checked against an independent autograd restatement (CPU only)."""
import math

import numpy as np
import pytest

from tests._cases import random_problem, rel_err, sample_batch

# src/graph.rs:697-705 build_edges()
EDGES = [(0, 1, 1.0), (1, 1, 3.0), (1, 2, 2.0), (2, 0, 2.5), (1, 0, 10.0)]


def test_csr_dedup_sorted_rows(oracle):
    # graph.rs:120-142 sorts edges by (from, to) before merging duplicates;
    # graph.rs:803-813 (test_par_iter_mut_for_each_doubles_weights) relies on
    # that order: node 1's weights are [10, 3, 2].
    rows, cols, w = oracle.csr_from_edges(EDGES, dedup=True)
    assert rows.tolist() == [0, 1, 4, 5]
    assert cols.tolist() == [1, 0, 1, 2, 0]
    assert w.tolist() == [1.0, 10.0, 3.0, 2.0, 2.5]
    assert (w * 2).tolist()[1:4] == [20.0, 6.0, 4.0]


def test_csr_insertion_order(oracle):
    # graph.rs:708-715 (construct_csr) and :718-727 (test_graph) expect the
    # insertion order within a row; that is what the code produces without
    # the (from, to) sort, i.e. with deduplicate = false.  (Those two tests
    # pass dedup = true, contradicting graph.rs:124 and :803-813; the code
    # is followed.)
    rows, cols, w = oracle.csr_from_edges(EDGES, dedup=False)
    assert rows.tolist() == [0, 1, 4, 5]
    assert cols.tolist() == [1, 1, 2, 0, 0]
    assert w.tolist() == [1.0, 3.0, 2.0, 10.0, 2.5]


def test_cdf_known_answers(oracle):
    # graph.rs:751-761 (construct_cdf), in the insertion order of that test
    rows, cols, w = oracle.csr_from_edges(EDGES, dedup=False)
    cdf = oracle.cdf_convert(rows, w)
    np.testing.assert_allclose(cdf, [1.0, 3 / 15, 5 / 15, 15 / 15, 1.0], rtol=0, atol=1e-7)
    # graph.rs:764-776 (construct_cdf_to_p): CDF -> probabilities
    p = np.diff(np.concatenate([[0.0], cdf[1:4].astype(np.float64)]))
    np.testing.assert_allclose(p, [3 / 15, 2 / 15, 10 / 15], atol=1e-7)
    # last entry of every non-empty row is exactly 1 (graph.rs:689-690)
    rows, cols, w = oracle.csr_from_edges(EDGES, dedup=True)
    cdf = oracle.cdf_convert(rows, w)
    assert cdf[rows[1:] - 1].tolist() == [1.0, 1.0, 1.0]


def test_cdf_empty_and_zero_rows(oracle):
    # graph.rs:781-787: empty rows are a no-op; zero-weight rows become uniform (:675-681)
    rows = np.array([0, 0, 3, 3], np.uint64)
    w = np.zeros(3, np.float32)
    cdf = oracle.cdf_convert(rows, w)
    np.testing.assert_allclose(cdf, [1 / 3, 2 / 3, 1.0], atol=1e-7)


def test_zero_degree_node(oracle):
    # graph.rs:831-847: node 1 has no out-edges
    rows, cols, w = oracle.csr_from_edges([(0, 2, 1.0), (2, 0, 2.0)], dedup=True)
    assert rows.tolist() == [0, 1, 1, 2]


def _two_feature_case(oracle, loss, gamma, t_row, h_row, u_row):
    # anchor 0 has feature 0 (h), its one neighbour 1 has feature 1 (t), the
    # negative 2 has feature 2 (u)
    table = np.array([h_row, t_row, u_row], np.float32)
    fptr = np.array([0, 1, 2, 3], np.uint64)
    fids = np.array([0, 1, 2], np.uint32)
    rows = np.array([0, 1, 2, 3], np.uint64)
    cfg = oracle.loss_cfg(loss=loss, gamma=gamma)
    return oracle.batch(fptr, fids, 3, table, rows, [0], [0, 1], [1], [1.0], [[2]], cfg, "f64")


def test_euclidean_known_answer(oracle):
    # loss.rs:250-255: |[1,3] - [3,5]| = sqrt(8).  Margin loss with h=[1,3],
    # t=[3,5] and a negative at distance 0.5 from t: L = 1 + sqrt(8) - 0.5;
    # dL/dh = -(t-h)/|t-h| = -[1,1]/sqrt(2).
    loss, status, grad, touched = _two_feature_case(oracle, oracle.LOSS_MARGIN, 1.0, [3, 5], [1, 3], [3.3, 5.4])
    assert status.tolist() == [0]
    assert loss[0] == pytest.approx(1.0 + math.sqrt(8.0) - 0.5, abs=1e-6)
    np.testing.assert_allclose(grad[0], [-1 / math.sqrt(2), -1 / math.sqrt(2)], atol=1e-6)


def test_l2norm_known_answer(oracle):
    # loss.rs:258-263: il2norm([1,3]) = [1,3]/sqrt(10).  StarSpace with
    # t=[1,3], h=[3,1], u=[1,3]: cos(t,h) = 6/10, cos(h,u) = 6/10, so
    # L = gamma - (0.6 - 0.6) = gamma.
    loss, status, grad, touched = _two_feature_case(oracle, oracle.LOSS_STARSPACE, 0.5, [1, 3], [3, 1], [1, 3])
    assert status.tolist() == [0]
    assert loss[0] == pytest.approx(0.5, abs=1e-7)
    # dL/du = (I - uu^T/|u|^2) h_hat / |u| with |u| = sqrt(10)
    u = np.array([1, 3.0]) / math.sqrt(10)
    hh = np.array([3, 1.0]) / math.sqrt(10)
    gu = (hh - u * u.dot(hh)) / math.sqrt(10)
    np.testing.assert_allclose(grad[2], gu, atol=1e-7)


# Hand-derived known answers for the two default losses (loss.rs:59-105),
# every role's gradient written out from the formulas, not from any
# restatement.  Count weights (model.rs:257-278): an occurrence of a feature
# of node u in a role counts w_u + 1 (w_u = 1 for the anchor and the
# negatives, the given neighbour weight in the reconstruction); a feature's
# leaf gradient is its count share of the role's gradient (model.rs:448-463).
#
# Margin, gamma = 1, R = 3:
#   h = mean(E0, E1) = mean((0,2), (2,0)) = (1,1);   t = E2 = (4,5)
#   u1 = E3 = (4,1): |t-u1| = 4, l1 = 1 + 5 - 4 = 2  (kept)
#   u2 = E4 = (1,5): |t-u2| = 3, l2 = 1 + 5 - 3 = 3  (kept)
#   u3 = E5 = (4,15): |t-u3| = 10, l3 = -4           (dropped: no gradient)
#   L = (2 + 3) / 2 = 2.5
#   dL/dh  = -(t-h)/|t-h| = (-0.6, -0.8)              -> E0, E1 get half each
#   dL/dt  = [2 (t-h)/5 - (t-u1)/4 - (t-u2)/3] / 2 = (0.1, 0.3)
#   dL/du1 = (t-u1)/4 / 2 = (0, 0.5);  dL/du2 = (t-u2)/3 / 2 = (0.5, 0)
MARGIN_KAT = dict(
    table=[[0, 2], [2, 0], [4, 5], [4, 1], [1, 5], [4, 15]],
    fptr=[0, 2, 3, 4, 5, 6], fids=[0, 1, 2, 3, 4, 5],
    nbr_ptr=[0, 1], nbr=[1], nbr_w=[1.0], neg=[[2, 3, 4]], gamma=1.0, loss=2.5,
    grad={0: [-0.3, -0.4], 1: [-0.3, -0.4], 2: [0.1, 0.3], 3: [0.0, 0.5], 4: [0.5, 0.0]})
# StarSpace, gamma = 0.5, R = 2, with x^ = x/|x| and d x^ = (I - x^ x^T)/|x|:
#   h = E0 = (2,0): h^ = (1,0)
#   t = (2 E1 + 4 E2) / 6 with neighbour weights 1 and 3 (counts 2 and 4),
#       E1 = (-2,1), E2 = (1,1): t = (0,1) = t^
#   u1 = E3 = (3,4): u1^ = (.6,.8); l1 = .5 - (t^.h^ - h^.u1^) = 1.1  (kept)
#   u2 = E4 = (-1,0): l2 = .5 - (0 - (-1)) = -.5 -> max(0, .) = 0     (dropped)
#   L = 1.1
#   dL/dh  = (I - h^h^T)/2 (u1^ - t^) = (0, -0.1)
#   dL/dt  = (I - t^t^T)/1 (-h^)      = (-1, 0)  -> E1 gets 2/6, E2 4/6
#   dL/du1 = (I - u1^u1^T)/5 h^       = (0.128, -0.096)
STARSPACE_KAT = dict(
    table=[[2, 0], [-2, 1], [1, 1], [3, 4], [-1, 0]],
    fptr=[0, 1, 2, 3, 4, 5], fids=[0, 1, 2, 3, 4],
    nbr_ptr=[0, 2], nbr=[1, 2], nbr_w=[1.0, 3.0], neg=[[3, 4]], gamma=0.5, loss=1.1,
    grad={0: [0.0, -0.1], 1: [-1 / 3, 0.0], 2: [-2 / 3, 0.0], 3: [0.128, -0.096]})


# Contrastive, pos_margin (gamma) = 0.875, neg_margin = 0.5 (both exact in
# f32, as the reference holds them), R = 2 (loss.rs:107-128: mean over the
# kept terms of (cos(h^,u^) - neg_margin)+ and (pos_margin - cos(t^,h^))+, a
# term kept when positive):
#   h = E0 = (3,4): h^ = (.6,.8), |h| = 5;  t = E1 = (0,2) (one neighbour,
#       weight 1): t^ = (0,1), |t| = 2;  pos term .875 - .8 = .075  (kept)
#   u1 = E2 = (4,3): u1^ = (.8,.6), |u1| = 5; cos = .96: .96 - .5 = .46 (kept)
#   u2 = E3 = (-1,0): cos = -.6 -> -1.1                               (dropped)
#   L = (.46 + .075) / 2 = .2675
#   dL/dh  = (I - h^h^T)/5 (u1^ - t^)/2     = (0.0704, -0.0528)
#   dL/dt  = (I - t^t^T)/2 (-h^/2)           = (-0.15, 0)
#   dL/du1 = (I - u1^u1^T)/5 (h^/2)          = (-0.0168, 0.0224)
CONTRASTIVE_KAT = dict(
    table=[[3, 4], [0, 2], [4, 3], [-1, 0]],
    fptr=[0, 1, 2, 3, 4], fids=[0, 1, 2, 3],
    nbr_ptr=[0, 1], nbr=[1], nbr_w=[1.0], neg=[[2, 3]], gamma=0.875, neg_margin=0.5, loss=0.2675,
    grad={0: [0.0704, -0.0528], 1: [-0.15, 0.0], 2: [-0.0168, 0.0224]})

KATS = {"margin": (MARGIN_KAT, 0), "starspace": (STARSPACE_KAT, 1), "contrastive": (CONTRASTIVE_KAT, 2)}


def kat_args(k):
    n = len(k["fptr"]) - 1
    rows = np.arange(n + 1, dtype=np.uint64)          # one (unused) edge per node
    return (np.array(k["fptr"], np.uint64), np.array(k["fids"], np.uint32), len(k["table"]),
            np.array(k["table"], np.float32), rows, [0], k["nbr_ptr"], k["nbr"], k["nbr_w"], k["neg"])


@pytest.mark.parametrize("name", ["margin", "starspace", "contrastive"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_default_losses_known_answers(oracle, name, prec):
    k, lid = KATS[name]
    cfg = oracle.loss_cfg(loss=lid, gamma=k["gamma"], neg_margin=k.get("neg_margin", 0.0))
    loss, st, g, t = oracle.batch(*kat_args(k), cfg, prec)
    tol = 1e-12 if prec == "f64" else 1e-6
    assert st.tolist() == [0]
    assert abs(loss[0] - k["loss"]) < tol * 10
    assert sorted(np.nonzero(t)[0].tolist()) == sorted(k["grad"])
    for f, row in k["grad"].items():
        np.testing.assert_allclose(g[f], row, atol=tol * 10, rtol=0)


@pytest.mark.parametrize("loss", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("grad_mode", [0, 1])
@pytest.mark.parametrize("weighting", [0, 1, 2])
def test_c_oracle_matches_autograd(oracle, loss, grad_mode, weighting):
    prob = random_problem(7 + loss, n=80, n_feat=50, dims=8)
    smp = sample_batch(11 + grad_mode, prob, B=24, K=3, R=4, weighted=weighting == 2)
    gamma = {0: 1.0, 3: 0.3, 4: 0.3, 5: 1.0}.get(loss, 0.5)      # rank losses: tau
    cfg = oracle.loss_cfg(loss=loss, gamma=gamma, neg_margin=0.1, grad_mode=grad_mode, loss_weighting=weighting,
                          lw_exp=0.5)
    args = (prob["fptr"], prob["fids"], prob["n_feat"], prob["table"], prob["rows"], smp["anchors"], smp["nbr_ptr"],
            smp["nbr"], smp["nbr_w"], smp["neg"])
    l64, s64, g64, t64 = oracle.batch(*args, cfg, "f64")
    la, sa, ga, ta = oracle.batch_autograd(*args, loss=loss, gamma=gamma, neg_margin=0.1, grad_mode=grad_mode,
                                           loss_weighting=weighting, lw_exp=0.5)
    assert (s64 == sa).all() and (t64 == ta).all()
    assert rel_err(l64, la) < 1e-12
    assert rel_err(g64, ga) < 1e-12
    l32, s32, g32, t32 = oracle.batch(*args, cfg, "f32")
    assert (s32 == sa).all()
    assert rel_err(g32, ga) < 1e-5


def test_rank_loss_known_answer(oracle):
    # h = [1, 0], t = [.5, .5], u = [0, 1]: logits u.h = 0 and h.t = .5, so
    # p = e^.5 / (1 + e^.5); L = -ln p (p < tau = .9); dL/du = (1 - p) h,
    # dL/dt = (p - 1) h, dL/dh = (1 - p) u + (p - 1) t (loss.rs:130-155)
    table = np.array([[1.0, 0.0], [0.5, 0.5], [0.0, 1.0]], np.float32)
    fptr = np.array([0, 1, 2, 3], np.uint64)
    fids = np.array([0, 1, 2], np.uint32)
    rows = np.array([0, 1, 2, 3], np.uint64)
    args = (fptr, fids, 3, table, rows, [0], [0, 1], [1], [1.0], [[2]])
    loss, st, g, t = oracle.batch(*args, oracle.loss_cfg(loss=oracle.LOSS_RANK, gamma=0.9), "f64")
    p = math.exp(0.5) / (1 + math.exp(0.5))
    assert st.tolist() == [0] and abs(loss[0] + math.log(p)) < 1e-7
    np.testing.assert_allclose(g[2], [1 - p, 0], atol=1e-7)
    np.testing.assert_allclose(g[1], [p - 1, 0], atol=1e-7)
    np.testing.assert_allclose(g[0], [(p - 1) * 0.5, (1 - p) + (p - 1) * 0.5], atol=1e-7)
    # p >= tau: no loss, no gradient
    loss, st, g, t = oracle.batch(*args, oracle.loss_cfg(loss=oracle.LOSS_RANK, gamma=0.5), "f64")
    assert st.tolist() == [1] and not t.any()


def test_first_occurrence_rule(oracle):
    # A feature shared by h(v) and a negative: in reference mode the negative's
    # contribution is dropped (mod.rs:367); in true mode both add up.
    table = np.array([[1.0, 0.0], [0.0, 1.0], [0.6, 0.8]], np.float32)
    fptr = np.array([0, 2, 3, 4], np.uint64)       # node0: f0,f2  node1: f1  node2: f2
    fids = np.array([0, 2, 1, 2], np.uint32)
    rows = np.array([0, 1, 2, 3], np.uint64)
    args = (fptr, fids, 3, table, rows, [0], [0, 1], [1], [1.0], [[2]])
    _, _, gr, _ = oracle.batch(*args, oracle.loss_cfg(loss=0, gamma=2.0, grad_mode=0), "f64")
    _, _, gt, _ = oracle.batch(*args, oracle.loss_cfg(loss=0, gamma=2.0, grad_mode=1), "f64")
    la, sa, ga, ta = oracle.batch_autograd(*args, loss=0, gamma=2.0, grad_mode=0)
    np.testing.assert_allclose(gr, ga, atol=1e-12)
    assert not np.allclose(gr[2], gt[2])


def test_nan_roles_are_dropped(oracle):
    # t == h exactly: d|t-h| is NaN (sqrt at 0), so h's and t's features are
    # skipped while the negative's gradient survives (mod.rs:370).
    table = np.array([[1.0, 2.0], [1.3, 2.4]], np.float32)   # |t - u| = 0.5
    fptr = np.array([0, 1, 2, 3], np.uint64)
    fids = np.array([0, 0, 1], np.uint32)          # anchor and neighbour share feature 0
    rows = np.array([0, 1, 2, 3], np.uint64)
    args = (fptr, fids, 2, table, rows, [0], [0, 1], [1], [1.0], [[2]])
    loss, st, g, t = oracle.batch(*args, oracle.loss_cfg(loss=0, gamma=1.0), "f64")
    la, sa, ga, ta = oracle.batch_autograd(*args, loss=0, gamma=1.0)
    assert st.tolist() == [0] and sa.tolist() == [0]
    assert t.tolist() == [False, True] and ta.tolist() == [False, True]
    np.testing.assert_allclose(g, ga, atol=1e-12)


def test_adam_known_answer(oracle):
    # optimizer.rs:43-81 by hand for one element, t = pass + 1 = 2
    table = np.array([[0.5]], np.float32)
    m = np.zeros((1, 1), np.float32)
    v = np.zeros((1, 1), np.float32)
    g = np.array([[0.2]], np.float32)
    t2, m2, v2 = oracle.adam(table, m, v, g, np.array([1], np.uint8), 0.01, 1)
    mh = (0.1 * 0.2) / (1 - 0.9 ** 2)
    vh = (0.001 * 0.04) / (1 - 0.999 ** 2)
    assert t2[0, 0] == pytest.approx(0.5 - 0.01 * mh / (math.sqrt(vh) + 1e-8), rel=1e-5)
    # rows containing NaN are skipped (optimizer.rs:56)
    t3, m3, v3 = oracle.adam(table, m, v, np.array([[np.nan]], np.float32), np.array([1], np.uint8), 0.01, 1)
    assert t3[0, 0] == 0.5 and m3[0, 0] == 0.0


def test_lr_schedule(oracle):
    # scheduler.rs:120-137 with mod.rs:133-137
    a = 0.01
    assert oracle.lr_cos_decay(a / 100, a, 20, 100, 10) == pytest.approx(a / 100 + 0.5 * (a - a / 100), rel=1e-6)
    assert oracle.lr_cos_decay(a / 100, a, 20, 100, 50) == pytest.approx(
        a / 100 + 0.5 * (a - a / 100) * (1 + math.cos(math.pi * 0.5)), rel=1e-6)


def test_oracle_training_learns_communities(oracle):
    from cloverleaf_gb300 import datagen
    from tests._eval import community_recall

    w = datagen.workload("sbm10k")
    ep = w["ep"]
    table, st = oracle.train(w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                             alpha=ep["alpha"], loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"],
                             negatives=ep["negatives"], batch_size=ep["batch_size"], passes=ep["passes"],
                             max_nodes=(oracle.SAMPLE_FIXED, ep["max_nodes"]), threads=4)
    assert st.batches == 5 * 40 and st.anchors == 5 * 10_000
    r = community_recall(w["fptr"], w["fids"], table, w["community"])
    assert r > 0.5, r


def test_align_known_answer(oracle):
    # node 0 -> (1, p=.25), (2, p=.75); node 1 -> (0, p=1); node 2 no edges
    rows = np.array([0, 2, 3, 3], np.uint64)
    cols = np.array([1, 2, 0], np.uint32)
    wcdf = np.array([0.25, 1.0, 1.0], np.float32)
    emb = np.array([[1.0, 0.0], [0.0, 2.0], [4.0, 4.0]], np.float32)
    out = oracle.align(rows, cols, wcdf, emb, alpha=0.5)
    np.testing.assert_allclose(out[0], 0.5 * (0.25 * emb[1] + 0.75 * emb[2]) + 0.5 * emb[0], atol=1e-7)
    np.testing.assert_allclose(out[1], 0.5 * emb[0] + 0.5 * emb[1], atol=1e-7)
    np.testing.assert_allclose(out[2], 0.5 * emb[2], atol=1e-7)
    # max_neighbors 1: only the first edge, its probability not renormalised
    out = oracle.align(rows, cols, wcdf, emb, alpha=0.0, max_neighbors=1)
    np.testing.assert_allclose(out[0], 0.25 * emb[1], atol=1e-7)
    # adaptive: a = min(1, 1/ln(deg + 1)); deg 2 -> 1/ln 3, deg 1 -> 1 (1/ln 2 > 1)
    out = oracle.align(rows, cols, wcdf, emb)
    a = 1 / math.log(3)
    np.testing.assert_allclose(out[0], (1 - a) * (0.25 * emb[1] + 0.75 * emb[2]) + a * emb[0], rtol=1e-6)
    np.testing.assert_allclose(out[1], emb[1], atol=1e-7)
    np.testing.assert_allclose(out[2], emb[2], atol=1e-7)
