"""RankLoss, RankSpace and PPR on the GPU (src/algos/ep/loss.rs:15-38,
75-79, 130-222), through the C ABI.

Per-batch gradients are compared with the FP64 oracle on explicit samples
(FP32 within 1e-4 relative, the BF16 form within 1e-2 on its BF16-rounded
table, as for the other losses); the PPR sampler's walk end nodes are checked
for their structure; trained recall is compared with the CPU oracle's."""
import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import random_problem, sample_batch
from tests.test_gpu_parity import TOL_GRAD_BF16, check_parity, make_ctx

pytestmark = pytest.mark.gpu

RANK, RANKSPACE, PPR = _native.LOSS_RANK, _native.LOSS_RANKSPACE, _native.LOSS_PPR


def _gamma(loss):
    return 1.0 if loss == PPR else 0.3      # rank losses: tau


@pytest.mark.parametrize("loss", [RANK, RANKSPACE, PPR])
@pytest.mark.parametrize("dims", [32, 100])
@pytest.mark.parametrize("grad_mode", [0, 1])
def test_rank_losses_batch_parity(oracle, loss, dims, grad_mode):
    prob = random_problem(500 + dims + loss, n=300, n_feat=200, dims=dims, scale=0.5)
    smp = sample_batch(7 + loss, prob, B=96, K=5, R=6)
    g = _gamma(loss)
    ctx = make_ctx(prob, loss=loss, gamma=g, R=6, grad_mode=grad_mode)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=loss, gamma=g, grad_mode=grad_mode)


def test_rank_loss_keeps_some_anchors_and_drops_others(oracle):
    # tau splits the anchors: p of the positive above tau gives no loss
    prob = random_problem(61, n=300, n_feat=200, dims=32, scale=0.5)
    smp = sample_batch(62, prob, B=128, K=5, R=4)
    ctx = make_ctx(prob, loss=RANK, gamma=0.25, R=4)
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    _, gst, _, _ = ctx.batch_grad(s, prob["n_feat"], prob["dims"])
    assert 0 < (gst == 0).sum() < len(gst), np.bincount(gst)
    check_parity(oracle, prob, smp, ctx, prob["table"], loss=RANK, gamma=0.25)


def test_rankspace_fused_bf16(oracle):
    prob = random_problem(71, n=300, n_feat=200, dims=128, scale=0.5)
    smp = sample_batch(72, prob, B=128, K=5, R=5)
    ctx = make_ctx(prob, loss=RANKSPACE, gamma=0.3, R=5, form=1)
    table_bf16 = ctx.get_table(prob["n_feat"], prob["dims"])
    check_parity(oracle, prob, smp, ctx, table_bf16, grad_tol=TOL_GRAD_BF16, loss=RANKSPACE, gamma=0.3)


def _ppr_ctx(prob, R, restart):
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.batch_size, cfg.valid_pct = prob["dims"], R, 256, 0.0
    cfg.loss, cfg.gamma, cfg.ppr_restart_p = PPR, 1.0, restart
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    ctx.set_table(None)
    return ctx


def _bfs(rows, cols, src, limit=10):
    dist = {src: 0}
    frontier = [src]
    for d in range(1, limit + 1):
        nxt = []
        for u in frontier:
            for x in cols[int(rows[u]):int(rows[u + 1])].tolist():
                if x not in dist:
                    dist[x] = d
                    nxt.append(x)
        frontier = nxt
    return dist


def test_ppr_positives_are_walk_ends():
    # construct_positive (loss.rs:166-187): R walks of <= 10 moves; each
    # yields its end node, or a neighbour of v when it ends on v; weight 1;
    # a node without edges has only itself
    prob = random_problem(41, n=3000, n_feat=200, dims=16, deg=(0, 3))
    rows, cols = prob["rows"], prob["cols"]
    R, B = 7, 256
    anchors = np.arange(B, dtype=np.uint32) * 11
    means = {}
    for restart in (1.0, 0.0):
        ctx = _ppr_ctx(prob, R, restart)
        cnt, nbr, w, _ = ctx.sample(anchors, 3, R)
        again = ctx.sample(anchors, 3, R)
        assert np.array_equal(cnt, again[0]) and np.array_equal(nbr, again[1])
        dists = []
        for a, v in enumerate(anchors.tolist()):
            deg = int(rows[v + 1] - rows[v])
            ends = nbr[a, :cnt[a]].tolist()
            assert (w[a, :cnt[a]] == 1.0).all()
            if deg == 0:
                assert ends == [v]
                continue
            assert cnt[a] == R
            dist = _bfs(rows, cols, v, 10)
            nb = set(cols[int(rows[v]):int(rows[v + 1])].tolist())
            for u in ends:
                assert u in dist and (u != v or v in nb)
            dists += [dist[u] for u in ends]
        means[restart] = np.mean(dists)
        if restart == 1.0:
            # restart 1: the walk stops after its second move (unless on v)
            assert np.mean(np.array(dists) <= 2) > 0.9
    assert means[0.0] > means[1.0] + 0.5, means


@pytest.mark.parametrize("kind", ["rank", "rankspace", "ppr"])
def test_rank_losses_recall_matches_cpu_reference(oracle, kind):
    import cloverleaf_gb300 as cl
    from cloverleaf_gb300 import datagen
    from tests._eval import community_recall
    w = datagen.workload("sbm10k")
    ep = w["ep"]
    g = cl.Graph.from_csr(w["rows"], w["cols"], w["weights"])
    fs = cl.FeatureSet.from_csr(g, w["fptr"], w["fids"], w["n_feat"])
    loss = {"rank": cl.EPLoss.rank(0.5, ep["negatives"]), "rankspace": cl.EPLoss.rankspace(0.5, ep["negatives"]),
            "ppr": cl.EPLoss.ppr(0.5, ep["negatives"], 0.5)}[kind]
    code = {"rank": oracle.LOSS_RANK, "rankspace": oracle.LOSS_RANKSPACE, "ppr": oracle.LOSS_PPR}[kind]
    prop = cl.EmbeddingPropagator(alpha=ep["alpha"], loss=loss, batch_size=ep["batch_size"], dims=ep["dims"],
                                  passes=ep["passes"], max_nodes=ep["max_nodes"], valid_pct=0.0, indicator=False,
                                  form="fused")
    emb = prop.learn_features(g, fs)
    r_gpu = community_recall(w["fptr"], w["fids"], emb.table, w["community"])
    table, _ = oracle.train(w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                            alpha=ep["alpha"], loss=code, gamma=0.5, negatives=ep["negatives"],
                            batch_size=ep["batch_size"], passes=ep["passes"],
                            max_nodes=(oracle.SAMPLE_FIXED, ep["max_nodes"]), ppr_restart_p=0.5, threads=0)
    r_cpu = community_recall(w["fptr"], w["fids"], table, w["community"])
    print(f"{kind}: recall@10 gpu {r_gpu:.4f} cpu {r_cpu:.4f}")
    assert abs(r_gpu - r_cpu) <= 0.02, (r_gpu, r_cpu)
