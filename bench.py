#!/usr/bin/env python
"""Benchmark: Embedding Propagation training throughput on GB300.

A step is one training batch (one optimizer step) of the 10M-node Chung-Lu
workload (``cl10m``: 10M nodes, ~160M directed edges, degree exponent 2.0,
degrees clipped to [1, 10^4]; Poisson(6) features over 2M Zipf(1.05) slots;
dims 256, max_neighbors 25, 10 negatives, StarSpace margin 0.5, batch 8192).

Legs in one run (rank 0, N=1):
  value        fused BF16 form, inputs resident in HBM, CUDA-event time of the
               timed batches (replays of a CUDA graph of 16 batches, and one
               graph for a run's remainder, built and uploaded beforehand)
  plain_fp32   the plain FP32 form on the same workload and steps
  cpu_baseline the oracle's CPU restatement of the reference training loop on
               a bounded sample of the same workload, all host threads
  e2e          one full pass through the C ABI from pinned host buffers:
               context creation, graph/feature upload, table init, training,
               table download, all inside the timed region (median of three
               such passes)
  roofline     algorithmic bytes of the dominant stage / its mean CUDA-event
               duration from a stage-by-stage profile of the same batches
  recall_at_10 held-out-edge recall@10 (scripts/evaluate.py:29-61) of the
               fused, plain and CPU-restatement forms after one pass on the
               same graph with 1% of its edges held out
  largest      the 50M-node / ~1B-edge workload: fused and plain nodes/s
               over a bounded run of batches
  plain_drop_in_cl1m  the 1M-node bipartite workload: plain FP32 and fused
               nodes/s and the CPU restatement on the same graph

``--impl reference`` times only the CPU reference restatement (the Rust
reference cannot be built here) and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EP train nodes/sec & HBM roofline %: fused BF16 vs plain FP32 GPU vs CPU ref"
UNIT = "nodes/sec"
E2E_PASSES = 3
def l2_note(n_feat, dims, n_edges):
    """Why no L2 flush is needed: the inputs each step touches exceed L2."""
    gb = lambda b: f"{b / 1e9:.1f} GB"
    return (f"inputs larger than L2 (BF16 table {gb(n_feat * dims * 2)}, CSR {gb(n_edges * 8)}, "
            f"FP32 Adam moments {gb(n_feat * dims * 8)}, read at each step's random rows)")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def loaded_libraries():
    """Base names of this repository's shared libraries mapped into the
    process (the trainer, the workload generators, the oracle)."""
    names = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and path.endswith(".so"):
                    names.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(names)


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                vendor = next((l.split(":", 1)[1].strip() for l in out.splitlines()
                               if l.split(":")[0].strip() == "Vendor ID"), "")
                name = line.split(":", 1)[1].strip()
                return f"{vendor} {name}".strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="cl10m")
    p.add_argument("--scale", type=float, default=1.0, help="shrink the Chung-Lu node count (profiling)")
    p.add_argument("--loss", default="starspace", choices=["starspace", "margin"])
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-knn", action="store_true")
    p.add_argument("--no-recall", action="store_true", help="skip the held-out-edge recall@10 leg")
    p.add_argument("--recall-queries", type=int, default=20000)
    p.add_argument("--no-large", action="store_true", help="skip the 50M-node leg")
    p.add_argument("--large-steps", type=int, default=100)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cl1m", action="store_true", help="skip the 1M-node bipartite leg")
    p.add_argument("--profile-steps", type=int, default=100)
    return p.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


_PINNED = []   # keeps the page-locked tensors behind the numpy views alive


def pinned_copy(a: np.ndarray) -> np.ndarray:
    """A copy of `a` in page-locked host memory (so host->device copies run at
    full link speed)."""
    import torch

    t = torch.empty(a.shape, dtype={np.uint64: torch.int64, np.uint32: torch.int32,
                                    np.float32: torch.float32}[a.dtype.type], pin_memory=True)
    _PINNED.append(t)
    out = t.numpy().view(a.dtype)
    out[...] = a
    return out


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    rows.append((float(p[1]), float(p[2]), p[5:9]))
                except ValueError:
                    continue
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        mx = max(r[1] for r in rows)
        load = [r for r in rows if r[0] >= 0.5 * mx] or rows
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def fused_mode():
    """Adam placement of the fused form (the library default is 2: Adam in the
    reducer through a per-warp queue; 1: a separate Adam kernel)."""
    try:
        return int(os.environ.get("EP_FUSED_MODE", "2"))
    except ValueError:
        return 2


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(unique_rows):
    """DRAM bytes per launch of the dominant kernel (the fused reducer) from
    the committed ncu summary (profiles/traffic.json): the bytes measured on
    a reduced workload of the same batch shape, plus each further unique row
    of this batch at its Adam-state bytes (table row read and written, m and
    v read and written).  None when there is no summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)["k_reduce"]
        return t["bytes_per_launch"] + (unique_rows - t["unique_rows"]) * t["bytes_per_extra_row"]
    except Exception:
        return None


def knn_leg(peak_tflops):
    """Exact cosine top-10 on the tensor cores (ep_knn_cosine): 19,456
    queries (128 per SM) against 262,144 rows of 256 dims.  GEMM FLOP =
    2 * n_q * n_db * 256; time = the top-k kernel's CUDA-event time."""
    from cloverleaf_gb300 import _native

    rng = np.random.default_rng(11)
    n_db, n_q, d, k = 262144, 19456, 256, 10
    db = rng.standard_normal((n_db, d), dtype=np.float32)
    q = db[:n_q]
    _native.knn_cosine(db[:4096], q[:256], k)          # warm-up
    _native.knn_cosine(db, q, k)
    ms = float(_native.lib().ep_knn_last_kernel_ms())
    tflops = 2.0 * n_q * n_db * d / (ms / 1e3) / 1e12
    return {"kernel": "k_cos_topk (tcgen05, BF16 x BF16 -> FP32 TMEM, fused top-k)", "n_db": n_db, "n_q": n_q,
            "dims": d, "k": k, "kernel_ms": ms, "tflops": tflops, "peak_bf16_tflops": peak_tflops,
            "frac": tflops / peak_tflops if peak_tflops else None}


def make_config(ep, form, loss, passes=1):
    from cloverleaf_gb300 import _native

    cfg = _native.default_config()
    cfg.alpha, cfg.dims, cfg.batch_size, cfg.passes = ep["alpha"], ep["dims"], ep["batch_size"], passes
    cfg.loss = _native.LOSS_STARSPACE if loss == "starspace" else _native.LOSS_MARGIN
    cfg.gamma, cfg.negatives = ep["gamma"], ep["negatives"]
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(ep["max_nodes"])
    cfg.valid_pct = 0.0
    cfg.form = _native.FORM_FUSED_BF16 if form == "fused" else _native.FORM_PLAIN_FP32
    cfg.device = int(os.environ.get("LOCAL_RANK", "0"))
    return cfg


def gpu_leg(w, form, loss, steps, warmup, world, sampler_device=None):
    from cloverleaf_gb300 import _native

    ctx = _native.Context(make_config(w["ep"], form, loss))
    ctx.upload_graph(w["rows"], w["cols"], w["weights"])
    ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
    ctx.set_table(None)
    ctx.train_batches(warmup)
    clocks = None
    barrier(world)
    t0 = time.perf_counter()
    if sampler_device is not None:
        with ClockSampler(sampler_device) as cs:
            st = ctx.train_batches(steps)
        clocks = cs.summary()
    else:
        st = ctx.train_batches(steps)
    wall = time.perf_counter() - t0
    barrier(world)
    return ctx, st, wall, clocks


def recall_leg(w, loss, queries):
    """Held-out-edge recall@10 (scripts/evaluate.py:29-61) after the
    workload's passes, for the fused and plain GPU forms and the CPU
    restatement, all trained on the same graph with 1% of its undirected
    edges held out (seeded)."""
    from cloverleaf_gb300 import _native, evaluate
    from oracle import ep_oracle as O

    ep = w["ep"]
    t0 = time.time()
    rows, cols, wts, test = evaluate.holdout_edges(w["rows"], w["cols"], w["weights"], 0.01, seed=5,
                                                   max_test=queries)
    out = {"k": 10, "test_edges": int(len(test)), "held_out_fraction": 0.01, "passes": ep["passes"],
           "metric": "share of held-out edges (u, v) with v among the 10 nearest node embeddings of u (cosine); "
                     "auc: share with cos(u, v) > cos(u, random node)"}
    for form in ("fused", "plain"):
        ctx = _native.Context(make_config(ep, form, loss, passes=ep["passes"]))
        ctx.upload_graph(rows, cols, None)
        ctx.upload_features(w["fptr"], w["fids"], w["n_feat"])
        ctx.set_table(None)
        ctx.train(ep["passes"])
        table = ctx.get_table(w["n_feat"], ep["dims"])
        ctx.close()
        out[form] = evaluate.heldout_recall(w["fptr"], w["fids"], table, test)
        out[form]["table_checksum"] = float(table.sum(dtype=np.float64))
        del table
        log(f"[bench] recall {form}: {out[form]}")
    t1 = time.time()
    table, st = O.train(rows, cols, wts, w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"], alpha=ep["alpha"],
                        loss=O.LOSS_STARSPACE if loss == "starspace" else O.LOSS_MARGIN, gamma=ep["gamma"],
                        negatives=ep["negatives"], batch_size=ep["batch_size"], passes=ep["passes"],
                        max_nodes=(O.SAMPLE_FIXED, float(ep["max_nodes"])), threads=0)
    out["cpu_train_seconds"] = round(time.time() - t1, 1)
    # the CPU restatement over one whole pass (all host threads): its rate
    # over the pass's timed region, next to the bounded sample of cpu_baseline
    out["cpu_full_pass"] = {"value": st.anchors / max(st.seconds, 1e-9), "unit": UNIT, "anchors": int(st.anchors),
                            "seconds": round(st.seconds, 2)}
    out["cpu"] = evaluate.heldout_recall(w["fptr"], w["fids"], table, test)
    del table
    for form in ("fused", "plain"):
        out[f"{form}_minus_cpu"] = out[form]["recall"] - out["cpu"]["recall"]
    out["seconds"] = round(time.time() - t0, 1)
    log(f"[bench] recall cpu: {out['cpu']} ({out['cpu_train_seconds']} s of CPU training)")
    return out


def cl1m_leg(loss, steps, warmup, world, cpu_seconds):
    """The 1M-node bipartite Chung-Lu workload (weights U[1,5], dims 128, 25
    neighbours, 10 negatives, batch 1024): PLAIN FP32 and FUSED nodes/s, and
    the CPU restatement on a bounded sample, all on this graph."""
    from cloverleaf_gb300 import datagen

    w = datagen.workload("cl1m")
    ep = w["ep"]
    n = len(w["rows"]) - 1
    out = {"workload": f"cl1m: bipartite Chung-Lu {n} nodes / {len(w['cols'])} directed edges, weights U[1,5], "
                       f"dims {ep['dims']}, max_neighbors {ep['max_nodes']}, {ep['negatives']} negatives, "
                       f"batch {ep['batch_size']}", "steps": steps, "warmup": warmup}
    for form in ("plain", "fused"):
        ctx, st, wall, _ = gpu_leg(w, form, loss, steps, warmup, world)
        ctx.close()
        ms = allmax(st["ms"], world)
        out[form] = {"value": allsum(st["anchors"], world) / (ms / 1e3), "unit": UNIT,
                     "ms_per_step": ms / max(st["batches"], 1)}
    cv, cst, cores, nb = cpu_reference(w, loss, cpu_seconds)
    out["cpu"] = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port",
                  "sample": f"{cst.batches} batches of {ep['batch_size']} anchors, {cst.seconds:.1f}s"}
    out["plain_vs_cpu"] = out["plain"]["value"] / cv
    out["fused_vs_plain"] = out["fused"]["value"] / out["plain"]["value"]
    log(f"[bench] cl1m: plain {out['plain']['value'] / 1e6:.2f} M, fused {out['fused']['value'] / 1e6:.2f} M, "
        f"cpu {cv / 1e3:.1f} k nodes/s")
    return out


def large_leg(loss, steps, warmup, world):
    """The 50M-node / ~1B-edge Chung-Lu workload (dims 256, max_neighbors 32,
    16 negatives, batch 32768): fused and plain nodes/s over `steps` batches,
    and the fused form's per-stage profile."""
    from cloverleaf_gb300 import datagen

    t0 = time.time()
    w = datagen.workload("cl50m")
    gen_s = time.time() - t0
    ep = w["ep"]
    n = len(w["rows"]) - 1
    out = {"workload": f"cl50m: Chung-Lu {n} nodes / {len(w['cols'])} directed edges, dims {ep['dims']}, "
                       f"max_neighbors {ep['max_nodes']}, {ep['negatives']} negatives, batch {ep['batch_size']}",
           "generate_seconds": round(gen_s, 1), "steps": steps, "warmup": warmup}
    log(f"[bench] cl50m generated in {gen_s:.1f}s: {n} nodes, {len(w['cols'])} edges")
    for form in ("fused", "plain"):
        ctx, st, wall, _ = gpu_leg(w, form, loss, steps, warmup, world)
        ms = allmax(st["ms"], world)
        rec = {"value": allsum(st["anchors"], world) / (ms / 1e3), "unit": UNIT,
               "ms_per_step": ms / max(st["batches"], 1),
               "step_gbs": st["alg_bytes"] / (st["ms"] / 1e3) / 1e9}
        if form == "fused":
            stage_ms, pst = ctx.profile_batches(20)
            rec["stage_ms"] = stage_ms
        ctx.close()
        out[form] = rec
        log(f"[bench] cl50m {form}: {rec['value'] / 1e6:.2f} M nodes/s ({rec['ms_per_step']:.3f} ms/batch)")
    out["fused_speedup"] = out["fused"]["value"] / out["plain"]["value"]
    return out


def cpu_reference(w, loss, seconds, threads=0, max_batches=None):
    """The oracle's restatement of the reference loop on host cores, on a
    bounded number of batches sized to take about `seconds`."""
    from oracle import ep_oracle as O

    ep = w["ep"]
    kw = dict(dims=ep["dims"], alpha=ep["alpha"], loss=O.LOSS_STARSPACE if loss == "starspace" else O.LOSS_MARGIN,
              gamma=ep["gamma"], negatives=ep["negatives"], batch_size=ep["batch_size"], passes=1,
              max_nodes=(O.SAMPLE_FIXED, float(ep["max_nodes"])), threads=threads)
    args = (w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"])
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    if max_batches is None:
        # one batch per thread: the restatement runs batches concurrently, so
        # fewer would leave threads idle and underestimate the rate
        _, st = O.train(*args, max_batches=max(2, cores), **kw)
        rate = cpu_rate(st)
        max_batches = max(cores, int(seconds * rate / ep["batch_size"]))
    _, st = O.train(*args, max_batches=max_batches, **kw)
    return cpu_rate(st), st, cores, max_batches


def cpu_rate(st):
    """Anchors per second of a run of the CPU restatement.  A bounded sample
    of b batches stands for b / steps_per_pass of a pass, so it carries that
    share of the pass's one shuffle of the anchor order (mod.rs:173), not all
    of it."""
    share = min(1.0, st.batches / max(st.steps_per_pass, 1))
    return st.anchors / max(st.seconds - st.shuffle_seconds * (1.0 - share), 1e-9)


def main():
    args = parse()
    rank, world = dist_setup(args.gpus)
    from cloverleaf_gb300 import datagen

    if args.impl == "reference" and rank != 0:
        return 0
    t0 = time.time()
    w = datagen.workload(args.workload, scale=args.scale)
    ep = w["ep"]
    n_nodes = len(w["rows"]) - 1
    if rank == 0:
        log(f"[bench] {args.workload}: {n_nodes} nodes, {len(w['cols'])} directed edges, "
            f"{len(w['fids'])} feature occurrences, {w['n_feat']} slots ({time.time() - t0:.1f}s)")
    kind = "SBM" if args.workload.startswith("sbm") else "Chung-Lu"
    wl = (f"{args.workload}: {kind} {n_nodes} nodes / {len(w['cols'])} directed edges, dims {ep['dims']}, "
          f"max_neighbors {ep['max_nodes']}, {ep['negatives']} negatives, batch {ep['batch_size']}, {args.loss} 0.5")
    config = {"workload": wl, "nodes": n_nodes, "edges": int(len(w["cols"])), "dims": ep["dims"],
              "batch": ep["batch_size"], "max_neighbors": ep["max_nodes"], "negatives": ep["negatives"],
              "loss": args.loss, "table_dtype": "bf16", "moments_dtype": "f32",
              "l2": l2_note(w["n_feat"], ep["dims"], len(w["cols"])),
              "parallelism": f"replicas{world}" if world > 1 else "single"}

    if args.impl == "reference":
        cores = os.cpu_count() or 1
        _, stw, _, _ = cpu_reference(w, args.loss, 0, max_batches=max(args.warmup, 1))
        value, st, cores, nb = cpu_reference(w, args.loss, 0, max_batches=max(args.steps, 1))
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": nb, "warmup": args.warmup, "ms_per_step": 1e3 * st.anchors / value / max(st.batches, 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": dict(config, table_dtype="f32"),
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": "port",
                                 "sample": f"{st.batches} batches of {ep['batch_size']} anchors "
                                           f"({st.anchors} anchors) of the {args.workload} workload"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "loaded_libraries": loaded_libraries()}
        print(json.dumps(line), flush=True)
        return 0

    # pinned host copies: the e2e leg uploads from these
    for k in ("rows", "cols", "weights", "fptr", "fids"):
        w[k] = pinned_copy(np.ascontiguousarray(w[k]))
    dev = int(os.environ.get("LOCAL_RANK", "0"))

    # --- fused BF16 (headline) ---
    ctx, st, wall, clocks = gpu_leg(w, "fused", args.loss, args.steps, args.warmup, world,
                                    sampler_device=dev if rank == 0 else None)
    ms = allmax(st["ms"], world)
    anchors = allsum(st["anchors"], world)
    value = anchors / (ms / 1e3)
    log(f"[bench] fused: {st['anchors']} anchors in {st['ms']:.1f} ms device / {wall:.2f} s wall "
        f"-> {value / 1e6:.2f} M nodes/s; loss {st['train_loss']:.4f}")
    stage_ms, pst = ctx.profile_batches(min(args.profile_steps, args.steps))
    ctx.close()
    B = pst["batches"] or 1
    d, s_el = ep["dims"], 2.0
    G, U, S, A = pst["gathered_rows"] / B, pst["unique_rows"] / B, pst["sampled_neighbors"] / B, pst["anchors"] / B
    items = pst["items"] / B
    # Algorithmic HBM bytes per launch of each stage's kernels (per batch):
    #   forward  gathered table rows G*d*s, their feature ids 4G, sampled
    #            neighbour ids 4S, per-role scale/valid 8*B*(R+2)
    #   reduce   sorted item keys and values 12*items, plus (Adam in the
    #            reducer) U*d*(2s+16): m, v read+written (FP32), table row
    #            read+written; (Adam split off) the U*d*4 gradient rows
    #   adam     (split form only) gradient rows + Adam state U*d*(2s+20)
    split = fused_mode() == 1
    stage_bytes = {"forward": G * d * s_el + 4 * G + 4 * S + 8 * A * (ep["negatives"] + 2),
                   "reduce": 12 * items + (U * d * 4 if split else U * d * (2 * s_el + 16)),
                   "adam": U * d * (2 * s_el + 20) if split else 0.0}
    kernel_of = {"forward": "k_fwd_gather+k_fwd_loss", "adam": "k_adam_dense",
                 "reduce": "k_reduce (gradient rows)" if split else "k_reduce (Adam fused, cp.async queue)"}
    dom = max(stage_ms, key=stage_ms.get)
    peak, peak_kind = load_peaks()
    rf_stage = max(("forward", "reduce", "adam"), key=lambda k: stage_ms[k])
    achieved = stage_bytes[rf_stage] / (stage_ms[rf_stage] / 1e3) / 1e9
    step_bytes = pst["alg_bytes"] / B
    step_ms = st["ms"] / max(st["batches"], 1)
    roofline = {"bound": "hbm", "kernel": kernel_of[rf_stage],
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                "traffic": load_traffic(U) if split is False else None, "alg_bytes_per_launch": stage_bytes[rf_stage],
                "stage_ms": stage_ms, "dominant_stage": dom,
                "stage_gbs": {k: stage_bytes[k] / (stage_ms[k] / 1e3) / 1e9 for k in stage_bytes if stage_bytes[k]},
                "step": {"achieved": step_bytes / (step_ms / 1e3) / 1e9, "alg_bytes_per_step": step_bytes,
                         "frac": step_bytes / (step_ms / 1e3) / 1e9 / peak},
                "per_batch": {"G": G, "U": U, "S": S, "items": items}}
    log(f"[bench] stages (ms/batch): " + ", ".join(f"{k} {v:.3f}" for k, v in stage_ms.items()))

    # --- end to end through the C ABI from pinned host buffers (one pass) ---
    e2e = None
    if not args.no_e2e:
        from cloverleaf_gb300 import _native

        out = pinned_copy(np.zeros((w["n_feat"], d), np.float32))    # the caller's result buffer
        # a single pass takes under a second and its wall time varies with the
        # host (allocator state after the other legs): time E2E_PASSES whole
        # passes, each a fresh context, and report the median
        secs, phases = [], []
        for _ in range(E2E_PASSES):
            barrier(world)
            t = [time.perf_counter()]
            ectx = _native.Context(make_config(ep, "fused", args.loss, passes=1))
            ectx.upload_graph(w["rows"], w["cols"], w["weights"])
            ectx.upload_features(w["fptr"], w["fids"], w["n_feat"])
            ectx.set_table(None)
            t.append(time.perf_counter())
            est = ectx.train(1)[0]
            t.append(time.perf_counter())
            table = ectx.get_table(w["n_feat"], d, out=out)
            t.append(time.perf_counter())
            ectx.close()
            t.append(time.perf_counter())
            secs.append(allmax(t[-1] - t[0], world))
            phases.append({"setup": round(t[1] - t[0], 4), "train": round(t[2] - t[1], 4),
                           "download": round(t[3] - t[2], 4), "close": round(t[4] - t[3], 4),
                           "train_device_ms": round(est["ms"], 2)})
        e_sec = float(np.median(secs))
        h2d = sum(w[k].nbytes for k in ("rows", "cols", "weights", "fptr", "fids"))
        nb = max(est["batches"], 1)
        e2e = {"value": allsum(est["anchors"], world) / e_sec, "unit": UNIT, "h2d_bytes_per_step": h2d / nb,
               "d2h_bytes_per_step": table.nbytes / nb, "steps": nb, "seconds": e_sec,
               "passes_timed": E2E_PASSES, "seconds_each": [round(x, 4) for x in secs], "phases": phases,
               "note": "one full pass via ep_create/upload/set_table/ep_train/ep_get_table; median of the passes"}
        log(f"[bench] e2e: {e2e['value'] / 1e6:.2f} M nodes/s over {nb} steps ({e_sec:.2f}s)")

    # --- plain FP32 ---
    plain = None
    if not args.no_plain:
        pctx, pst2, pwall, _ = gpu_leg(w, "plain", args.loss, args.steps, args.warmup, world)
        pctx.close()
        pms = allmax(pst2["ms"], world)
        pv = allsum(pst2["anchors"], world) / (pms / 1e3)
        plain = {"value": pv, "unit": UNIT, "ms_per_step": pms / max(pst2["batches"], 1),
                 "fused_speedup": value / pv}
        log(f"[bench] plain fp32: {pv / 1e6:.2f} M nodes/s (fused {value / pv:.2f}x)")

    # --- CPU reference restatement (rank 0) ---
    cpu = None
    if rank == 0 and not args.no_cpu:
        cv, cst, cores, nb = cpu_reference(w, args.loss, args.cpu_seconds)
        cpu = {"value": cv, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": "port",
               "sample": f"{cst.batches} batches of {ep['batch_size']} anchors ({cst.anchors} anchors) of "
                         f"{args.workload}, {cst.seconds:.1f}s"}
        log(f"[bench] cpu reference: {cv / 1e3:.1f} k nodes/s on {cores} threads")

    if rank == 0:
        knn = None
        if not args.no_knn:
            try:
                with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                    pk_bf16 = float(json.load(f)["bf16_tflops"])
            except Exception:
                pk_bf16 = 1900.0
            knn = knn_leg(pk_bf16)
            log(f"[bench] knn: {knn['tflops']:.1f} TFLOP/s ({knn['kernel_ms']:.2f} ms) = "
                f"{100 * knn['frac']:.1f}% of {pk_bf16:.0f}")
        recall = None
        single = args.workload == "cl10m" and args.scale == 1.0 and world == 1
        if not args.no_recall and world == 1:
            recall = recall_leg(w, args.loss, args.recall_queries)
        drop_in = None
        if not args.no_cl1m and single:
            drop_in = cl1m_leg(args.loss, 300, max(args.warmup, 3), world, 8.0)
        large = None
        if not args.no_large and single:
            del w
            _PINNED.clear()
            large = large_leg(args.loss, args.large_steps, max(args.warmup, 3), world)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / max(st["batches"], 1), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "bf16 table storage, f32 accumulation and Adam moments",
                "data": "synthetic", "config": config,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(st["launches"]),
                "clocks": clocks, "plain_fp32": plain,
                "speedup_vs_cpu": (value / cpu["value"]) if cpu else None,
                "recall_at_10": recall, "largest": large, "plain_drop_in_cl1m": drop_in,
                "loaded_libraries": loaded_libraries(),
                "eval_knn": knn}
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
