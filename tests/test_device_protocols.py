"""Models of two pieces of device logic whose correctness is a matter of
ordering, checked exhaustively or under random schedules on the CPU (the GPU
tests check the kernels themselves: test_gpu_train.py's ring-shape equality
tests and test_gpu_parity.py::test_batch_grad_multi_chunk_spans).

* The reducer ring of Adam placement 3 (ep_red.cu, OUT_RING): reducing warps
  take tickets from a counter without waiting (slot t % S, round t / S), wait
  until the slot's consumed-rounds word reaches their round, fill the slot and
  arrive on its `full` mbarrier; Adam warp k owns the slots congruent to k
  modulo cw and takes their rounds in order, waiting on `full` by parity.
  The model checks, under random interleavings, that every parity test is
  exact (the barrier's completed-phase count is r or r + 1 when round r is
  tested), that no slot is overwritten before it is consumed, that every
  ticket is consumed once, and that nothing deadlocks.
* The fix-ups' 32-ary search for the last item of a feature spanning
  reducer chunks (owner_last in ep_red.cu).
* The test k_reduce and k_fixup share to tell long spans (more than
  FIX_SHORT later chunks, left to k_fixup_long) from short ones, against the
  span's true end.
* k_reduce's item loop: per-warp lists of the kept items and the feature
  starts, walked NF items at a time with a branch-free path for groups that
  hold no feature start, against the plain sequential walk (same closes, same
  sums in the same order).
"""
import random

import pytest


def ring_run(pw, cw, slots, rows, seed):
    assert slots % cw == 0
    rng = random.Random(seed)
    tail = done = 0
    full = [0] * slots            # completed phases of each slot's `full` mbarrier
    consumed = [0] * slots        # the slot's consumed-rounds word
    held = [None] * slots         # round stored in the slot, not yet consumed
    got = []
    prod = [{"left": rows[i], "state": "take", "t": None} for i in range(pw)]
    cons = [{"h": k, "state": "wait"} for k in range(cw)]
    for _ in range(10 ** 6):
        actors = [("p", i) for i in range(pw) if prod[i]["state"] != "done"] + \
                 [("c", k) for k in range(cw) if cons[k]["state"] != "done"]
        if not actors:
            break
        kind, i = rng.choice(actors)
        if kind == "p":
            p = prod[i]
            if p["state"] == "take":
                if p["left"] == 0:
                    done += 1
                    p["state"] = "done"
                    continue
                p["t"], tail = tail, tail + 1
                p["state"] = "fill"
            else:
                s, r = p["t"] % slots, p["t"] // slots
                if r > 0 and consumed[s] < r:
                    continue                       # waits for the consumer of round r - 1
                assert held[s] is None, "slot overwritten before it was consumed"
                assert full[s] == r
                held[s] = r
                full[s] += 1                       # arrive + bulk copies complete
                p["left"] -= 1
                p["state"] = "take"
        else:
            c = cons[i]
            s, r = c["h"] % slots, c["h"] // slots
            assert full[s] in (r, r + 1), "parity test ambiguous"
            if full[s] == r + 1:
                assert held[s] == r
                held[s] = None
                consumed[s] = r + 1
                got.append(c["h"])
                c["h"] += cw
            elif done == pw and tail <= c["h"]:
                c["state"] = "done"
    else:
        raise AssertionError("no progress: deadlock")
    assert sorted(got) == list(range(tail)), "every ticket consumed once"


@pytest.mark.parametrize("shape", [(12, 4, 32), (6, 2, 4), (2, 14, 56), (1, 1, 2), (15, 1, 3), (3, 3, 3), (8, 8, 8)])
def test_ring_protocol_model(shape):
    pw, cw, slots = shape
    for seed in range(100):
        rr = random.Random(seed)
        ring_run(pw, cw, slots, [rr.randint(0, 30) for _ in range(pw)], seed)


def owner_last_search(lo, hi, last):
    """The device search: skey[i] == f for i <= last (a prefix of [lo, hi))."""
    while hi - lo > 1:
        span = hi - lo
        step = span // 32 if span > 32 else 1
        k = sum(1 for lane in range(32) if lo + (lane + 1) * step < hi and lo + (lane + 1) * step <= last)
        nlo = lo + k * step
        if k < 32:
            hi = min(hi, nlo + step)
        lo = nlo
    return lo


def test_owner_last_search_model():
    rng = random.Random(1)
    for _ in range(50000):
        lo = rng.randint(0, 1000)
        hi = lo + rng.randint(1, 5000)
        last = rng.randint(lo, hi - 1)
        assert owner_last_search(lo, hi, last) == last
    # the case the 1M-node parity test met: 32 probes inside, stride 2, the end 15 past them
    assert owner_last_search(64511, 162315, 65542) == 65542


# --- features spanning reducer chunks: which spans k_reduce queues as long ---

FIX_SHORT = 16


def span_is_long(keys, c, f, C):
    """k_reduce / k_fixup: the owner chunk c's feature f still fills the
    start of chunk c + 1 + FIX_SHORT."""
    probe = (c + 1 + FIX_SHORT) * C
    return probe < len(keys) and keys[probe] == f


def test_long_span_test_matches_the_span_end():
    rng = random.Random(3)
    for trial in range(300):
        C = rng.choice([32, 64, 128])
        keys, f = [], 0
        while len(keys) < 60 * C:
            run = rng.choice([1, 2, 5, 40, C - 1, C, C + 1, 3 * C, 16 * C, 17 * C, 17 * C + 1, 18 * C - 1, 40 * C])
            keys += [f] * run
            f += 1
        M = len(keys)
        last_item = {}
        for i, k in enumerate(keys):
            last_item[k] = i
        for c in range((M + C - 1) // C):
            i1 = min((c + 1) * C, M)
            f_last = keys[i1 - 1]
            owner = i1 < M and keys[i1] == f_last and keys.index(f_last) >= c * C
            if not owner:
                continue
            last_chunk = last_item[f_last] // C
            assert span_is_long(keys, c, f_last, C) == (last_chunk - c > FIX_SHORT), (trial, c)


# --- the reducer's item loop: per-warp lists, then a walk in list order ---

def sequential_walk(items, head_open):
    """Items (feature, kept, weight) of one chunk in sorted order, the first
    feature possibly continuing from the previous chunk (head_open).  Returns
    the closes in order: (feature, sum of kept weights, any kept, head)."""
    out = []
    cur, acc, any_kept, head = items[0][0], 0, False, head_open
    for f, kept, wgt in items:
        if f != cur:
            out.append((cur, acc, any_kept, head))
            cur, acc, any_kept, head = f, 0, False, False
        if kept:
            acc += wgt
            any_kept = True
    out.append((cur, acc, any_kept, head))
    return out


def list_walk(items, head_open, RW=128, NF=3):
    """k_reduce's form: per window of RW items, phase 1 (32 items per step)
    appends the kept items and the feature starts (with the number of kept
    items before them) to lists; phase 2 takes the kept items NF at a time,
    a group with no feature start in one piece, closing a feature when the
    walk reaches the first kept item of the next; features with no kept item
    after their start close at the window's end."""
    out = []
    cur, acc, any_kept, head = items[0][0], 0, False, head_open

    def close_open(fnew):
        nonlocal cur, acc, any_kept, head
        out.append((cur, acc, any_kept, head))
        cur, acc, any_kept, head = fnew, 0, False, False

    prev_f = None if not head_open else items[0][0]
    for wb in range(0, len(items), RW):
        ents, segs = [], []
        for ib in range(wb, min(wb + RW, len(items)), 32):
            batch = items[ib:ib + 32]
            for lane, (f, kept, wgt) in enumerate(batch):
                pf = batch[lane - 1][0] if lane else prev_f
                seg_start = f != pf
                if seg_start and ib + lane != 0:
                    segs.append((f, len(ents)))
                if kept:
                    ents.append(wgt)
            prev_f = batch[-1][0]
        nk, ns, j = len(ents), len(segs), 0
        next_b = segs[0][1] if ns else float("inf")
        for k in range(0, nk, NF):
            if k + NF <= nk and k + NF <= next_b:
                acc += sum(ents[k:k + NF])
                any_kept = True
                continue
            for u in range(NF):
                if k + u < nk:
                    while k + u >= next_b:
                        close_open(segs[j][0])
                        j += 1
                        next_b = segs[j][1] if j < ns else float("inf")
                    acc += ents[k + u]
                    any_kept = True
        while j < ns:
            close_open(segs[j][0])
            j += 1
    out.append((cur, acc, any_kept, head))
    return out


@pytest.mark.parametrize("nf", [1, 2, 3, 4])
def test_item_list_walk_matches_the_sequential_walk(nf):
    rng = random.Random(11 + nf)
    for trial in range(2000):
        n = rng.randint(1, 400)
        items, f = [], rng.randint(0, 5)
        while len(items) < n:
            run = rng.choice([1, 1, 2, 3, 5, 8, 33, 70, 130])
            p_kept = rng.choice([0.0, 0.3, 0.8, 1.0])
            for _ in range(min(run, n - len(items))):
                items.append((f, rng.random() < p_kept, rng.randint(1, 1000)))
            f += rng.randint(1, 3)
        head_open = rng.random() < 0.5
        assert list_walk(items, head_open, NF=nf) == sequential_walk(items, head_open), trial
