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
