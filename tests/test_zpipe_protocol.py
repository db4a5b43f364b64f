"""The pipelined z pass's copy / barrier protocol, modelled on the host (CPU).

`k_pass_c_pipe` (csrc/zpass_pipe.cuh) runs nw warps per CTA over the CTA's nk
lines: warp w takes right-hand sides w, w + nw, ... of every line; its next
task's rows are fetched into its staging buffer right after its first stage
has read the current ones; the Green spectrum of line k sits in buffer k & 1,
and the copy of line k + 2 is issued by the last warp to finish its Green
step of line k (a shared counter).  This test replays that protocol with the
kernel's own task formulas, warps interleaved in random orders, and checks
that no warp ever waits for a copy that will never be issued (no deadlock),
that a spectrum buffer is refilled only after every warp is done with it,
that every warp reads the spectrum of the line it is working on, and that
every copy issued is waited for before the CTA ends.
"""
import random

import pytest


def _run(nk, L, nw, seed):
    rng = random.Random(seed)
    # per warp: (k, l) of the current task, phase, staged task
    state = [{"k": 0, "l": w, "phase": "wait_x", "staged": (0, w), "done": False} for w in range(nw)]
    gbuf = {0: 0}                      # buffer -> line whose spectrum it holds (issued copies)
    if nk > 1:
        gbuf[1] = 1
    gdone = [0, 0]
    waited_g = set()                   # (warp, line) pairs whose spectrum the warp waited for
    issued_g = {0, 1} if nk > 1 else {0}
    steps = 0
    while not all(s["done"] for s in state):
        runnable = []
        for w, s in enumerate(state):
            if s["done"]:
                continue
            if s["phase"] == "wait_g" and gbuf.get(s["k"] & 1) != s["k"]:
                continue               # the spectrum of this line has not been issued into its buffer
            runnable.append(w)
        assert runnable, f"deadlock: {state}"
        w = rng.choice(runnable)
        s = state[w]
        k, l = s["k"], s["l"]
        if s["phase"] == "wait_x":
            assert s["staged"] == (k, l)          # the staged rows are this task's
            # first stage read the rows: the next task's rows are fetched now
            k2, l2 = k, l + nw
            if l2 >= L:
                k2, l2 = k + 1, w
            s["next"] = (k2, l2)
            s["staged"] = (k2, l2) if k2 < nk else None
            s["phase"] = "wait_g"
        elif s["phase"] == "wait_g":
            assert gbuf[k & 1] == k                # the buffer holds this line's spectrum
            waited_g.add((w, k))
            if l + nw >= L:                        # this warp's last Green step of line k
                gdone[k & 1] += 1
                if gdone[k & 1] == nw:
                    gdone[k & 1] = 0
                    if k + 2 < nk:
                        # every warp is past its Green step of line k
                        assert all(st is s or st["done"] or st["k"] > k for st in state)
                        gbuf[k & 1] = k + 2
                        issued_g.add(k + 2)
            k2, l2 = s["next"]
            s["k"], s["l"] = k2, l2
            s["phase"] = "wait_x"
            if k2 >= nk:
                s["done"] = True
                assert s["staged"] is None        # no copy left in flight for this warp
        steps += 1
        assert steps < 10 * nk * L + 100
    # every spectrum issued was waited for by every warp
    assert issued_g == set(range(nk))
    for k in range(nk):
        for w in range(nw):
            assert (w, k) in waited_g


@pytest.mark.parametrize("nk,L", [(1, 1), (1, 8), (2, 3), (5, 8), (7, 12), (9, 32), (4, 17)])
def test_protocol_terminates_and_keeps_buffers_consistent(nk, L):
    nw = min(L, 8)
    for seed in range(40):
        _run(nk, L, nw, seed)
