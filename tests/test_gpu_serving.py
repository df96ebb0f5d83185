"""Serving under a device memory budget, cancellation and late consumers
(jp2g_submit / jp2g_poll / jp2g_cancel, jp2g_encode_batch under a budget).

Failures are made on the host: a budget that refuses pool growth, a request
cancelled while queued or on the device, a consumer that polls seconds late,
an engine destroyed with requests still queued. No GPU fault is involved.
Every page that completes must still give the oracle's bytes."""
import threading
import time

import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu

MIB = 1 << 20


def _pages(n, seed, sizes=((64, 64), (100, 70), (257, 129), (33, 7), (150, 150))):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = sizes[int(rng.integers(len(sizes)))]
        c = int(rng.choice([1, 3]))
        q = int(rng.choice([50, 75, 85, 100]))
        px = synth_page(w, h, c, 9000 + seed * 100 + i, photo_w=w // 3, photo_h=h // 3)
        out.append({"px": px, "w": w, "h": h, "ncomp": c, "quality": q, "fmt": i % 2})
    return out


def _oracle(orc, p):
    return orc.encode(p["px"], p["w"], p["h"], p["ncomp"], p["quality"], fmt=p["fmt"])


def test_served_requests_complete_under_a_small_budget(orc):
    # one page fits the 40 MiB budget on its own, the 24-page queue does not:
    # waves are retried from empty pools and split, never failed
    pages = _pages(24, 1)
    eng = jl.Engine(0, hbm_budget_bytes=40 * MIB)
    try:
        tickets = [eng.submit(p) for p in pages]
        got = [eng.poll(t) for t in tickets]
        for p, g in zip(pages, got):
            assert g == _oracle(orc, p)
        # the batch path splits its waves the same way
        outs = eng.encode_batch(pages)
        assert outs == got
    finally:
        eng.close()


def test_budget_too_small_for_any_page_fails_each_page_with_a_message():
    pages = _pages(3, 2)
    eng = jl.Engine(0, hbm_budget_bytes=256 << 10)
    try:
        tickets = [eng.submit(p) for p in pages]
        for t in tickets:
            with pytest.raises(jl.EncodeFailed, match="budget"):
                eng.poll(t, 60000)
        with pytest.raises(jl.EncodeFailed, match="budget"):
            eng.encode(pages[0]["px"], pages[0]["w"], pages[0]["h"], pages[0]["ncomp"], 85, 0)
        outs = eng.encode_batch(pages)
        assert all(isinstance(o, jl.EncodeFailed) for o in outs)
    finally:
        eng.close()


def test_slow_consumer_polls_seconds_late(orc):
    pages = _pages(8, 3)
    eng = jl.Engine(0)
    try:
        tickets = [eng.submit(p) for p in pages]
        time.sleep(2.0)
        for p, t in zip(pages, tickets):
            data = eng.poll(t, 0)  # long done: no wait
            assert data == _oracle(orc, p)
    finally:
        eng.close()


def test_cancelled_requests_are_dropped_and_the_rest_complete(orc):
    big = {"px": synth_page(2550, 3300, 3, 1001, photo_w=800, photo_h=600), "w": 2550, "h": 3300,
           "ncomp": 3, "quality": 75, "fmt": 1}
    small = _pages(10, 4)
    eng = jl.Engine(0)
    try:
        first = eng.submit(big)  # keeps the device busy while the others queue
        tickets = [eng.submit(p) for p in small]
        cancel = tickets[1::2]
        removed = {t: eng.cancel(t) for t in cancel}
        assert eng.poll(first) == eng.encode(big["px"], 2550, 3300, 3, 75, 1)
        for p, t in zip(small, tickets):
            if t not in removed:
                assert eng.poll(t) == _oracle(orc, p)
            elif removed[t]:
                # removed before reaching the device: the ticket is released
                with pytest.raises(jl.InvalidInput, match="unknown ticket"):
                    eng.poll(t, 0)
            else:
                # its wave was in flight: the result is dropped
                with pytest.raises(jl.EncodeFailed, match="cancelled"):
                    eng.poll(t)
        with pytest.raises(jl.InvalidInput):
            eng.cancel(123456789)
    finally:
        eng.close()


def test_cancel_wakes_a_waiting_poll():
    # several big pages keep the device busy so the small request is most
    # likely still queued when it is cancelled; every interleaving is checked
    bigs = [{"px": synth_page(2550, 3300, 3, 1002 + i, photo_w=800, photo_h=600), "w": 2550, "h": 3300,
             "ncomp": 3, "quality": 75, "fmt": 1} for i in range(6)]
    eng = jl.Engine(0)
    try:
        firsts = [eng.submit(b) for b in bigs]
        t = eng.submit(_pages(1, 5)[0])
        outcome = {}
        started = threading.Event()

        def waiter():
            started.set()
            try:
                outcome["data"] = eng.poll(t, 60000)
            except jl.Jp2LamError as e:
                outcome["err"] = e

        th = threading.Thread(target=waiter)
        th.start()
        started.wait()
        time.sleep(0.01)
        try:
            removed = eng.cancel(t)
        except jl.InvalidInput:
            removed = None  # the poll had already returned the result
        th.join(60)
        assert not th.is_alive()
        if removed is None:
            assert "data" in outcome
        elif removed:
            # EncodeFailed ("request cancelled") when the poll was waiting;
            # InvalidInput (unknown ticket) if it started after the cancel;
            # the result itself if the request had finished first
            assert "data" in outcome or isinstance(outcome["err"], (jl.EncodeFailed, jl.InvalidInput))
        else:
            assert isinstance(outcome.get("err"), jl.EncodeFailed) and "cancelled" in str(outcome["err"])
        for f in firsts:
            eng.poll(f)
    finally:
        eng.close()


def test_destroy_with_requests_still_queued_does_not_hang():
    pages = _pages(12, 6)
    eng = jl.Engine(0)
    for p in pages:
        eng.submit(p)
    t0 = time.time()
    eng.close()
    assert time.time() - t0 < 60


def test_staged_waves_alongside_direct_and_batch_calls(orc):
    # Without a budget the stager gathers and uploads each served wave
    # through its own pixel buffers while the worker runs the previous one;
    # direct encodes and batches from other threads use the engine's own
    # buffers in between. Planar RGB requests are always gathered in pinned
    # memory, the others are copied straight from the caller's memory.
    served = _pages(30, 7, sizes=((640, 480), (1275, 1650), (257, 129), (64, 64)))
    for p in served[::3]:
        if p["ncomp"] == 3:
            p["px"] = np.ascontiguousarray(p["px"].reshape(p["h"] * p["w"], 3).T)
            p["interleaved"] = False
    direct = _pages(6, 8)
    batch = _pages(8, 9, sizes=((640, 480), (300, 200)))
    eng = jl.Engine(0)
    results, errors = {}, []

    def run(name, f):
        try:
            results[name] = f()
        except Exception as e:  # reported below
            errors.append((name, e))

    def serve():
        tickets = []
        for p in served:
            tickets.append(eng.submit(p))
            time.sleep(0.003)
        return [eng.poll(t, 120000) for t in tickets]

    jobs = {
        "served": serve,
        "direct": lambda: [eng.encode(p["px"], p["w"], p["h"], p["ncomp"], p["quality"], p["fmt"]) for p in direct],
        "batch": lambda: eng.encode_batch(batch),
    }
    try:
        threads = [threading.Thread(target=run, args=(k, f)) for k, f in jobs.items()]
        for t in threads:
            t.start()
        for t in threads:
            t.join(180)
        assert not any(t.is_alive() for t in threads)
        assert not errors, errors
        for p, data in zip(served, results["served"]):
            want = p if p.get("interleaved", True) else dict(
                p, px=np.ascontiguousarray(p["px"].T).ravel())
            assert data == _oracle(orc, want)
        for p, data in zip(direct, results["direct"]):
            assert data == _oracle(orc, p)
        for p, data in zip(batch, results["batch"]):
            assert data == _oracle(orc, p)
    finally:
        eng.close()
