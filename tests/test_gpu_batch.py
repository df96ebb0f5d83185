"""Batched and served encoding (jp2g_encode_batch, jp2g_submit/jp2g_poll):
every page's codestream must be byte-identical to the single-page path and
to the oracle, alone and in any mix, whatever the wave split, the MQ
blocks-per-warp setting or the arrival order."""
import random
import threading

import numpy as np
import pytest

import jp2lam_gb300 as jl
from jp2lam_gb300 import _native
from jp2lam_gb300._native import synth_page

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = jl.Engine(0)
    yield e
    e.close()


def _mix(n, seed, big=False):
    """Pages of mixed size, colour, quality and format, like the uneven batch
    (sizes scaled down so the oracle stays quick)."""
    rng = random.Random(seed)
    sizes = [(64, 64), (100, 70), (257, 129), (320, 413), (1, 1), (33, 7)]
    if big:
        sizes += [(1275, 1650)]
    pages = []
    for i in range(n):
        w, h = rng.choice(sizes)
        c = rng.choice([1, 3])
        q = rng.choice([50, 75, 85, 100, 20])
        fmt = rng.choice([0, 1])
        px = synth_page(w, h, c, 5000 + i, photo_w=w // 3, photo_h=h // 3)
        pages.append({"px": px, "w": w, "h": h, "ncomp": c, "quality": q, "fmt": fmt})
    return pages


def _single(eng, p):
    return eng.encode(p["px"], p["w"], p["h"], p["ncomp"], p["quality"], p["fmt"])


def test_batch_matches_single_and_oracle(eng, orc):
    pages = _mix(24, 1)
    outs = eng.encode_batch(pages)
    for p, o in zip(pages, outs):
        assert isinstance(o, bytes)
        assert o == _single(eng, p)
        assert o == orc.encode(p["px"], p["w"], p["h"], p["ncomp"], p["quality"], p["fmt"])


@pytest.mark.parametrize("wave_blocks", [1, 7, 100, 160000])
def test_wave_split_does_not_change_output(eng, wave_blocks):
    pages = _mix(12, 2)
    ref = [_single(eng, p) for p in pages]
    old = eng.get_option(_native.OPT_WAVE_BLOCKS)
    try:
        eng.set_option(_native.OPT_WAVE_BLOCKS, wave_blocks)
        assert eng.encode_batch(pages) == ref
    finally:
        eng.set_option(_native.OPT_WAVE_BLOCKS, old)


@pytest.mark.parametrize("bpw", [1, 3, 8, 32])
def test_mq_blocks_per_warp_does_not_change_output(eng, bpw):
    pages = _mix(8, 3, big=True)
    eng.set_option(_native.OPT_MQ_BLOCKS_PER_WARP, 0)
    ref = eng.encode_batch(pages)
    try:
        eng.set_option(_native.OPT_MQ_BLOCKS_PER_WARP, bpw)
        assert eng.encode_batch(pages) == ref
        assert _single(eng, pages[0]) == ref[0]
    finally:
        eng.set_option(_native.OPT_MQ_BLOCKS_PER_WARP, 0)


@pytest.mark.parametrize("wave_blocks", [1, 40, 160000])
def test_batch_failure_is_per_page(eng, wave_blocks):
    # invalid pages hold host pixels but no place in the wave's pixel
    # buffer: whatever wave they fall in, nothing of theirs is uploaded
    pages = _mix(6, 4)
    bad = dict(pages[1])
    bad["ncomp"] = 2
    bad["px"] = np.full(bad["w"] * bad["h"] * 2, 200, np.uint8)
    bad2 = dict(pages[3])
    bad2["quality"] = 300
    batch = [pages[0], bad, pages[2], bad2, pages[4], pages[5]]
    old = eng.get_option(_native.OPT_WAVE_BLOCKS)
    try:
        eng.set_option(_native.OPT_WAVE_BLOCKS, wave_blocks)
        outs = eng.encode_batch(batch)
    finally:
        eng.set_option(_native.OPT_WAVE_BLOCKS, old)
    assert isinstance(outs[1], jl.InvalidInput) and isinstance(outs[3], jl.InvalidInput)
    for k in (0, 2, 4, 5):
        assert outs[k] == _single(eng, batch[k])


def test_empty_batch(eng):
    assert eng.encode_batch([]) == []


def test_batch_planar_and_device_inputs(eng):
    torch = pytest.importorskip("torch")
    w, h = 301, 203
    px = synth_page(w, h, 3, 77, photo_w=100, photo_h=60)
    planar = np.ascontiguousarray(px.reshape(h * w, 3).T)
    dev = torch.from_numpy(px.copy()).cuda()
    torch.cuda.synchronize()
    outs = eng.encode_batch([
        {"px": px, "w": w, "h": h, "ncomp": 3, "quality": 85, "fmt": 1},
        {"px": planar, "w": w, "h": h, "ncomp": 3, "quality": 85, "fmt": 1, "interleaved": False},
        {"px": dev.data_ptr(), "w": w, "h": h, "ncomp": 3, "quality": 85, "fmt": 1, "on_device": True},
    ])
    assert outs[0] == outs[1] == outs[2] == eng.encode(px, w, h, 3, 85, 1)


def test_option_validation(eng):
    with pytest.raises(jl.InvalidInput):
        eng.set_option(_native.OPT_MQ_BLOCKS_PER_WARP, 33)
    with pytest.raises(jl.InvalidInput):
        eng.set_option(_native.OPT_WAVE_BLOCKS, 0)
    with pytest.raises(jl.InvalidInput):
        eng.set_option(99, 1)


def test_submit_poll_matches_single(eng):
    pages = _mix(16, 5)
    tickets = [eng.submit(p) for p in pages]
    results = {t: eng.poll(t) for t in reversed(tickets)}
    for p, t in zip(pages, tickets):
        assert results[t] == _single(eng, p)


def test_submit_from_threads_in_any_order(eng):
    pages = _mix(20, 6)
    ref = [_single(eng, p) for p in pages]
    got = [None] * len(pages)

    def client(idx):
        rng = random.Random(idx)
        mine = list(range(idx, len(pages), 4))
        tickets = []
        for i in mine:
            tickets.append((i, eng.submit(pages[i])))
            if rng.random() < 0.5:
                threading.Event().wait(0.001 * rng.random())
        rng.shuffle(tickets)
        for i, t in tickets:
            r = None
            while r is None:
                r = eng.poll(t, 50)
            got[i] = r

    th = [threading.Thread(target=client, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert got == ref


def test_submit_rejects_invalid_before_queueing(eng):
    with pytest.raises(jl.InvalidInput):
        eng.submit({"px": np.zeros(4, np.uint8), "w": 2, "h": 1, "ncomp": 2, "quality": 85, "fmt": 0})
    with pytest.raises(jl.InvalidInput):
        eng.poll(123456789, 0)


def test_server_and_batch_encoder_api(eng):
    imgs = [jl.Image.from_gray_bytes(97, 61, synth_page(97, 61, 1, s).tobytes()) for s in range(3)]
    opts = jl.EncodeOptions(85, jl.OutputFormat.JP2)
    ref = [jl.encode(im, opts, eng) for im in imgs]
    assert jl.BatchEncoder(opts, eng).encode_all(imgs) == ref
    srv = jl.Server(eng)
    tickets = [srv.submit(im, opts) for im in imgs]
    assert [srv.result(t) for t in tickets] == ref
    enc = jl.BatchEncoder(opts, eng)
    other = jl.Image.from_gray_bytes(61, 97, synth_page(61, 97, 1, 9).tobytes())
    with pytest.raises(jl.InvalidInput):
        enc.encode_all([imgs[0], imgs[1], other])
    assert enc.encoded_count() == 2


@pytest.mark.parametrize("wps,pipes,heavy,chains", [(-1, 0, 0, 0), (1, -1, 0, 0), (8, -1, 0, 0), (64, -1, 0, 0),
                                                    (0, 1, 0, 0), (0, 4, 0, 0), (0, 32, 0, 0), (0, 4, 1, 0),
                                                    (0, 2, 37, 0), (0, 1, 0, 2), (0, 8, 0, 2), (0, 32, 0, 2),
                                                    (0, 4, 3, 2), (0, 2, 37, 2), (0, 8, 0, 4), (0, 2, 37, 4)])
@pytest.mark.parametrize("q", [85, 100, 20])
def test_mq_schedules_do_not_change_output(eng, orc, wps, pipes, heavy, chains, q):
    # static warps, single-warp pulling, producer/consumer pipelines with one
    # or two chains per pair, and pipelines for the heaviest blocks with the
    # rest packed 32 to a warp
    w, h = 600, 500
    px = synth_page(w, h, 1, 91, photo_w=200, photo_h=150)
    opts = (_native.OPT_MQ_WARPS_PER_SM, _native.OPT_MQ_PIPES_PER_SM, _native.OPT_MQ_HEAVY,
            _native.OPT_MQ_CHAINS_PER_PAIR)
    old = [eng.get_option(o) for o in opts]
    try:
        for o, v in zip(opts, (wps, pipes, heavy, chains)):
            eng.set_option(o, v)
        assert eng.encode(px, w, h, 1, q, 1) == orc.encode(px, w, h, 1, q, 1)
    finally:
        for o, v in zip(opts, old):
            eng.set_option(o, v)


def test_autotune_keeps_output_and_leaves_its_choice_set(eng):
    pages = _mix(8, 8, big=True)
    ref = eng.encode_batch(pages)
    opts = list(range(_native.NUM_OPTS))
    old = [eng.get_option(o) for o in opts]
    try:
        best, ms = eng.autotune(pages, repeats=1)
        assert ms > 0
        assert [eng.get_option(o) for o in opts] == [best[o] for o in opts]
        assert 0 <= best[_native.OPT_MQ_BLOCKS_PER_WARP] <= 32
        assert best[_native.OPT_WAVE_BLOCKS] in (old[0], 20000, 40000, 80000, 160000, 240000)
        assert best[_native.OPT_HOST_THREADS] == old[_native.OPT_HOST_THREADS]
        assert eng.encode_batch(pages) == ref
    finally:
        for o, v in zip(opts, old):
            eng.set_option(o, v)


def test_autotune_rejects_an_empty_sample(eng):
    with pytest.raises(jl.InvalidInput):
        eng.autotune([], repeats=1)
    with pytest.raises(jl.InvalidInput):
        eng.autotune(_mix(1, 9), repeats=0)


def test_wave_size_is_capped_to_addressable_payload_slots(eng):
    # 40 sRGB 2550x3300 pages hold 252,840 64x64 code-blocks: more than one
    # wave can address, so a larger wave-size option still splits them
    pages = [{"px": synth_page(2550, 3300, 3, 1000 + i, photo_w=800, photo_h=600), "w": 2550, "h": 3300,
              "ncomp": 3, "quality": 75, "fmt": 1} for i in range(40)]
    ref = eng.encode_batch(pages[:2])
    old = eng.get_option(_native.OPT_WAVE_BLOCKS)
    try:
        eng.set_option(_native.OPT_WAVE_BLOCKS, 10 ** 9)
        outs = eng.encode_batch(pages)
    finally:
        eng.set_option(_native.OPT_WAVE_BLOCKS, old)
    assert all(isinstance(o, bytes) for o in outs)
    assert outs[:2] == ref


@pytest.mark.parametrize("chains", [1, 2, 4])
def test_pipelines_with_many_blocks_per_chain_are_deterministic(eng, chains):
    # a wave of ~12k code-blocks forced through the pipelines: every chain
    # codes several blocks in turn; repeated encodes and one chain per pair
    # must give the same bytes
    pages = [{"px": synth_page(1275, 1650, 3 if i % 2 else 1, 7000 + i, photo_w=400, photo_h=300),
              "w": 1275, "h": 1650, "ncomp": 3 if i % 2 else 1, "quality": (85, 50, 100)[i % 3], "fmt": 1}
             for i in range(12)]
    opts = (_native.OPT_MQ_BLOCKS_PER_WARP, _native.OPT_MQ_PIPES_PER_SM, _native.OPT_MQ_CHAINS_PER_PAIR)
    old = [eng.get_option(o) for o in opts]
    try:
        for o, v in zip(opts, (1, 8, 1)):
            eng.set_option(o, v)
        ref = eng.encode_batch(pages)
        eng.set_option(_native.OPT_MQ_CHAINS_PER_PAIR, chains)
        for _ in range(4 if chains == 4 else 2):
            assert eng.encode_batch(pages) == ref
    finally:
        for o, v in zip(opts, old):
            eng.set_option(o, v)
    assert ref[0] == _single(eng, pages[0])
