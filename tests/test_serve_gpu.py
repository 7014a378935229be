"""Serving runtime (Vship_Serve*): each request's results are identical alone and inside a mix
(cache hits, uncached sources, both metrics, two resolutions, admission waits, evictions), and
equal the batched multi-resolution path's on the same pairs (SSIMULACRA2 with FP16-delta
candidates, Butteraugli)."""
import time

import numpy as np
import pytest
import torch

from vship_gb300 import synth

pytestmark = pytest.mark.gpu

RES = [(256, 144), (131, 75)]
STEPS = [4, 8, 16, 26, 32]


def _dev(frame, keep):
    t = [torch.from_numpy(np.asarray(p, dtype=np.int32)).to(torch.int16).cuda() for p in frame]
    keep.append(t)
    return ([x.data_ptr() for x in t], t[0].stride(0) * 2, t[1].stride(0) * 2)


def _pool(keep, nsrc=3):
    """Per resolution: nsrc sources, each with 5 DCT candidates, as device frames."""
    pool = {}
    for r, (w, h) in enumerate(RES):
        for k in range(nsrc):
            src = synth.yuv420p10_source(h, w, k, 40 + r)
            cands = []
            for st in STEPS:
                c = (synth.block_dct_quantise(src[0], st, 64, 940), synth.block_dct_quantise(src[1], 2 * st, 64, 960),
                     synth.block_dct_quantise(src[2], 2 * st, 64, 960))
                cands.append(_dev(c, keep))
            pool[(r, k)] = (_dev(src, keep), cands)
    return pool


def _requests():
    """(id, metric, res, key, source index, candidate indices): repeated sources, key 0."""
    return [
        (1, 0, 0, 101, 0, [0, 1, 2]),
        (2, 1, 0, 201, 1, [1, 3]),
        (3, 0, 1, 301, 0, [4]),
        (4, 0, 0, 101, 0, [3, 4]),      # cache hit of request 1's source
        (5, 1, 1, 0, 2, [0, 1, 2]),     # never cached
        (6, 1, 0, 201, 1, [0]),         # cache hit of request 2's source
        (7, 0, 0, 102, 2, [0, 2, 4]),
        (8, 1, 1, 401, 1, [2, 3, 4]),
        (9, 0, 1, 0, 2, [0, 1]),
        (10, 0, 0, 101, 0, [0, 1, 2]),  # same pairs as request 1
    ]


def _run(vlib, pool, reqs, **kw):
    srv = vlib.Server(RES, vlib.IN_YUV420P10, **kw)
    outs = {}
    for rid, metric, res, key, si, ci in reqs:
        src, cands = pool[(res, si)]
        out = np.zeros(len(ci) * (1 if metric == 0 else 3))
        srv.submit(rid, metric, res, key, src, [cands[j] for j in ci], out)
        outs[rid] = out
    done = {}
    t0 = time.time()
    while len(done) < len(reqs) and time.time() - t0 < 60:
        for rid, status, lat in srv.poll(64, 1.0):
            done[rid] = (status, lat)
    stats = srv.stats()
    srv.free()
    assert len(done) == len(reqs)
    assert all(s == 0 and lat > 0 for s, lat in done.values()), done
    return {k: v.tolist() for k, v in outs.items()}, stats


def test_serve_alone_equals_mix(vlib):
    keep = []
    pool = _pool(keep)
    reqs = _requests()
    mix, stats = _run(vlib, pool, reqs)
    assert stats["cache_hits"] >= 3 and stats["completed"] == len(reqs)
    for q in reqs:
        alone, _ = _run(vlib, pool, [q])
        assert alone[q[0]] == mix[q[0]], q
    assert mix[1] == mix[10]


def test_serve_matches_multi(vlib):
    keep = []
    pool = _pool(keep, nsrc=2)
    reqs = [(1, 0, 0, 7, 0, [0, 1, 2, 3, 4]), (2, 1, 0, 8, 1, [0, 2, 4]), (3, 0, 1, 9, 1, [1, 3])]
    got, _ = _run(vlib, pool, reqs)
    for rid, metric, res, key, si, ci in reqs:
        src, cands = pool[(res, si)]
        flags = vlib.MULTI_FP16 | (vlib.MULTI_SSIMU2 if metric == 0 else vlib.MULTI_BUTTERAUGLI)
        ms = [1 if r == res else 0 for r in range(len(RES))]
        mp = [len(ci) if r == res else 0 for r in range(len(RES))]
        sc = vlib.MultiScorer(RES, ms, mp, flags)
        s2 = torch.zeros(len(ci), dtype=torch.float64, device="cuda")
        bn = torch.zeros(3 * len(ci), dtype=torch.float64, device="cuda")
        sc.compute_async([src], [res], [cands[j] for j in ci], [0] * len(ci), vlib.IN_YUV420P10,
                         s2.data_ptr() if metric == 0 else 0, bn.data_ptr() if metric == 1 else 0,
                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        sc.free()
        want = (s2 if metric == 0 else bn).cpu().tolist()
        assert got[rid] == want, (rid, got[rid], want)


def test_serve_admission_and_eviction(vlib):
    keep = []
    pool = _pool(keep)
    reqs = _requests()
    mix, _ = _run(vlib, pool, reqs)
    w, h = RES[0]
    # room for one 3-pair Butteraugli request at the larger size at a time; a cache a little
    # larger than one Butteraugli source at that size (2.9 MB), far below the stream's sources
    tight, stats = _run(vlib, pool, reqs, admission_bytes=124 * w * h * 3, cache_bytes=3_500_000,
                        max_batch_pairs=4)
    assert tight == mix
    assert stats["admission_waits"] > 0 and stats["cache_evictions"] > 0
    assert stats["admission_peak_bytes"] <= 124 * w * h * 3
    assert stats["max_batch_pairs"] <= 4


def test_serve_rejects_oversized(vlib):
    keep = []
    pool = _pool(keep, nsrc=1)
    w, h = RES[0]
    srv = vlib.Server(RES, vlib.IN_YUV420P10, admission_bytes=48 * w * h * 2)
    src, cands = pool[(0, 0)]
    with pytest.raises(vlib.VshipError):
        srv.submit(1, 0, 0, 5, src, cands[:3], np.zeros(3))
    out = np.zeros(2)
    srv.submit(2, 0, 0, 5, src, cands[:2], out)
    srv.drain()
    assert [c[0] for c in srv.poll()] == [2] and all(0 < s <= 100 for s in out)
    srv.free()


def test_serve_yuv_format_is_fixed_after_first_submit(vlib):
    # cached source state is keyed by source, not by format: a format change after a submit
    # would score later candidates against sources decoded under the old format
    keep = []
    pool = _pool(keep, nsrc=1)
    srv = vlib.Server(RES, vlib.IN_YUV420P10)
    srv.set_yuv_format(vlib.yuv_format(bits=10))  # before any submit: accepted
    src, cands = pool[(0, 0)]
    out = np.zeros(2)
    srv.submit(1, 0, 0, 5, src, cands[:2], out)
    with pytest.raises(vlib.VshipError) as e:
        srv.set_yuv_format(vlib.yuv_format(bits=10, full_range=True))
    assert e.value.code == vlib.BadPointer
    srv.drain()
    assert [c[0] for c in srv.poll()] == [1] and all(0 < s <= 100 for s in out)
    srv.free()
