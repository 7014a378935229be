"""Failure paths, injected on the host (no GPU fault): allocation failure at init maps to
Vship_OutOfVRAM / Vship_OutOfRAM and leaves the library usable; a serving batch whose device
block cannot be allocated reports its requests as failed while later requests succeed (and
the sources it had put in the cache are dropped); queued serving requests can be withdrawn."""
import ctypes
import time

import numpy as np
import pytest
import torch

from vship_gb300 import synth

pytestmark = pytest.mark.gpu


def _init_ssimu2(vlib):
    h = vlib.Handler()
    rc = vlib.lib().Vship_SSIMU2Init(ctypes.byref(h), 64, 48)
    return rc, h


def test_device_allocation_failure_at_init(vlib, monkeypatch):
    L = vlib.lib()
    for n in (0, 1, 3):
        monkeypatch.setenv("VSHIP_FAIL_DEVICE_ALLOC_AFTER", str(n))
        rc, _ = _init_ssimu2(vlib)
        assert rc == vlib.OutOfVRAM, n
        h = vlib.Handler()
        assert L.Vship_ButteraugliInitv2(ctypes.byref(h), 64, 48, 2, ctypes.c_float(203.0)) == vlib.OutOfVRAM
        with pytest.raises(vlib.VshipError) as e:
            vlib.MultiScorer([(64, 48)], [1], [2], vlib.MULTI_SSIMU2 | vlib.MULTI_BUTTERAUGLI)
        assert e.value.code == vlib.OutOfVRAM
        monkeypatch.delenv("VSHIP_FAIL_DEVICE_ALLOC_AFTER")
    rc, h = _init_ssimu2(vlib)
    assert rc == 0
    assert L.Vship_SSIMU2Free(h) == 0


def test_pinned_allocation_failure(vlib, monkeypatch):
    L = vlib.lib()
    monkeypatch.setenv("VSHIP_FAIL_PINNED_ALLOC_AFTER", "0")
    p = ctypes.c_void_p()
    assert L.Vship_PinnedMalloc(ctypes.byref(p), 4096) == vlib.OutOfRAM
    rc, _ = _init_ssimu2(vlib)  # the host path's pinned result slot
    assert rc == vlib.OutOfRAM
    monkeypatch.delenv("VSHIP_FAIL_PINNED_ALLOC_AFTER")
    assert L.Vship_PinnedMalloc(ctypes.byref(p), 4096) == 0
    assert L.Vship_PinnedFree(p) == 0


def _frames(keep, w, h, n):
    src = synth.yuv420p10_source(h, w, 0, 21)
    t = [torch.from_numpy(np.asarray(p, dtype=np.int32)).to(torch.int16).cuda() for p in src]
    keep.append(t)
    sfd = ([x.data_ptr() for x in t], t[0].stride(0) * 2, t[1].stride(0) * 2)
    cands = []
    for k in range(n):
        c = [synth.block_dct_quantise(p, 4 + 4 * k, 64, 960) for p in src]
        tc = [torch.from_numpy(np.asarray(p, dtype=np.int32)).to(torch.int16).cuda() for p in c]
        keep.append(tc)
        cands.append(([x.data_ptr() for x in tc], tc[0].stride(0) * 2, tc[1].stride(0) * 2))
    return sfd, cands


def _wait(srv, n, timeout=60):
    done = {}
    t0 = time.time()
    while len(done) < n and time.time() - t0 < timeout:
        for rid, st, lat in srv.poll(64, 0.5):
            done[rid] = st
    return done


def test_serving_batch_allocation_failure(vlib, monkeypatch):
    keep = []
    w, h = 128, 96
    src, cands = _frames(keep, w, h, 3)
    srv = vlib.Server([(w, h)], vlib.IN_YUV, admission_bytes=1 << 30, cache_bytes=1 << 28)
    good = np.zeros(3)
    srv.submit(1, 0, 0, 7, src, cands, good)
    srv.drain()
    assert _wait(srv, 1) == {1: 0}
    monkeypatch.setenv("VSHIP_FAIL_DEVICE_ALLOC_AFTER", "0")
    bad = np.zeros(3)
    srv.submit(2, 0, 0, 8, src, cands, bad)  # source 8 is new: its cache entry must be dropped
    srv.drain()
    st = _wait(srv, 1)
    assert st[2] == vlib.OutOfVRAM
    monkeypatch.delenv("VSHIP_FAIL_DEVICE_ALLOC_AFTER")
    again = np.zeros(3)
    srv.submit(3, 0, 0, 8, src, cands, again)
    srv.drain()
    assert _wait(srv, 1) == {3: 0}
    stats = srv.stats()
    srv.free()
    assert again.tolist() == good.tolist()
    assert stats["failed"] == 1 and stats["completed"] == 3


def test_serving_cancel_queued(vlib):
    keep = []
    w, h = 256, 144
    src, cands = _frames(keep, w, h, 4)
    # admission for one 4-pair Butteraugli request at a time: the rest wait in the queue
    srv = vlib.Server([(w, h)], vlib.IN_YUV, admission_bytes=124 * w * h * 4, cache_bytes=0, max_batch_pairs=4)
    outs = {}
    for i in range(12):
        outs[i] = np.zeros(12)
        srv.submit(i, 1, 0, 0, src, cands, outs[i])
    cancelled = [i for i in range(11, 3, -1) if srv.cancel(i)]
    assert not srv.cancel(1000)
    srv.drain()
    st = _wait(srv, 12)
    srv.free()
    assert len(st) == 12 and cancelled
    for i, s in st.items():
        assert s == (vlib.SERVE_CANCELLED if i in cancelled else 0), (i, s)
    first = outs[0].tolist()
    for i in range(12):
        if i not in cancelled:
            assert outs[i].tolist() == first
