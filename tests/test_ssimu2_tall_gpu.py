"""SSIMULACRA2 launches of many pairs (16 or more) tile the stats kernel in taller segments (576
rows on the levels that keep at least 24 of them per frame) than single-pair calls (192 rows).
Only the order of the FP32 pooled partial sums differs, so the scores agree to that rounding:
within 1e-5 of the per-pair scores here, and within the SSIMULACRA2 tolerance of the FP64 oracle.
The 800x200 frames put 25 segment columns on the full-resolution level, so the tall tiling is
in use there.
"""
import numpy as np
import pytest
import torch

from helpers import grating_float_pair

pytestmark = pytest.mark.gpu

W, H, N = 800, 200, 16


def test_tall_segments_match_per_pair(vlib, orc):
    pairs = [grating_float_pair(H, W, t=t, distortion="dct" if t % 2 else "blur_noise") for t in range(N)]
    with vlib.SSIMU2Handler(W, H) as hd:
        want = [hd.compute(a, b) for a, b in pairs]
    dev = [(torch.from_numpy(np.stack(a)).cuda(), torch.from_numpy(np.stack(b)).cuda()) for a, b in pairs]
    frames = []
    for ta, tb in dev:
        for t in (ta, tb):
            frames.append(([t[c].data_ptr() for c in range(3)], t.stride(1) * 4))
    table = vlib.device_frames_table(frames)
    out = torch.zeros(N, dtype=torch.float64, device="cuda")
    bt = vlib.SSIMU2Batch(W, H, N)
    bt.compute_async(table.data_ptr(), N, vlib.IN_FLOAT, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    bt.free()
    got = out.cpu().tolist()
    assert max(abs(g - w) for g, w in zip(got, want)) <= 1e-5, (got, want)
    exact = orc.ssimu2(*pairs[1], precision=64)
    assert abs(got[1] - exact) <= 1e-3, (got[1], exact)
