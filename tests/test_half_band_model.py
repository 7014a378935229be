"""Which Butteraugli bands may be stored as FP16, checked in the oracle's model of that storage
(CPU only; oracle/oracle.cpp store_bands_half).

The FP16 form (Vship_ButterHalfBands) keeps only the UHF bands as FP16 (oracle precision 19).
On the frames that decided it, that model stays within the path's 1e-4 relative of FP64 on all
three norms, while FP16 storage of every band (precision 16) misses it by an order of magnitude:
the MF and HF bands' rounding moves the Malta maps' squared line sums.
"""
import pytest

from helpers import grating_float_pair

FRAMES = [(270, 480, "dct", 5), (131, 257, "dct", 2), (131, 257, "blur_noise", 2)]


@pytest.mark.parametrize("h,w,distortion,t", FRAMES)
def test_uhf_only_half_storage_within_tolerance(orc, h, w, distortion, t):
    a, b = grating_float_pair(h, w, t=t, distortion=distortion)
    exact = orc.butteraugli(a, b, precision=64)
    model = orc.butteraugli(a, b, precision=19)
    rel = [abs(m - e) / abs(e) for m, e in zip(model, exact)]
    assert max(rel) <= 1e-4, rel


def test_every_band_half_misses_tolerance(orc):
    a, b = grating_float_pair(270, 480, t=5, distortion="dct")
    exact = orc.butteraugli(a, b, precision=64)
    model = orc.butteraugli(a, b, precision=16)
    rel = [abs(m - e) / abs(e) for m, e in zip(model, exact)]
    assert rel[0] > 1e-3, rel
