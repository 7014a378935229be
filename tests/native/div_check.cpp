// The decoders' division by a constant (div_by in vship_gb300/csrc/common.cuh): product with the
// rounded reciprocal plus one FMA residual correction. Checks, for every numerator the decoders
// produce, that it equals IEEE division: n / 255 (8-bit), n / 65535 (16-bit), (Y - 64) / 876 for
// every 10-bit Y, (C - 512) / 896 for every 10-bit chroma value interpolated in sixteenths.
#include <cmath>
#include <cstdio>

template <int D>
static float div_by(float n) {
    const float d = (float)D, r = 1.0f / (float)D;
    const float q = n * r;
    return std::fma(std::fma(-q, d, n), r, q);
}

template <int D>
static int check(float n) {
    volatile float vn = n, vd = (float)D;
    const float ref = vn / vd;
    if (div_by<D>(n) != ref) {
        std::printf("mismatch n=%.9g D=%d\n", n, D);
        return 1;
    }
    return 0;
}

int main() {
    int bad = 0;
    for (int u = 0; u < 256; u++) bad += check<255>((float)u);
    for (int u = 0; u < 65536; u++) bad += check<65535>((float)u);
    for (int y = 0; y < 1024; y++) bad += check<876>((float)y - 64.f);
    for (int k = 0; k <= 1023 * 16; k++) bad += check<896>((float)k / 16.f - 512.f);
    std::printf(bad ? "FAIL %d\n" : "ok\n", bad);
    return bad ? 1 : 0;
}
