// ssimu2.cu -- SSIMULACRA2 scoring on sm_103a.
//
// Three kernels per launch, all batched over frame pairs:
//   1. ssimu2_pyramid  : decode + x^2.4 linearisation + the 6-level 2x2 box pyramid + positive
//                        XYB, one 32x32 level-0 tile per CTA with every coarser level computed
//                        from shared memory (the pyramid is tile-local: a 2^k-aligned level-0
//                        tile maps exactly onto its level-k tile, edge clamp included).
//                        Reference: ssimu2/main.hpp:15-32, makeXYB.hpp:4-98, downsample.hpp:3-31.
//   2. ssimu2_stats    : all six scales in one launch. Per 32-column segment (576 or 192 rows),
//                        in 64- or 48-row chunks, it stages I1 and I2 (8-px halo, zero outside)
//                        in shared memory, runs the 17-tap separable Gaussian (border-
//                        renormalised) for four moments (mu1, mu2, E[(I1 - I2)^2], E[I1 I2]) with
//                        register blocking and a carry buffer or a ring of
//                        horizontal-pass rows, forms the SSIM / artifact / detail-loss maps and
//                        emits 18 partial sums (6 pools x 3 channels) per CTA.
//                        Reference: ssimu2/score.hpp:95-196, gaussianblur.hpp:24-92.
//   3. ssimu2_finalize : combine of the partial sums (float-float), then in FP64 the means, 4th
//                        roots, the 108-feature permutation, weighted sum and score mapping
//                        (score.hpp:198-401, main.hpp:83-98).
#include "common.cuh"
#include "ssimu2.h"
#include "profile.h"

#include <cmath>
#include <vector>

namespace vship {

// ------------------------------------------------------------------------------------------
// Gaussian table (sigma 1.5, radius 8): taps k and prefix integral I, built on the host exactly
// as ssimu2/gaussianblur.hpp:7-18 builds them. The stats kernels blur with the taps divided by
// the kernel's total mass K = I[17] - I[0] ({k/K, k/K} pairs for the f32x2 FMA), so that a window
// inside the image needs no renormalisation; a window that a border cuts (beg in 0..8 taps cut
// on one side, end in 9..17) is multiplied by K / (I[end] - I[beg]), its inverse in-bounds mass
// relative to K, from a table rather than by a division (exactly 1 for an uncut window).
__constant__ f2_t c_s2_k2n[17];
__constant__ float c_s2_invmn[9][9];
// SSIMULACRA2 feature weights (ssimu2/score.hpp:272-379), FP64.
__constant__ double c_s2_w[108];

static const double kSsimu2Weights[108] = {
    0.0, 0.0007376606707406586, 0.0, 0.0, 0.0007793481682867309, 0.0,
    0.0, 0.0004371155730107379, 0.0, 1.1041726426657346, 0.00066284834129271, 0.00015231632783718752,
    0.0, 0.0016406437456599754, 0.0, 1.8422455520539298, 11.441172603757666, 0.0,
    0.0007989109436015163, 0.000176816438078653, 0.0, 1.8787594979546387, 10.94906990605142, 0.0,
    0.0007289346991508072, 0.9677937080626833, 0.0, 0.00014003424285435884, 0.9981766977854967, 0.00031949755934435053,
    0.0004550992113792063, 0.0, 0.0, 0.0013648766163243398, 0.0, 0.0,
    0.0, 0.0, 0.0, 7.466890328078848, 0.0, 17.445833984131262,
    0.0006235601634041466, 0.0, 0.0, 6.683678146179332, 0.00037724407979611296, 1.027889937768264,
    225.20515300849274, 0.0, 0.0, 19.213238186143016, 0.0011401524586618361, 0.001237755635509985,
    176.39317598450694, 0.0, 0.0, 24.43300999870476, 0.28520802612117757, 0.0004485436923833408,
    0.0, 0.0, 0.0, 34.77906344483772, 44.835625328877896, 0.0,
    0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
    0.0, 0.0008680556573291698, 0.0, 0.0, 0.0, 0.0,
    0.0, 0.0005313191874358747, 0.0, 0.00016533814161379112, 0.0, 0.0,
    0.0, 0.0, 0.0, 0.0004179171803251336, 0.0017290828234722833, 0.0,
    0.0020827005846636437, 0.0, 0.0, 8.826982764996862, 23.19243343998926, 0.0,
    95.1080498811086, 0.9863978034400682, 0.9834382792465353, 0.0012286405048278493, 171.2667255897307, 0.9807858872435379,
    0.0, 0.0, 0.0, 0.0005130064588990679, 0.0, 0.00010854057858411537,
};

static int upload_constants_once() {
    // Constant memory is per device; the tables are uploaded on every engine init (cheap).
    float k[17], I[18];
    const float sigma = 1.5f;
    I[0] = 0.f;
    for (int i = 0; i < 17; i++) {
        float e = std::exp((float)(-(8 - i) * (8 - i)) / (2 * sigma * sigma));
        k[i] = (float)((double)e / std::sqrt(6.28318530718 * sigma * sigma));
        I[i + 1] = I[i] + k[i];
    }
    const float K = I[17] - I[0];
    float k2n[34], invmn[9][9];
    for (int i = 0; i < 17; i++) k2n[2 * i] = k2n[2 * i + 1] = k[i] / K;
    for (int b = 0; b < 9; b++)
        for (int e = 0; e < 9; e++) invmn[b][e] = K / (I[9 + e] - I[b]);
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_s2_k2n, k2n, sizeof(k2n)));
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_s2_invmn, invmn, sizeof(invmn)));
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_s2_w, kSsimu2Weights, sizeof(kSsimu2Weights)));
    return E_OK;
}

// ------------------------------------------------------------------------------------------
// XYB (ssimu2/makeXYB.hpp:4-50) as the metric sees it. The reference adds positive offsets at the
// end (X * 14 + 0.42, Y + 0.01, B - Y + 0.55); every SSIMULACRA2 map is invariant under one
// constant added to a channel of both images (the means' difference, the variances, the
// covariance and |I - mu| all cancel it), so these planes hold X * 14, Y - 0.4 and B - Y instead,
// three adds fewer per sample and level (the offsets are double constants, each an add pair in
// FP32). The stats kernel still shifts each segment's samples by one of its own values: that
// keeps flat areas and frames of a few pixels exact, where a blur's border renormalisation leaves
// a few ulps of x^2 in E[x^2] - E[x]^2.
__device__ __forceinline__ void centred_xyb(float& r, float& g, float& b) {
    const float bias = 0.0037930734f;
    float ox = fmaf(0.30f, r, fmaf(0.622f, g, fmaf(0.078f, b, bias)));
    float oy = fmaf(0.23f, r, fmaf(0.692f, g, fmaf(0.078f, b, bias)));
    float oz = fmaf(0.24342269f, r, fmaf(0.20476745f, g, fmaf(0.55180986f, b, bias)));
    const float abs_bias = -0.1559542025327239f;
    ox = cbrt_pos(fmaxf(ox, 0.f)) + abs_bias;
    oy = cbrt_pos(fmaxf(oy, 0.f)) + abs_bias;
    oz = cbrt_pos(fmaxf(oz, 0.f)) + abs_bias;
    float X = 0.5f * (ox - oy);
    float Y = X + oy;
    float B = oz;
    r = X * 14.0f;
    g = Y - 0.4f;
    b = B - Y;
}

// ------------------------------------------------------------------------------------------
// Kernel 1: decode + linearise + pyramid + XYB, one 32x32 level-0 tile per CTA (256 threads).
// A pyramid is written either as FP32 planes, or (DELTA) as FP16 differences against an FP32
// reference pyramid of the same geometry: the batched form keeps each source's pyramid in FP32
// and its candidates' as FP16 deltas (identical samples stay exactly identical, small
// distortions keep FP16's relative precision).
struct PyrOut {
    float* f32;         // FP32 planes [3][plane_elems]
    __half* d16;        // FP16 delta planes [3][plane_elems]
    const float* ref;   // reference FP32 planes for the deltas
};

template <bool DELTA>
__device__ __forceinline__ void pyr_store(const PyrOut& out, int64_t pe, int64_t o, float X, float Y, float B) {
    if (DELTA) {
        out.d16[o] = __float2half_rn(X - __ldg(out.ref + o));
        out.d16[pe + o] = __float2half_rn(Y - __ldg(out.ref + pe + o));
        out.d16[2 * pe + o] = __float2half_rn(B - __ldg(out.ref + 2 * pe + o));
    } else {
        out.f32[o] = X;
        out.f32[pe + o] = Y;
        out.f32[2 * pe + o] = B;
    }
}

// One kPyrTile x kPyrTile (32 x 32) level-0 tile per CTA, levels 1..5 from shared memory.
template <int IT, bool DELTA>
__device__ __forceinline__ void pyramid_tile(const FrameDesc& fd, const YuvParams& yp, const PyrOut& out,
                                             const Ssimu2Geom& g, int bx, int by) {
    __shared__ float smA[3 * 32 * 33];
    __shared__ float smB[3 * 16 * 17];
    const int64_t pe = g.plane_elems;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    // Level 0 four pixels per thread (4 consecutive columns of one row): R'G'B' planes whose rows
    // allow it load them with one vector load per plane (8 bytes of uint16, 16 of float), Y'CbCr
    // loads each chroma sample once for the four (yuv_rgb4); FP32 pyramids store the 4 outputs
    // per channel as one float4 (level rows are 16-byte aligned, columns a multiple of 4).
    const bool vec = rgb4_vectorizable<IT>(fd);
    if (IT == IN_YUV || vec) {
        const Ssimu2Level L = g.lv[0];
        const int ly = threadIdx.x >> 3, lx = 4 * (threadIdx.x & 7);
        const int gx = bx * 32 + lx, gy = by * 32 + ly;
        float v[3][4] = {};
        if (gy < L.h && gx < L.w) {
            load_rgb4<IT>(fd, yp, gx, gy, L.w, L.h, vec, v);
            float o[3][4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float lin = (IT == IN_YUV && yp.linear_out) ? v[c][i] : to_linear_fast<IT>(v[c][i]);
                    v[c][i] = gx + i < L.w ? lin : 0.f;  // frames converted to linear light skip x^2.4
                }
                float X = v[0][i], Y = v[1][i], B = v[2][i];
                centred_xyb(X, Y, B);
                o[0][i] = X;
                o[1][i] = Y;
                o[2][i] = B;
            }
            const int64_t e = L.off + (int64_t)gy * L.pitch + gx;
            if (!DELTA && gx + 3 < L.w) {
#pragma unroll
                for (int c = 0; c < 3; c++)
                    *reinterpret_cast<float4*>(out.f32 + c * pe + e) = make_float4(o[c][0], o[c][1], o[c][2], o[c][3]);
            } else if (DELTA && gx + 3 < L.w) {
                // four deltas per channel: one 16-byte load of the reference, one 8-byte store
                // (e is a multiple of 4 elements)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float4 r = __ldg(reinterpret_cast<const float4*>(out.ref + c * pe + e));
                    const __half2 lo = __floats2half2_rn(o[c][0] - r.x, o[c][1] - r.y);
                    const __half2 hi = __floats2half2_rn(o[c][2] - r.z, o[c][3] - r.w);
                    uint2 u;
                    u.x = *reinterpret_cast<const unsigned*>(&lo);
                    u.y = *reinterpret_cast<const unsigned*>(&hi);
                    *reinterpret_cast<uint2*>(out.d16 + c * pe + e) = u;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++)
                    if (gx + i < L.w) pyr_store<DELTA>(out, pe, e + i, o[0][i], o[1][i], o[2][i]);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int i = 0; i < 4; i++) smA[(c * 32 + ly) * 33 + lx + i] = v[c][i];
    } else {
        const Ssimu2Level L = g.lv[0];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int ly = ty + 8 * r;
            const int gx = bx * 32 + tx, gy = by * 32 + ly;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f;
            if (gx < L.w && gy < L.h) {
                load_rgb<IT>(fd, yp, gx, gy, L.w, L.h, v0, v1, v2);
                if (!(IT == IN_YUV && yp.linear_out)) {  // frames converted to linear light skip x^2.4
                    v0 = to_linear_fast<IT>(v0);
                    v1 = to_linear_fast<IT>(v1);
                    v2 = to_linear_fast<IT>(v2);
                }
                float X = v0, Y = v1, B = v2;
                centred_xyb(X, Y, B);
                pyr_store<DELTA>(out, pe, L.off + (int64_t)gy * L.pitch + gx, X, Y, B);
            }
            smA[(0 * 32 + ly) * 33 + tx] = v0;
            smA[(1 * 32 + ly) * 33 + tx] = v1;
            smA[(2 * 32 + ly) * 33 + tx] = v2;
        }
    }
    __syncthreads();
    float* cur = smA;
    float* nxt = smB;
    // levels 1..5: the tile side halves each level (16, 8, 4, 2, 1), so indices are shifts.
    // Level 1 (256 samples) takes every thread; levels 2..5 (85 samples) are warp 0's alone,
    // ordered by warp barriers, so the other seven warps leave and free their slots.
    auto level = [&](int k, int nthreads) {
        const int cside = 32 >> (k - 1), nside = 32 >> k, lg = 5 - k;
        const Ssimu2Level L = g.lv[k], P = g.lv[k - 1];
        const int ox = bx * nside, oy = by * nside;
        const int pox = bx * cside, poy = by * cside;
        for (int i = threadIdx.x; i < nside * nside; i += nthreads) {
            const int lx = i & (nside - 1), ly = i >> lg;
            const int gx = ox + lx, gy = oy + ly;
            float v[3] = {0.f, 0.f, 0.f};
            if (gx < L.w && gy < L.h) {
                const int x0 = 2 * lx, y0 = 2 * ly;
                const int x1 = min(2 * gx + 1, P.w - 1) - pox;
                const int y1 = min(2 * gy + 1, P.h - 1) - poy;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float* cb = cur + c * cside * (cside + 1);
                    float s = cb[y0 * (cside + 1) + x0];
                    s += cb[y1 * (cside + 1) + x0];
                    s += cb[y0 * (cside + 1) + x1];
                    s += cb[y1 * (cside + 1) + x1];
                    v[c] = s * 0.25f;
                }
                float X = v[0], Y = v[1], B = v[2];
                centred_xyb(X, Y, B);
                pyr_store<DELTA>(out, pe, L.off + (int64_t)gy * L.pitch + gx, X, Y, B);
            }
#pragma unroll
            for (int c = 0; c < 3; c++) nxt[c * nside * (nside + 1) + ly * (nside + 1) + lx] = v[c];
        }
        float* t = cur;
        cur = nxt;
        nxt = t;
    };
    level(1, 256);
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 2; k < 6; k++) {
            level(k, 32);
            __syncwarp();
        }
    }
}

// grid (tiles_x0, tiles_y0, 2*npairs)
template <int IT>
__global__ void __launch_bounds__(256, IT == IN_YUV ? 6 : 8) ssimu2_pyramid_kernel(const FrameDesc* __restrict__ frames,
                                                             float* __restrict__ pyr, Ssimu2Geom g, YuvParams yp) {
    const int img = blockIdx.z;  // pair*2 + image
    const FrameDesc fd = frames[img];
    PyrOut out{pyr + (int64_t)img * 3 * g.plane_elems, nullptr, nullptr};
    pyramid_tile<IT, false>(fd, yp, out, g, blockIdx.x, blockIdx.y);
}

// FP16-delta form of the per-pair engine: grid (tiles_x0, tiles_y0, npairs). Without DELTA each
// pair's reference image writes FP32 planes into ref[pair]; with DELTA (a second launch, after
// the first) its distorted image writes half(distorted - reference) into d16[pair]. Two launches
// rather than one CTA building both tiles: the single-tile kernel keeps 8 CTAs per SM and its
// warps leave while warp 0 builds the small levels; a CTA building both tiles back to back (the
// distorted tile reading the reference's values from shared memory) took 31.2 ms against 26.3 ms
// for the two launches, per 10 launches of 120 pairs at 1920x1080.
template <int IT, bool DELTA>
__global__ void __launch_bounds__(256, IT == IN_YUV ? 6 : 8) ssimu2_pyramid_pair_kernel(
    const FrameDesc* __restrict__ frames, float* __restrict__ ref, __half* __restrict__ d16, Ssimu2Geom g,
    YuvParams yp) {
    const int pair = blockIdx.z;
    const FrameDesc fd = frames[2 * pair + (DELTA ? 1 : 0)];
    const int64_t o = (int64_t)pair * 3 * g.plane_elems;
    PyrOut out{DELTA ? nullptr : ref + o, DELTA ? d16 + o : nullptr, DELTA ? ref + o : nullptr};
    pyramid_tile<IT, DELTA>(fd, yp, out, g, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------------------------------------
// Kernel 2: fused moment blur + SSIM/edge maps + per-CTA pooling, all scales in one launch.
// grid (tiles_total, npairs), 256 threads, dynamic smem kStatsSmem, three CTAs per SM.
//
// Per CTA: one segment of one scale -- a 32-column strip, L.seg rows tall -- walked down in
// chunks of 48 output rows. For each channel and chunk the raw I1 and I2 rows (8-px halo) are
// staged with cp.async (bytes outside the image are zero-filled); one CTA's loads overlap the
// arithmetic of the other CTAs on its SM. The horizontal pass reads the raw rows as float4 (row
// pitch 52 floats: the 8 lanes of each quarter-warp phase hit distinct bank quads), forms the
// shifted samples and their products in registers and scatters them into 8 outputs x 4 moments,
// into a ring of horizontal-pass rows; the vertical pass gathers 22 ring rows per thread and
// evaluates the maps. The ring keeps the 16 rows a chunk shares with the next, so the vertical
// halo is blurred horizontally once per segment instead of once per chunk (64 instead of 48
// horizontal rows per 48 output rows).
constexpr int ST_TW = 32, ST_TH = 48, ST_R = 8;
// Segment heights (output rows). Each segment's first chunk blurs the 16 halo rows above it, so
// taller segments blur fewer rows twice. In a tall geometry (make_ssimu2_geom(w, h, true), for
// launches of many pairs) a level that still has at least kSegTallMin segments of ST_SEG_TALL
// rows per frame uses them (1080p: 3.0 % faster stats than 192 rows throughout, 576 measured best
// among 384, 576 and 768); other levels, and every level of the default geometry, keep ST_SEG
// rows, so that a small frame or a lone pair still spreads over enough CTAs.
constexpr int ST_SEG = 4 * ST_TH;
constexpr int ST_SEG_TALL = 12 * ST_TH;
constexpr int kSegTallMin = 24;
constexpr int ST_IW = ST_TW + 2 * ST_R;  // 48 input columns
constexpr int ST_IH = ST_TH + 2 * ST_R;  // 64 raw rows per chunk (image rows ty0 - 8 ..)
constexpr int ST_RP = 52;                // raw-tile row pitch (floats; 16-byte multiple, 13 quads)
constexpr int ST_RAW = ST_IH * ST_RP;    // one raw tile
constexpr int ST_RING = 64;              // ring slots (power of two): row h of a segment -> h & 63
constexpr int ST_WIN = ST_TH / 8 + 2 * ST_R;             // 22 ring rows per vertical window
constexpr int ST_HROWS = ST_RING + ST_WIN;               // slots [0, 22) mirrored at [64, 86)
// The ring is column-major: column x of a ring plane starts at float pair x * ST_HROWS + 8 * (x / 8)
// (the 8-pair gap between column groups makes a half-warp's 8-byte stores of two groups hit
// disjoint banks), so the vertical pass reads its 22 slots as 11 16-byte loads (43 quads per
// column, odd: 8 neighbouring columns hit distinct bank quads).
constexpr int ST_HPLANE = ST_TW * ST_HROWS + 8 * (ST_TW / 8 - 1);  // float pairs per ring plane
// smem: the 2 raw images, the ring as two float-pair planes {m1, m2} and {s11 + s22, s12}, and
// the per-warp pools: 70 KB, so that three CTAs share an SM
constexpr int kStatsSmem = (2 * ST_RAW + 4 * ST_HPLANE + 3 * 8 * 6) * 4;

__device__ __forceinline__ float s2_inv_mass(int pos, int extent) {
    // in-bounds kernel mass of a 17-tap window centred on pos, inverted and relative to the
    // whole kernel's (reference: out / tot); 1 for a window inside the image
    const int beg = max(0, pos - 8) - (pos - 8);
    const int end = min(extent, pos + 9) - (pos - 8);
    // positions past the edge (whose outputs are never pooled) are clamped onto the table
    return c_s2_invmn[beg][max(end - 9, 0)];
}

// Per-thread pooled sums of the three maps: (sum d0, sum d1) and (sum d0^4, sum d1^4) as f32x2
// pairs, sum d2 and sum d2^4; pool index map * 2 + norm.
struct S2Pools {
    f2_t s01, q01;
    float s2, q2;
};
__device__ __forceinline__ S2Pools s2_pools_zero() { return S2Pools{f2_pack(0.f, 0.f), f2_pack(0.f, 0.f), 0.f, 0.f}; }
__device__ __forceinline__ void s2_pools_unpack(const S2Pools& p, float* v) {
    f2_unpack(p.s01, v[0], v[2]);
    f2_unpack(p.q01, v[1], v[3]);
    v[4] = p.s2;
    v[5] = p.q2;
}

// The SSIM, artifact and detail-loss maps of one pixel (score.hpp:141-153), pooled into P. All
// values are on samples shifted by the segment's constant: m1 = E[a], m2 = E[b],
// dd = E[(a - b)^2], m12 = E[a b] (blurred), i1, i2 the pixel's own samples.
// The reference's SSIM map is max(1 - (1 - (m1 - m2)^2) (2 s12 + C2) / (s11 + s22 + C2), 0).
// With t = dd - (m1 - m2)^2 = s11 + s22 - 2 s12 (the variance of a - b) and n = 2 s12 + C2 its
// denominator is t + n, and the map is max((t + (m1 - m2)^2 n) / (t + n), 0): the same quantity
// without the cancellation in 1 - num / den or in s11 + s22, and exactly 0 for identical images
// (a - b = 0 makes dd and m1 - m2 exactly 0). The edge maps: (|I2 - m2| + 1) / (|I1 - m1| + 1) - 1
// written as (|I2 - m2| - |I1 - m1|) / (|I1 - m1| + 1); |I - mu| is shift-invariant.
__device__ __forceinline__ void s2_pixel_maps(float m1, float m2, float dd, float m12, float i1, float i2,
                                              S2Pools& P) {
    const float md = m1 - m2;
    const float md2 = md * md;
    const float t = dd - md2;
    const float n = fmaf(fmaf(-m1, m2, m12), 2.0f, 0.0009f);
    const float d0 = fmaxf(__fdividef(fmaf(md2, n, t), t + n), 0.0f);
    const float e1 = fabsf(i1 - m1), e2 = fabsf(i2 - m2);
    const float v = __fdividef(e2 - e1, e1 + 1.0f);
    const float d1 = fmaxf(v, 0.0f), d2 = fmaxf(-v, 0.0f);
    const f2_t d01 = f2_pack(d0, d1);
    P.s01 = f2_add(P.s01, d01);
    const f2_t q = f2_mul(d01, d01);
    P.q01 = f2_fma(q, q, P.q01);
    P.s2 += d2;
    const float q2 = d2 * d2;
    P.q2 = fmaf(q2, q2, P.q2);
}

// FP16 delta tile: 64 rows x 48 halves, row pitch 56 halves (7 quads: conflict-free 16-byte reads)
constexpr int ST_DP = 56;

// One segment (32 columns x up to L.seg rows) of one scale: the four moments, the maps and 18
// pooled sums written to out[pool * stride] (pool = map * 2 + norm, times 3 channels). im1 / im2
// point at the tile's scale in the channel-0 plane; DELTA: im2 holds FP16 differences against im1.
template <bool DELTA>
__device__ __forceinline__ void stats_tile(const float* __restrict__ im1, const void* __restrict__ im2v, int64_t pe,
                                           const Ssimu2Level& L, int lt, float* __restrict__ out, int stride) {
    extern __shared__ __align__(16) float sm[];
    float* raw = sm;                   // [image][64][52]
    float* hb = sm + 2 * ST_RAW;       // [2 pair planes][32 columns of 86 slots, 8-pair gaps]
    float* red = hb + 4 * ST_HPLANE;   // [3 channels][8 warps][6 pools]
    const float* im2 = static_cast<const float*>(im2v);
    const __half* im2h = static_cast<const __half*>(im2v);
    const int tx0 = (lt % L.tiles_x) * ST_TW;
    const int sy0 = (lt / L.tiles_x) * L.seg;
    const int nchunk = (min(L.seg, L.h - sy0) + ST_TH - 1) / ST_TH;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool x_inside = tx0 >= ST_R && tx0 + ST_TW + ST_R <= L.w;

    // H pass mapping: output columns 8*hg .. 8*hg+7 (inputs 8*hg .. 8*hg+23) of 8 consecutive raw
    // rows per warp x 4 column groups, which keeps the float4 raw reads and the float-pair stores
    // into the column-major ring bank-conflict free.
    const int hg = lane >> 3;
    // V pass mapping: column vc (0..31), output rows 6*vg .. 6*vg+5 of the chunk. Both passes'
    // border renormalisations (out / tot, gaussianblur.hpp:63-92) are applied here as one product.
    const int vc = tid & 31, vg = tid >> 5;
    const float rxv = s2_inv_mass(tx0 + vc, L.w);
    float* r1 = raw;
    float* r2 = raw + ST_RAW;

#pragma unroll 1
    for (int c = 0; c < 3; c++) {
        S2Pools P = s2_pools_zero();
        float shift = 0.f;
#pragma unroll 1
        for (int k = 0; k < nchunk; k++) {
            const int ty0 = sy0 + k * ST_TH;
            stage_tile_t<ST_IH, 12>(r1, ST_RP, im1 + (int64_t)c * pe, L.pitch, L.w, L.h, tx0 - ST_R, ty0 - ST_R);
            if (DELTA)
                stage_tile_t<ST_IH, 6>(reinterpret_cast<__half*>(r2), ST_DP, im2h + (int64_t)c * pe, L.pitch, L.w, L.h,
                                       tx0 - ST_R, ty0 - ST_R);
            else
                stage_tile_t<ST_IH, 12>(r2, ST_RP, im2 + (int64_t)c * pe, L.pitch, L.w, L.h, tx0 - ST_R, ty0 - ST_R);
            cp_async_commit();
            cp_async_wait<0>();
            __syncthreads();
            // Moments are formed on values shifted by one per-segment constant (the reference
            // image's value at the segment origin). The blur is normalised, so sigma =
            // E[(x-s)^2] - (E[x]-s)^2 is unchanged, while the FP32 cancellation of E[x^2] - E[x]^2
            // shrinks by the square of |x| / |x - s|. Samples outside the image must carry
            // nothing: on border chunks their slots are set to the shift itself, so that x - s is
            // exactly zero there.
            if (k == 0) shift = r1[ST_R * ST_RP + ST_R];
            if (!(x_inside && ty0 >= ST_R && ty0 + ST_TH + ST_R <= L.h)) {
                for (int e = tid; e < ST_IH * ST_IW; e += 256) {
                    const int r = e / ST_IW, col = e - r * ST_IW;
                    const int gx = tx0 - ST_R + col, gy = ty0 - ST_R + r;
                    if (gx < 0 || gx >= L.w || gy < 0 || gy >= L.h) {
                        r1[r * ST_RP + col] = shift;
                        if (!DELTA) r2[r * ST_RP + col] = shift;  // FP16 deltas arrive as zeros there
                    }
                }
                __syncthreads();
            }
            // Horizontal pass over the raw rows whose ring row is new: rows 0..63 of the first
            // chunk (8 warps), rows 16..63 later (6 warps, the two idle ones rotating with the
            // chunk so that the SM's four schedulers share the work evenly). Segment row
            // h = 48k + r goes to ring slot h & 63, and to slot 64 + (h & 63) as well when that is
            // below 22. The SSIM map needs the two variances only as their sum (score.hpp:147), so
            // four moments are blurred: {a, b} and {(a - b)^2, a b} (s2_pixel_maps), each pair
            // through the f32x2 FMA with a shared weight.
            const int rr = k == 0 ? 8 * warp + (lane & 7) : 2 * ST_R + 8 * ((warp + 2 * k) & 7) + (lane & 7);
            if (rr < ST_IH) {
                f2_t h1[8], h2[8];
                const f2_t z2 = f2_pack(0.f, 0.f);
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    h1[o] = z2;
                    h2[o] = z2;
                }
                const float* ra = r1 + rr * ST_RP + 8 * hg;
                const float* rb = r2 + rr * ST_RP + 8 * hg;
                float dl[24];  // DELTA: the 24 deltas of this thread's window
                if (DELTA) {
                    const __half* rd = reinterpret_cast<const __half*>(r2) + rr * ST_DP + 8 * hg;
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        const uint4 v4 = *reinterpret_cast<const uint4*>(rd + 8 * q);
                        const __half2* hq = reinterpret_cast<const __half2*>(&v4);
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const float2 f = __half22float2(hq[u]);
                            dl[8 * q + 2 * u] = f.x;
                            dl[8 * q + 2 * u + 1] = f.y;
                        }
                    }
                }
#pragma unroll
                for (int j4 = 0; j4 < 6; j4++) {
                    const float4 va = *reinterpret_cast<const float4*>(ra + 4 * j4);
                    float4 vb = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (!DELTA) vb = *reinterpret_cast<const float4*>(rb + 4 * j4);
                    const float la[4] = {va.x, va.y, va.z, va.w};
                    const float lb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int j = 4 * j4 + u;
                        const float a = la[u] - shift;
                        const float b = DELTA ? a + dl[j] : lb[u] - shift;
                        const float d = DELTA ? dl[j] : la[u] - lb[u];  // b - a or a - b: squared
                        const f2_t p1 = f2_pack(a, b);
                        const f2_t p2 = f2_pack(d * d, a * b);
#pragma unroll
                        for (int o = 0; o < 8; o++) {
                            const int i = j - o;  // tap index
                            if (i >= 0 && i < 17) {
                                h1[o] = f2_fma(p1, c_s2_k2n[i], h1[o]);
                                h2[o] = f2_fma(p2, c_s2_k2n[i], h2[o]);
                            }
                        }
                    }
                }
                const int slot = (k * ST_TH + rr) & (ST_RING - 1);
                f2_t* d1 = reinterpret_cast<f2_t*>(hb) + 8 * hg * (ST_HROWS + 1) + slot;
                f2_t* d2 = reinterpret_cast<f2_t*>(hb + 2 * ST_HPLANE) + 8 * hg * (ST_HROWS + 1) + slot;
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    d1[o * ST_HROWS] = h1[o];
                    d2[o * ST_HROWS] = h2[o];
                }
                if (slot < ST_WIN) {
#pragma unroll
                    for (int o = 0; o < 8; o++) {
                        d1[o * ST_HROWS + ST_RING] = h1[o];
                        d2[o * ST_HROWS + ST_RING] = h2[o];
                    }
                }
            }
            __syncthreads();
            // vertical pass + maps (column vc, chunk rows 6*vg .. 6*vg+5): the window is ring rows
            // s0 .. s0+21 with s0 = (48k + 6*vg) & 63, never past the mirrored slots. A chunk whose
            // windows all lie inside the image needs neither renormalisation nor bounds tests.
            const bool interior = x_inside && ty0 >= ST_R && ty0 + ST_TH + ST_R <= L.h;
            float rxy[6];
#pragma unroll
            for (int o = 0; o < 6; o++) rxy[o] = interior ? 1.0f : rxv * s2_inv_mass(ty0 + 6 * vg + o, L.h);
            float m[4][6];  // mu1, mu2, E[(a - b)^2], E[a b] (shifted)
            {
                const int s0 = (k * ST_TH + 6 * vg) & (ST_RING - 1);
                const int cb = vc * ST_HROWS + 8 * (vc >> 3) + s0;  // even: 16-byte aligned
                const f2_t* c1 = reinterpret_cast<const f2_t*>(hb) + cb;
                const f2_t* c2 = reinterpret_cast<const f2_t*>(hb + 2 * ST_HPLANE) + cb;
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const f2_t* col = q == 0 ? c1 : c2;
                    f2_t v[ST_WIN];
#pragma unroll
                    for (int j = 0; j < ST_WIN / 2; j++) {
                        const ulonglong2 p2 = reinterpret_cast<const ulonglong2*>(col)[j];
                        v[2 * j] = p2.x;
                        v[2 * j + 1] = p2.y;
                    }
#pragma unroll
                    for (int o = 0; o < 6; o++) {
                        f2_t a = f2_pack(0.f, 0.f);
#pragma unroll
                        for (int i = 0; i < 17; i++) a = f2_fma(v[o + i], c_s2_k2n[i], a);
                        if (!interior) a = f2_mul(a, f2_pack(rxy[o], rxy[o]));
                        f2_unpack(a, m[2 * q][o], m[2 * q + 1][o]);
                    }
                }
            }
#pragma unroll
            for (int o = 0; o < 6; o++) {
                const int y = ty0 + 6 * vg + o, x = tx0 + vc;
                if (interior || (x < L.w && y < L.h)) {
                    const int so = (6 * vg + o + ST_R) * ST_RP + vc + ST_R;
                    const float i1 = r1[so] - shift;  // shifted samples
                    const float i2 = DELTA ? i1 + __half2float(reinterpret_cast<const __half*>(r2)[(6 * vg + o + ST_R) * ST_DP +
                                                                                                     vc + ST_R])
                                           : r2[so] - shift;
                    s2_pixel_maps(m[0][o], m[1][o], m[2][o], m[3][o], i1, i2, P);
                }
            }
            __syncthreads();  // the raw tiles and ring slots are rewritten by the next chunk
        }
        float pv[6];
        s2_pools_unpack(P, pv);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const float v = warp_sum(pv[i]);
            if (lane == 0) red[(c * 8 + warp) * 6 + i] = v;
        }
    }
    __syncthreads();
    // pools: out[(pool * 3 + channel) * stride], pool = map * 2 + norm
    if (tid < 18) {
        const int pool = tid / 3, c = tid - pool * 3;
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < 8; w++) v += red[(c * 8 + w) * 6 + pool];
        out[(int64_t)tid * stride] = v;
    }
}

// ------------------------------------------------------------------------------------------
// Second tile shape of the stats kernel: the same 32-column segments, walked in 64-row chunks.
// The horizontal pass writes a column-major buffer of 80 rows (the chunk's 64 and the 8-row
// halos) instead of the ring, and the 16 rows a chunk shares with the next are carried over
// (copied from buffer rows 64..79 to 0..15) rather than blurred again, so every chunk after the
// first blurs exactly 64 new rows: one 8-row block per warp, all 8 warps busy (the ring shape
// leaves 2 of 8 warps idle in that pass). The vertical pass gives each thread one column and 8
// consecutive output rows; it streams the 24 buffer rows of its window once (12 16-byte loads per
// moment pair) and scatters each into the 8 outputs it feeds. Fewer chunks and no idle warps
// halve the barrier waits; the larger window costs registers. The batched form's autotuner
// chooses between the two shapes per workload.
constexpr int SC_TH = 64;
constexpr int SC_IH = SC_TH + 2 * ST_R;  // 80 raw rows per chunk (image rows ty0 - 8 ..)
constexpr int SC_RAW = SC_IH * ST_RP;    // one raw tile
constexpr int SC_WIN = SC_TH / 8 + 2 * ST_R;  // 24 buffer rows per vertical window
// column x of a buffer plane starts at float pair x * SC_HP + 8 * (x / 8); SC_HP = 82 pairs is 41
// quads, odd, so the 16-byte loads of 8 neighbouring columns hit distinct bank quads, and the
// 8-pair gap between column groups keeps a half-warp's 8-byte stores of two groups apart
constexpr int SC_HP = 82;
constexpr int SC_HPLANE = ST_TW * SC_HP + 8 * (ST_TW / 8 - 1);
// smem: the 2 raw images, two float-pair planes {m1, m2} and {s11 + s22, s12}, the per-warp
// pools: 74.4 KB, still three CTAs per SM
constexpr int kStatsSmemC = (2 * SC_RAW + 4 * SC_HPLANE + 3 * 8 * 6) * 4;
static_assert(ST_SEG % SC_TH == 0 && ST_SEG_TALL % SC_TH == 0 && ST_SEG_TALL % ST_TH == 0,
              "both shapes walk the same segments");

template <bool DELTA>
__device__ __forceinline__ void stats_tile_c64(const float* __restrict__ im1, const void* __restrict__ im2v,
                                               int64_t pe, const Ssimu2Level& L, int lt, float* __restrict__ out,
                                               int stride) {
    extern __shared__ __align__(16) float sm[];
    float* raw = sm;                  // [image][80][52]
    float* hb = sm + 2 * SC_RAW;      // [2 pair planes][32 columns of 82 rows, 8-pair gaps]
    float* red = hb + 4 * SC_HPLANE;  // [3 channels][8 warps][6 pools]
    const float* im2 = static_cast<const float*>(im2v);
    const __half* im2h = static_cast<const __half*>(im2v);
    const int tx0 = (lt % L.tiles_x) * ST_TW;
    const int sy0 = (lt / L.tiles_x) * L.seg;
    const int nchunk = (min(L.seg, L.h - sy0) + SC_TH - 1) / SC_TH;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool x_inside = tx0 >= ST_R && tx0 + ST_TW + ST_R <= L.w;
    // H pass: output columns 8*hg .. 8*hg+7 of 8 consecutive raw rows per warp x 4 column groups.
    const int hg = lane >> 3, hr = lane & 7;
    // V pass: column vc, output rows 8*vg .. 8*vg+7 of the chunk; both passes' border
    // renormalisations (gaussianblur.hpp:63-92) applied there as one product.
    const int vc = tid & 31, vg = tid >> 5;
    const float rxv = s2_inv_mass(tx0 + vc, L.w);
    float* r1 = raw;
    float* r2 = raw + SC_RAW;
    f2_t* const hp1 = reinterpret_cast<f2_t*>(hb);
    f2_t* const hp2 = reinterpret_cast<f2_t*>(hb + 2 * SC_HPLANE);

#pragma unroll 1
    for (int c = 0; c < 3; c++) {
        S2Pools P = s2_pools_zero();
        float shift = 0.f;
#pragma unroll 1
        for (int k = 0; k < nchunk; k++) {
            const int ty0 = sy0 + k * SC_TH;
            // the first chunk stages raw rows 0..79 (image rows ty0 - 8 ..); later chunks rows
            // 8..79 only (rows 0..7 fed the carried rows and no output of this chunk)
            const int rlo = k == 0 ? 0 : ST_R;
            if (k == 0) {
                stage_tile_t<SC_IH, 12>(r1, ST_RP, im1 + (int64_t)c * pe, L.pitch, L.w, L.h, tx0 - ST_R, ty0 - ST_R);
                if (DELTA)
                    stage_tile_t<SC_IH, 6>(reinterpret_cast<__half*>(r2), ST_DP, im2h + (int64_t)c * pe, L.pitch, L.w,
                                           L.h, tx0 - ST_R, ty0 - ST_R);
                else
                    stage_tile_t<SC_IH, 12>(r2, ST_RP, im2 + (int64_t)c * pe, L.pitch, L.w, L.h, tx0 - ST_R,
                                            ty0 - ST_R);
            } else {
                stage_tile_t<SC_IH - ST_R, 12>(r1 + ST_R * ST_RP, ST_RP, im1 + (int64_t)c * pe, L.pitch, L.w, L.h,
                                               tx0 - ST_R, ty0);
                if (DELTA)
                    stage_tile_t<SC_IH - ST_R, 6>(reinterpret_cast<__half*>(r2) + ST_R * ST_DP, ST_DP,
                                                  im2h + (int64_t)c * pe, L.pitch, L.w, L.h, tx0 - ST_R, ty0);
                else
                    stage_tile_t<SC_IH - ST_R, 12>(r2 + ST_R * ST_RP, ST_RP, im2 + (int64_t)c * pe, L.pitch, L.w,
                                                   L.h, tx0 - ST_R, ty0);
            }
            cp_async_commit();
            cp_async_wait<0>();
            __syncthreads();
            // the per-segment shift and the border treatment of the ring shape (stats_tile)
            if (k == 0) shift = r1[ST_R * ST_RP + ST_R];
            if (!(x_inside && ty0 >= ST_R && ty0 + SC_TH + ST_R <= L.h)) {
                for (int e = tid + rlo * ST_IW; e < SC_IH * ST_IW; e += 256) {
                    const int r = e / ST_IW, col = e - r * ST_IW;
                    const int gx = tx0 - ST_R + col, gy = ty0 - ST_R + r;
                    if (gx < 0 || gx >= L.w || gy < 0 || gy >= L.h) {
                        r1[r * ST_RP + col] = shift;
                        if (!DELTA) r2[r * ST_RP + col] = shift;  // FP16 deltas arrive as zeros there
                    }
                }
                __syncthreads();
            }
            // Horizontal pass: raw rows 0..79 of the first chunk (ten 8-row blocks; warps 0 and 1
            // take two), rows 16..79 of later chunks (one block per warp); raw row r -> buffer row r.
            const int nblk = k == 0 ? SC_IH / 8 : SC_TH / 8;
            const int blk0 = k == 0 ? 0 : 2;
#pragma unroll 1
            for (int bi = warp; bi < nblk; bi += 8) {
                const int rr = 8 * (blk0 + bi) + hr;
                f2_t h1[8], h2[8];
                const f2_t z2 = f2_pack(0.f, 0.f);
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    h1[o] = z2;
                    h2[o] = z2;
                }
                const float* ra = r1 + rr * ST_RP + 8 * hg;
                const float* rb = r2 + rr * ST_RP + 8 * hg;
                float dl[24];  // DELTA: the 24 deltas of this thread's window
                if (DELTA) {
                    const __half* rd = reinterpret_cast<const __half*>(r2) + rr * ST_DP + 8 * hg;
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        const uint4 v4 = *reinterpret_cast<const uint4*>(rd + 8 * q);
                        const __half2* hq = reinterpret_cast<const __half2*>(&v4);
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const float2 f = __half22float2(hq[u]);
                            dl[8 * q + 2 * u] = f.x;
                            dl[8 * q + 2 * u + 1] = f.y;
                        }
                    }
                }
#pragma unroll
                for (int j4 = 0; j4 < 6; j4++) {
                    const float4 va = *reinterpret_cast<const float4*>(ra + 4 * j4);
                    float4 vb = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (!DELTA) vb = *reinterpret_cast<const float4*>(rb + 4 * j4);
                    const float la[4] = {va.x, va.y, va.z, va.w};
                    const float lb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int j = 4 * j4 + u;
                        const float a = la[u] - shift;
                        const float b = DELTA ? a + dl[j] : lb[u] - shift;
                        const float d = DELTA ? dl[j] : la[u] - lb[u];  // b - a or a - b: squared
                        const f2_t p1 = f2_pack(a, b);
                        const f2_t p2 = f2_pack(d * d, a * b);
#pragma unroll
                        for (int o = 0; o < 8; o++) {
                            const int i = j - o;  // tap index
                            if (i >= 0 && i < 17) {
                                h1[o] = f2_fma(p1, c_s2_k2n[i], h1[o]);
                                h2[o] = f2_fma(p2, c_s2_k2n[i], h2[o]);
                            }
                        }
                    }
                }
                f2_t* d1 = hp1 + 8 * hg * (SC_HP + 1) + rr;
                f2_t* d2 = hp2 + 8 * hg * (SC_HP + 1) + rr;
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    d1[o * SC_HP] = h1[o];
                    d2[o * SC_HP] = h2[o];
                }
            }
            __syncthreads();
            // vertical pass + maps: buffer rows 8*vg .. 8*vg+23 streamed once, each scattered into
            // the 8 outputs it feeds. A chunk whose windows all lie inside the image needs neither
            // renormalisation nor bounds tests.
            const bool interior = x_inside && ty0 >= ST_R && ty0 + SC_TH + ST_R <= L.h;
            // vertical pass + maps in one block per case, so that the scheduler can interleave
            // the maps of completed outputs with the taps of the others
            auto vpass = [&](f2_t* a1, f2_t* a2) {
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    a1[o] = f2_pack(0.f, 0.f);
                    a2[o] = a1[o];
                }
                const int cb = vc * SC_HP + 8 * (vc >> 3) + 8 * vg;  // even: 16-byte aligned
                const ulonglong2* c1 = reinterpret_cast<const ulonglong2*>(hp1 + cb);
                const ulonglong2* c2 = reinterpret_cast<const ulonglong2*>(hp2 + cb);
#pragma unroll
                for (int jj = 0; jj < SC_WIN / 2; jj++) {
                    const ulonglong2 q1 = c1[jj];
                    const ulonglong2 q2 = c2[jj];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int j = 2 * jj + h;
                        const f2_t v1 = h ? q1.y : q1.x;
                        const f2_t v2 = h ? q2.y : q2.x;
#pragma unroll
                        for (int o = 0; o < 8; o++) {
                            const int i = j - o;
                            if (i >= 0 && i < 17) {
                                a1[o] = f2_fma(v1, c_s2_k2n[i], a1[o]);
                                a2[o] = f2_fma(v2, c_s2_k2n[i], a2[o]);
                            }
                        }
                    }
                }
            };
            if (interior) {
                f2_t a1[8], a2[8];
                vpass(a1, a2);
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    float m1, m2, dd, m12;
                    f2_unpack(a1[o], m1, m2);
                    f2_unpack(a2[o], dd, m12);
                    const int so = (8 * vg + o + ST_R) * ST_RP + vc + ST_R;
                    const float i1 = r1[so] - shift;
                    const float i2 = DELTA ? i1 + __half2float(reinterpret_cast<const __half*>(r2)[(8 * vg + o + ST_R) * ST_DP +
                                                                                                     vc + ST_R])
                                           : r2[so] - shift;
                    s2_pixel_maps(m1, m2, dd, m12, i1, i2, P);
                }
            } else {
                f2_t a1[8], a2[8];
                vpass(a1, a2);
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    const int y = ty0 + 8 * vg + o, x = tx0 + vc;
                    if (x < L.w && y < L.h) {
                        const float rxy = rxv * s2_inv_mass(y, L.h);
                        float m1, m2, dd, m12;
                        f2_unpack(f2_mul(a1[o], f2_pack(rxy, rxy)), m1, m2);
                        f2_unpack(f2_mul(a2[o], f2_pack(rxy, rxy)), dd, m12);
                        const int so = (8 * vg + o + ST_R) * ST_RP + vc + ST_R;
                        const float i1 = r1[so] - shift;
                        const float i2 = DELTA ? i1 + __half2float(reinterpret_cast<const __half*>(r2)[(8 * vg + o + ST_R) * ST_DP +
                                                                                                         vc + ST_R])
                                               : r2[so] - shift;
                        s2_pixel_maps(m1, m2, dd, m12, i1, i2, P);
                    }
                }
            }
            __syncthreads();  // the raw tiles and buffer rows are rewritten for the next chunk
            if (k + 1 < nchunk) {
                // carry buffer rows 64..79 to rows 0..15: 2 planes x 32 columns x 8 16-byte row
                // pairs, two per thread (the next chunk's first barrier orders them before its
                // horizontal pass writes rows 16..79)
#pragma unroll
                for (int q = tid; q < 2 * ST_TW * 8; q += 256) {
                    f2_t* pl = q < ST_TW * 8 ? hp1 : hp2;
                    const int e = q & (ST_TW * 8 - 1), x = e >> 3, rp = e & 7;
                    ulonglong2* col = reinterpret_cast<ulonglong2*>(pl + x * SC_HP + 8 * (x >> 3));
                    col[rp] = col[SC_TH / 2 + rp];
                }
            }
        }
        float pv[6];
        s2_pools_unpack(P, pv);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const float v = warp_sum(pv[i]);
            if (lane == 0) red[(c * 8 + warp) * 6 + i] = v;
        }
    }
    __syncthreads();
    if (tid < 18) {
        const int pool = tid / 3, c = tid - pool * 3;
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < 8; w++) v += red[(c * 8 + w) * 6 + pool];
        out[(int64_t)tid * stride] = v;
    }
}

// tile shape 0: 48-row chunks through the ring (stats_tile); 1: 64-row chunks through the carry
// buffer (stats_tile_c64). Both walk the same segments and write the same 18 sums per segment.
template <int SHAPE, bool DELTA>
__device__ __forceinline__ void stats_segment(const float* __restrict__ im1, const void* __restrict__ im2v,
                                              int64_t pe, const Ssimu2Level& L, int lt, float* __restrict__ out,
                                              int stride) {
    if (SHAPE == 0) stats_tile<DELTA>(im1, im2v, pe, L, lt, out, stride);
    else stats_tile_c64<DELTA>(im1, im2v, pe, L, lt, out, stride);
}
constexpr int stats_smem(int shape) { return shape == 0 ? kStatsSmem : kStatsSmemC; }
// The per-pair entry points (and the no-allocation one, which must give their results bit for
// bit) use one fixed shape, the faster at 1920x1080 on a GB300.
constexpr int kPlainShape = 1;

// grid (tiles_total, npairs), dynamic smem stats_smem(SHAPE)
template <int SHAPE>
__global__ void __launch_bounds__(256, 3) ssimu2_stats_kernel(const float* __restrict__ pyr,
                                                              float* __restrict__ partials, Ssimu2Geom g) {
    const int pair = blockIdx.y;
    const int t = blockIdx.x;
    int s = 0;
#pragma unroll
    for (int k = 1; k < 6; k++) s += (t >= g.tile_begin[k]);
    const Ssimu2Level L = g.lv[s];
    const float* im1 = pyr + (int64_t)(pair * 2 + 0) * 3 * g.plane_elems + L.off;
    const float* im2 = pyr + (int64_t)(pair * 2 + 1) * 3 * g.plane_elems + L.off;
    stats_segment<SHAPE, false>(im1, im2, g.plane_elems, L, t - g.tile_begin[s],
                                partials + (int64_t)pair * 18 * g.tiles_total + t, g.tiles_total);
}

// the FP16-delta form: the reference's FP32 pyramid and the distorted image's FP16 deltas
template <int SHAPE>
__global__ void __launch_bounds__(256, 3) ssimu2_stats_delta_kernel(const float* __restrict__ ref,
                                                                    const __half* __restrict__ d16,
                                                                    float* __restrict__ partials, Ssimu2Geom g) {
    const int pair = blockIdx.y;
    const int t = blockIdx.x;
    int s = 0;
#pragma unroll
    for (int k = 1; k < 6; k++) s += (t >= g.tile_begin[k]);
    const Ssimu2Level L = g.lv[s];
    const int64_t o = (int64_t)pair * 3 * g.plane_elems + L.off;
    stats_segment<SHAPE, true>(ref + o, d16 + o, g.plane_elems, L, t - g.tile_begin[s],
                               partials + (int64_t)pair * 18 * g.tiles_total + t, g.tiles_total);
}

// ------------------------------------------------------------------------------------------
// Kernel 3: finalisation, one CTA of kFinThreads per pair. The 108 (scale, pool, channel) sums
// are reduced over their tiles by 32 warps at once (coalesced loads, four in flight per lane) as
// float-float sums; then 108 threads form the features in FP64 (mean, 4th root, weight) and sum
// them; only the score mapping runs on one thread. The kernel is latency-bound: on this GPU a
// dependent FP64 operation takes about 60 cycles, an FP64 square root or reciprocal several
// hundred and pow() several thousand, so the tile sums stay on the FP32 pipe, the means
// multiply by inverses computed while the loads are in flight, the 4th roots use division-free
// Newton steps and the score mapping exp2(e log2 x).
// partials: this pair's [18][tiles_total] block.
constexpr int kFinThreads = 1024;

// x^(1/4) in FP64 arithmetic without FP64 square roots: y ~ x^(-1/4) from the FP32
// approximations (relative error about 4e-7), two Newton steps for y^-4 = x,
// y' = y + y (1 - x y^4) / 4 (division-free; the relative error e becomes about 2.5 e^2 per step:
// 4e-13, then below FP64 rounding), then x^(1/4) = x y^3. Zero, NaN and values far outside
// FP32's range take the FP64 square roots.
__device__ __forceinline__ double root4(double x) {
    const float xf = (float)x;
    if (!(xf > 1e-30f && xf < 1e30f)) return sqrt(sqrt(x));
    double y = (double)rsqrtf(sqrtf(xf));
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const double y2 = y * y;
        y = fma(y, 0.25 * (1.0 - x * (y2 * y2)), y);
    }
    return (x * y) * (y * y);
}

__device__ __forceinline__ void finalize_pair(const float* __restrict__ partials, const Ssimu2Geom& g,
                                              double* __restrict__ score) {
    constexpr int NW = kFinThreads / 32;
    __shared__ FSum pooled[6][18];
    __shared__ double inv_px[6];
    __shared__ double red[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tiles_total = g.tiles_total;
    // the last warp has the fewest segments: it also computes 1 / pixels per scale
    if (warp == NW - 1 && lane < 6) inv_px[lane] = 1.0 / ((double)g.lv[lane].w * (double)g.lv[lane].h);
    for (int seg = warp; seg < 108; seg += NW) {
        const int s = seg / 18, i = seg - 18 * (seg / 18);
        const float* p = partials + (int64_t)i * tiles_total + g.tile_begin[s];
        const int n = g.tile_begin[s + 1] - g.tile_begin[s];
        FSum a{0.f, 0.f};
        for (int t0 = lane; t0 < n; t0 += 128) {
            float v[4];
#pragma unroll
            for (int k = 0; k < 4; k++) v[k] = t0 + 32 * k < n ? __ldg(p + t0 + 32 * k) : 0.f;
#pragma unroll
            for (int k = 0; k < 4; k++) a.add(v[k]);
        }
        a = warp_sum(a);
        if (lane == 0) pooled[s][i] = a;
    }
    __syncthreads();
    // feature k = plane*36 + scale*6 + norm*3 + map (ssimu2/main.hpp:83-95); pooled index
    // (map*2 + norm)*3 + plane; the mean over the scale's pixels, 4th root for the 4-norm
    // (score.hpp:263-267)
    if (tid < 128) {
        double v = 0.0;
        if (tid < 108) {
            const int plane = tid / 36, sc = (tid % 36) / 6, nrm = (tid % 6) / 3, mi = tid % 3;
            double x = pooled[sc][(mi * 2 + nrm) * 3 + plane].value() * inv_px[sc];
            if (nrm == 1) x = root4(x);
            v = c_s2_w[tid] * x;
        }
        v = warp_sum(v);
        if (lane == 0) red[warp] = v;
    }
    __syncthreads();
    if (tid == 0) {
        double ssim = 0.0;
        for (int w = 0; w < 4; w++) ssim += red[w];
        ssim *= 0.9562382616834844;  // score.hpp:388-397
        ssim = (6.248496625763138e-5 * ssim * ssim) * ssim + 2.326765642916932 * ssim -
               0.020884521182843837 * ssim * ssim;
        *score = ssim > 0.0 ? exp2(0.6276336467831387 * log2(ssim)) * -10.0 + 100.0 : 100.0;
    }
}

__global__ void __launch_bounds__(kFinThreads) ssimu2_finalize_kernel(const float* __restrict__ partials,
                                                              double* __restrict__ scores, Ssimu2Geom g) {
    finalize_pair(partials + (int64_t)blockIdx.x * 18 * g.tiles_total, g, scores + blockIdx.x);
}

// ------------------------------------------------------------------------------------------
// Work-list kernels of the batched multi-resolution form (Ssimu2MultiEngine).
// one 32x32 level-0 tile per CTA: items {image, tile x, tile y, unused}
template <int IT, bool DELTA>
__global__ void __launch_bounds__(256, IT == IN_YUV ? 6 : 8) ssimu2_multi_pyramid_kernel(const Ssimu2MultiImage* __restrict__ imgs,
                                                                   const int4* __restrict__ items,
                                                                   const Ssimu2Geom* __restrict__ geoms) {
    const int4 it = items[blockIdx.x];
    const Ssimu2MultiImage im = imgs[it.x];
    const PyrOut out{im.f32, static_cast<__half*>(im.d16), im.ref};
    pyramid_tile<IT, DELTA>(im.fd, im.yp, out, geoms[im.geom], it.y, it.z);
}

// persistent: CTA b takes items b, b + gridDim.x, ...; items {pair, tile}
template <bool DELTA, int SHAPE>
__global__ void __launch_bounds__(256, 3) ssimu2_multi_stats_kernel(const Ssimu2MultiPair* __restrict__ pairs,
                                                                    const int2* __restrict__ items, int nitems,
                                                                    const Ssimu2Geom* __restrict__ geoms) {
    for (int i = blockIdx.x; i < nitems; i += gridDim.x) {
        const int2 it = items[i];
        const Ssimu2MultiPair P = pairs[it.x];
        const Ssimu2Geom& g = geoms[P.geom];
        int s = 0;
#pragma unroll
        for (int k = 1; k < 6; k++) s += (it.y >= g.tile_begin[k]);
        const Ssimu2Level L = g.lv[s];
        const void* im2 = DELTA ? static_cast<const void*>(static_cast<const __half*>(P.cand) + L.off)
                                : static_cast<const void*>(static_cast<const float*>(P.cand) + L.off);
        stats_segment<SHAPE, DELTA>(P.src + L.off, im2, g.plane_elems, L, it.y - g.tile_begin[s], P.partials + it.y,
                                    g.tiles_total);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kFinThreads) ssimu2_multi_finalize_kernel(const Ssimu2MultiPair* __restrict__ pairs,
                                                                    const Ssimu2Geom* __restrict__ geoms) {
    const Ssimu2MultiPair P = pairs[blockIdx.x];
    finalize_pair(P.partials, geoms[P.geom], P.score);
}

// ------------------------------------------------------------------------------------------
// Host side

Ssimu2Geom make_ssimu2_geom(int64_t w, int64_t h, bool tall) {
    Ssimu2Geom g{};
    int64_t off = 0;
    int tiles = 0;
    int64_t cw = w, ch = h;
    for (int s = 0; s < 6; s++) {
        Ssimu2Level& L = g.lv[s];
        L.w = (int)cw;
        L.h = (int)ch;
        L.pitch = (int)round_up(cw, 8);
        L.off = off;
        off += round_up((int64_t)L.pitch * ch, 64);
        L.tiles_x = (int)ceil_div(cw, ST_TW);
        L.seg = tall && L.tiles_x * ceil_div(ch, ST_SEG_TALL) >= kSegTallMin ? ST_SEG_TALL : ST_SEG;
        L.tiles_y = (int)ceil_div(ch, L.seg);
        g.tile_begin[s] = tiles;
        tiles += L.tiles_x * L.tiles_y;
        cw = half_dim(cw);
        ch = half_dim(ch);
    }
    g.tile_begin[6] = tiles;
    g.tiles_total = tiles;
    g.plane_elems = off;
    return g;
}

int Ssimu2Engine::init(int64_t width, int64_t height, int max_pairs_, bool fp16_deltas) {
    w = width;
    h = height;
    max_pairs = max_pairs_;
    fp16 = fp16_deltas;
    geom = make_ssimu2_geom(w, h);
    geom_tall = make_ssimu2_geom(w, h, true);  // no more tiles than geom: the partials fit either
    int rc = upload_constants_once();
    if (rc) return rc;
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_stats_kernel<kPlainShape>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        stats_smem(kPlainShape)));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_stats_delta_kernel<kPlainShape>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, stats_smem(kPlainShape)));
    // FP32: [pair][image][channel][plane_elems] floats. FP16 deltas: the references' FP32 planes
    // [pair][channel][plane_elems], then the distorted images' FP16 planes in the same order
    // (plane_elems is a multiple of 64, so the half block starts 256-byte aligned).
    VSHIP_CUDA_TRY(vship_malloc((void**)&pyr, pyramid_bytes(geom, max_pairs, fp16)));
    d16 = fp16 ? reinterpret_cast<__half*>(pyr + (size_t)geom.plane_elems * 3 * max_pairs) : nullptr;
    VSHIP_CUDA_TRY(vship_malloc((void**)&partials, sizeof(float) * (size_t)geom.tiles_total * 18 * max_pairs));
    VSHIP_CUDA_TRY(vship_malloc((void**)&scores, sizeof(double) * max_pairs));
    return E_OK;
}

void Ssimu2Engine::destroy() {
    if (pyr) cudaFree(pyr);
    if (partials) cudaFree(partials);
    if (scores) cudaFree(scores);
    pyr = nullptr;
    d16 = nullptr;
    partials = nullptr;
    scores = nullptr;
}

size_t Ssimu2Engine::pyramid_bytes(const Ssimu2Geom& g, int pairs, bool fp16) {
    // both images' three channels: FP32 (4 + 4 bytes per element) or FP32 + FP16 (4 + 2)
    return (size_t)g.plane_elems * 3 * pairs * (fp16 ? 6 : 8);
}

size_t Ssimu2Engine::device_bytes(int64_t w, int64_t h, int pairs, bool fp16) {
    Ssimu2Geom g = make_ssimu2_geom(w, h);
    return pyramid_bytes(g, pairs, fp16) + sizeof(float) * (size_t)g.tiles_total * 18 * pairs + sizeof(double) * pairs;
}

int Ssimu2Engine::launch(const FrameDesc* frames_dev, int intype, int npairs, double* out_scores, cudaStream_t st,
                         const YuvParams* yuv) {
    if (npairs <= 0 || npairs > max_pairs) return E_BAD_POINTER;
    const YuvParams yp = yuv ? *yuv : yuv420p10_params();
    if (fp16) return launch_fp16(frames_dev, intype, npairs, out_scores, st, yp);
    const Ssimu2Geom& geom = npairs >= kSsimu2TallPairs ? geom_tall : this->geom;
    dim3 g1((unsigned)ceil_div(w, kPyrTile), (unsigned)ceil_div(h, kPyrTile), (unsigned)(2 * npairs));
    {
    ProfScope ps("ssimu2_pyramid", st);
    switch (intype) {
        case IN_UINT8: ssimu2_pyramid_kernel<IN_UINT8><<<g1, 256, 0, st>>>(frames_dev, pyr, geom, yp); break;
        case IN_UINT16: ssimu2_pyramid_kernel<IN_UINT16><<<g1, 256, 0, st>>>(frames_dev, pyr, geom, yp); break;
        case IN_HALF: ssimu2_pyramid_kernel<IN_HALF><<<g1, 256, 0, st>>>(frames_dev, pyr, geom, yp); break;
        case IN_YUV: ssimu2_pyramid_kernel<IN_YUV><<<g1, 256, 0, st>>>(frames_dev, pyr, geom, yp); break;
        default: ssimu2_pyramid_kernel<IN_FLOAT><<<g1, 256, 0, st>>>(frames_dev, pyr, geom, yp); break;
    }
    }
    dim3 g2((unsigned)geom.tiles_total, (unsigned)npairs);
    {
        ProfScope ps("ssimu2_stats", st);
        ssimu2_stats_kernel<kPlainShape><<<g2, 256, stats_smem(kPlainShape), st>>>(pyr, partials, geom);
    }
    {
        ProfScope ps("ssimu2_finalize", st);
        ssimu2_finalize_kernel<<<npairs, kFinThreads, 0, st>>>(partials, out_scores ? out_scores : scores, geom);
    }
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

template <bool DELTA>
static void launch_pyramid_pair(const FrameDesc* frames, float* ref, __half* d16, const Ssimu2Geom& g,
                                const YuvParams& yp, int intype, dim3 grid, cudaStream_t st) {
    switch (intype) {
        case IN_UINT8: ssimu2_pyramid_pair_kernel<IN_UINT8, DELTA><<<grid, 256, 0, st>>>(frames, ref, d16, g, yp); break;
        case IN_UINT16: ssimu2_pyramid_pair_kernel<IN_UINT16, DELTA><<<grid, 256, 0, st>>>(frames, ref, d16, g, yp); break;
        case IN_HALF: ssimu2_pyramid_pair_kernel<IN_HALF, DELTA><<<grid, 256, 0, st>>>(frames, ref, d16, g, yp); break;
        case IN_YUV: ssimu2_pyramid_pair_kernel<IN_YUV, DELTA><<<grid, 256, 0, st>>>(frames, ref, d16, g, yp); break;
        default: ssimu2_pyramid_pair_kernel<IN_FLOAT, DELTA><<<grid, 256, 0, st>>>(frames, ref, d16, g, yp); break;
    }
}

// The FP16-delta form: the references' pyramids first (FP32), then the distorted images' as FP16
// differences against them, then the stats kernel staging the deltas as halves.
int Ssimu2Engine::launch_fp16(const FrameDesc* frames_dev, int intype, int npairs, double* out_scores,
                              cudaStream_t st, const YuvParams& yp) {
    const Ssimu2Geom& geom = npairs >= kSsimu2TallPairs ? geom_tall : this->geom;
    const dim3 g1((unsigned)ceil_div(w, kPyrTile), (unsigned)ceil_div(h, kPyrTile), (unsigned)npairs);
    {
        ProfScope ps("ssimu2_pyramid", st);
        launch_pyramid_pair<false>(frames_dev, pyr, d16, geom, yp, intype, g1, st);
    }
    {
        ProfScope ps("ssimu2_pyramid_delta", st);
        launch_pyramid_pair<true>(frames_dev, pyr, d16, geom, yp, intype, g1, st);
    }
    dim3 g2((unsigned)geom.tiles_total, (unsigned)npairs);
    {
        ProfScope ps("ssimu2_stats", st);
        ssimu2_stats_delta_kernel<kPlainShape><<<g2, 256, stats_smem(kPlainShape), st>>>(pyr, d16, partials, geom);
    }
    {
        ProfScope ps("ssimu2_finalize", st);
        ssimu2_finalize_kernel<<<npairs, kFinThreads, 0, st>>>(partials, out_scores ? out_scores : scores, geom);
    }
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

// ------------------------------------------------------------------------------------------
// Entry points for callers that provide their own device scratch (used by noalloc.cu).

int ssimu2_prepare_device() {
    int rc = upload_constants_once();
    if (rc) return rc;
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_stats_kernel<kPlainShape>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        stats_smem(kPlainShape)));
    return E_OK;
}

size_t ssimu2_scratch_floats(const Ssimu2Geom& g) {
    return (size_t)g.plane_elems * 6 + (size_t)g.tiles_total * 18;
}

__global__ void ssimu2_store_frames_kernel(FrameDesc a, FrameDesc b, FrameDesc* dst) {
    dst[0] = a;
    dst[1] = b;
}

int ssimu2_launch_scratch(const FrameDesc& ref, const FrameDesc& dist, int intype, const Ssimu2Geom& geom,
                          FrameDesc* frames_scratch, float* scratch, double* out_score, cudaStream_t st) {
    const YuvParams yp = yuv420p10_params();
    float* pyr = scratch;
    float* partials = scratch + (size_t)geom.plane_elems * 6;
    ssimu2_store_frames_kernel<<<1, 1, 0, st>>>(ref, dist, frames_scratch);
    dim3 g1((unsigned)ceil_div(geom.lv[0].w, kPyrTile), (unsigned)ceil_div(geom.lv[0].h, kPyrTile), 2u);
    switch (intype) {
        case IN_UINT8: ssimu2_pyramid_kernel<IN_UINT8><<<g1, 256, 0, st>>>(frames_scratch, pyr, geom, yp); break;
        case IN_UINT16: ssimu2_pyramid_kernel<IN_UINT16><<<g1, 256, 0, st>>>(frames_scratch, pyr, geom, yp); break;
        case IN_HALF: ssimu2_pyramid_kernel<IN_HALF><<<g1, 256, 0, st>>>(frames_scratch, pyr, geom, yp); break;
        case IN_YUV: ssimu2_pyramid_kernel<IN_YUV><<<g1, 256, 0, st>>>(frames_scratch, pyr, geom, yp); break;
        default: ssimu2_pyramid_kernel<IN_FLOAT><<<g1, 256, 0, st>>>(frames_scratch, pyr, geom, yp); break;
    }
    ssimu2_stats_kernel<kPlainShape><<<dim3((unsigned)geom.tiles_total, 1u), 256, stats_smem(kPlainShape), st>>>(
        pyr, partials, geom);
    ssimu2_finalize_kernel<<<1, kFinThreads, 0, st>>>(partials, out_score, geom);
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

// ------------------------------------------------------------------------------------------
// Work-list launches (Ssimu2MultiEngine, multi.cu).

int ssimu2_multi_prepare() {
    int rc = ssimu2_prepare_device();
    if (rc) return rc;
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_multi_stats_kernel<false, 0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, stats_smem(0)));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_multi_stats_kernel<true, 0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, stats_smem(0)));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_multi_stats_kernel<false, 1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, stats_smem(1)));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(ssimu2_multi_stats_kernel<true, 1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, stats_smem(1)));
    return E_OK;
}

int ssimu2_default_stats_shape() { return kPlainShape; }

int ssimu2_multi_stats_blocks_per_sm(bool delta, int shape, int* blocks) {
    if (shape == 0)
        VSHIP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            blocks, delta ? ssimu2_multi_stats_kernel<true, 0> : ssimu2_multi_stats_kernel<false, 0>, 256,
            stats_smem(0)));
    else
        VSHIP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            blocks, delta ? ssimu2_multi_stats_kernel<true, 1> : ssimu2_multi_stats_kernel<false, 1>, 256,
            stats_smem(1)));
    return E_OK;
}

template <bool DELTA>
static void launch_multi_pyramid(const Ssimu2MultiImage* imgs, const int4* items, int nitems,
                                 const Ssimu2Geom* geoms, int intype, cudaStream_t st) {
    const unsigned n = (unsigned)nitems;
    switch (intype) {
        case IN_UINT8: ssimu2_multi_pyramid_kernel<IN_UINT8, DELTA><<<n, 256, 0, st>>>(imgs, items, geoms); break;
        case IN_UINT16: ssimu2_multi_pyramid_kernel<IN_UINT16, DELTA><<<n, 256, 0, st>>>(imgs, items, geoms); break;
        case IN_HALF: ssimu2_multi_pyramid_kernel<IN_HALF, DELTA><<<n, 256, 0, st>>>(imgs, items, geoms); break;
        case IN_YUV:
            ssimu2_multi_pyramid_kernel<IN_YUV, DELTA><<<n, 256, 0, st>>>(imgs, items, geoms);
            break;
        default: ssimu2_multi_pyramid_kernel<IN_FLOAT, DELTA><<<n, 256, 0, st>>>(imgs, items, geoms); break;
    }
}

int ssimu2_multi_pyramid(const Ssimu2MultiImage* imgs, const int4* items, int nitems, const Ssimu2Geom* geoms,
                         int intype, bool delta, cudaStream_t st) {
    if (nitems <= 0) return E_OK;
    ProfScope ps(delta ? "ssimu2_multi_pyramid_cand" : "ssimu2_multi_pyramid_src", st);
    if (delta)
        launch_multi_pyramid<true>(imgs, items, nitems, geoms, intype, st);
    else
        launch_multi_pyramid<false>(imgs, items, nitems, geoms, intype, st);
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

int ssimu2_multi_stats(const Ssimu2MultiPair* pairs, const int2* items, int nitems, const Ssimu2Geom* geoms,
                       bool delta, int grid, int shape, cudaStream_t st) {
    if (nitems <= 0) return E_OK;
    const unsigned gr = (unsigned)std::max(1, std::min(grid, nitems));
    ProfScope ps("ssimu2_multi_stats", st);
    const int smem = stats_smem(shape ? 1 : 0);
    if (shape == 0) {
        if (delta) ssimu2_multi_stats_kernel<true, 0><<<gr, 256, smem, st>>>(pairs, items, nitems, geoms);
        else ssimu2_multi_stats_kernel<false, 0><<<gr, 256, smem, st>>>(pairs, items, nitems, geoms);
    } else {
        if (delta) ssimu2_multi_stats_kernel<true, 1><<<gr, 256, smem, st>>>(pairs, items, nitems, geoms);
        else ssimu2_multi_stats_kernel<false, 1><<<gr, 256, smem, st>>>(pairs, items, nitems, geoms);
    }
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

int ssimu2_multi_finalize(const Ssimu2MultiPair* pairs, int npairs, const Ssimu2Geom* geoms, cudaStream_t st) {
    if (npairs <= 0) return E_OK;
    ProfScope ps("ssimu2_multi_finalize", st);
    ssimu2_multi_finalize_kernel<<<(unsigned)npairs, kFinThreads, 0, st>>>(pairs, geoms);
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

}  // namespace vship
