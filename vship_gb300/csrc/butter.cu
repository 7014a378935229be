// butter.cu -- Butteraugli scoring on sm_103a.
//
// Launch sequence for a batch of frame pairs (reference file:line per step):
//   decode      : strided input -> linear RGB at full and half resolution
//                 (butter/Planed.hpp:3-34, colors.hpp:7-23, downupsample.hpp:3-20, main.hpp:116-128)
//   then for the half scale and the full scale:
//   opsin       : 17-tap blur (sigma 1.2) of each channel in a 32x48 smem tile + opsin dynamics
//                 (colors.hpp:25-91)
//   lf_h, lf_v  : separable 43-tap blur (sigma 7.156); the vertical pass also forms D = XYB - LF
//                 and the LF "vals" (separatefrequencies.hpp:3-12,160-203)
//   mf          : separable 19-tap blur (sigma 3.225) of D, both passes in one kernel (the
//                 horizontal pass's rows stay in shared memory); forms MF with its range operators
//                 and HF_pre = D - MF with X suppressed by Y (:37-99)
//   hf          : 17-tap tile blur (sigma 1.564) of HF_pre -> HF and UHF (:117-140,189-200)
//   diff        : the six Malta maps from a register window over a smem tile of the asymmetric
//                 diffs, the L2 / L2-asymmetric terms and the mask precompute
//                 (maltaDiff.hpp, simplerdiff.hpp, maskPsycho.hpp:3-40, main.hpp:45-93)
//   mask_blur   : 17-tap tile blur (sigma 2.7) of both mask planes, adds 10*(B0-B1)^2
//                 (maskPsycho.hpp:113-135)
//   diffmap     : fuzzy erosion, MaskY/MaskDcY combine (combineMasks.hpp); at full scale also
//                 the 2x supersampled add of the half-scale map, the distortion-map store and the
//                 per-CTA norm partials (downupsample.hpp:287-301, diffnorms.hpp)
//   finalize    : FP64 p-norm / 3-norm / max combine (diffnorms.hpp:263-306)
#include "common.cuh"
#include "butter.h"
#include "profile.h"

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

namespace vship {

// ------------------------------------------------------------------------------------------
// Gaussian tables (butter/gaussianblur.hpp:3-14,21-42), built on the host with the reference's
// float arithmetic: index 0..4 = sigma {1.2, 1.56416327805, 2.7, 3.22489901262, 7.15593339443},
// radius {8, 8, 8, 9, 21}.
__constant__ float c_bk[5][43];
__constant__ float c_bI[5][44];
__constant__ float c_bInvIn[5];  // 1 / (full window mass): the renormalisation of interior outputs
__constant__ f2_t c_bk2_t[3][17];  // the radius-8 kernels' taps (index 0..2) as {k, k} pairs

static int upload_butter_tables() {
    static const double sig[5] = {1.2, 1.56416327805, 2.7, 3.22489901262, 7.15593339443};
    float k[5][43] = {}, I[5][44] = {};
    for (int t = 0; t < 5; t++) {
        const double sigma = sig[t];
        const int R = std::max((int)(sigma * 3), 8);
        const int n = 2 * R + 1;
        float acc = 0.f;
        for (int i = 0; i <= n; i++) {
            double q = (double)std::exp((float)(-(R - i) * (R - i) / (2 * sigma * sigma))) /
                       std::sqrt(6.28318530718 * sigma * sigma);
            if (i < n) k[t][i] = (float)q;
            I[t][i] = acc;
            acc = (float)((double)acc + q);
        }
    }
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_bk, k, sizeof(k)));
    float k2t[3][34];
    for (int t = 0; t < 3; t++)
        for (int i = 0; i < 17; i++) k2t[t][2 * i] = k2t[t][2 * i + 1] = k[t][i];
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_bk2_t, k2t, sizeof(k2t)));
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_bI, I, sizeof(I)));
    float inv[5];
    for (int t = 0; t < 5; t++) {
        const int n = 2 * std::max((int)(sig[t] * 3), 8) + 1;
        inv[t] = 1.0f / (I[t][n] - I[t][0]);  // the same float division b_inv_mass makes
    }
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_bInvIn, inv, sizeof(inv)));
    return E_OK;
}

template <int KI, int R>
__device__ __forceinline__ float b_inv_mass(int pos, int extent) {
    const int beg = max(0, pos - R) - (pos - R);
    const int end = min(extent, pos + R + 1) - (pos - R);
    return 1.0f / (c_bI[KI][end] - c_bI[KI][beg]);
}
// The same for n consecutive positions p0 .. p0+n-1: positions whose whole window lies inside
// the extent share the interior value (beg = 0, end = 2R + 1), divided once on the host.
template <int KI, int R, int N>
__device__ __forceinline__ void b_inv_mass_run(int p0, int extent, float out[N]) {
    if (p0 >= R && p0 + N - 1 + R < extent) {
        const float v = c_bInvIn[KI];
#pragma unroll
        for (int o = 0; o < N; o++) out[o] = v;
    } else {
#pragma unroll
        for (int o = 0; o < N; o++) out[o] = b_inv_mass<KI, R>(p0 + o, extent);
    }
}

// ------------------------------------------------------------------------------------------
// Workspace layout. Every image (a reference / source or a distorted / candidate frame) owns, per
// scale, NIMG dense planes of pitch p; a scored pair reads its two images' planes and writes its
// own planes into planes of the distorted image that are dead by then, so that an image shared by
// several pairs (a source scored against several candidates) is read-only after its own stage.
enum : int {
    I_LIN = 0,    // 0..2   linear RGB; dead after opsin
    I_TMP = 0,    // 0..2   the LF horizontal pass's output (reuses LIN); dead after lf_v
    I_XYB = 3,    // 3..5   XYB, then D = XYB - LF (in place); dead after the MF kernel
    I_HFP = 0,    // 0..1   HF_pre (X, Y), written by the MF kernel over TMP; dead after hf
    I_LFV = 6,    // 6..8   LF vals
    I_MF = 9,     // 9..11  MF
    I_HF = 12,    // 12..13 HF (X, Y)
    I_UHF = 14,   // 14..15 UHF (X, Y)
    NIMG = 16,
    I_PRE = 2,    // 2      the image's mask precompute (hf), in the dead TMP[2] plane
    // pair planes, inside the distorted image's dead TMP and XYB planes
    Q_SAC = 0,    // sum of AC terms            } written by diff
    Q_SDC = 1,    // sum of DC terms            }
    Q_B0 = 4,     // blurred mask of image 0 (mask_blur)
    Q_DIFF = 5    // diffmap of this scale (diffmap)
};

struct BScaleDev {
    int w, h, p;
    int64_t n;     // p*h
    int64_t base;  // offset inside the image's workspace
};
struct BGeom {
    BScaleDev s[2];  // 0 = full, 1 = half
    int64_t img_floats;
    int half_bands;  // UHF stored as FP16 (hplane); the other planes stay FP32
    int norm_tiles_x, norm_tiles;  // final-kernel tiling (32x32) at full scale
};

// ib[img] = that image's workspace (both scales); the launch's image list indexes it
__device__ __forceinline__ float* iplane(float* const* ib, const BGeom& g, const BScaleDev& S, int img, int id) {
    return ib[img] + S.base + (int64_t)id * S.n;
}
// Half-band storage: the UHF bands (X, Y), which only the pair stage reads, are kept as FP16 in a
// block after the fourteen FP32 planes; plane `id` in [I_UHF, I_UHF + 1] is the (id - I_UHF)-th
// half plane of the block, with the FP32 planes' element pitch. FP16 storage of the HF or MF bands
// moves the norms by more than 1e-4 relative on some frames (a stored value's relative step is
// 2^-11, and the Malta maps square differences of nearby values); of the UHF bands it does not.
__device__ __forceinline__ __half* hplane(float* const* ib, const BScaleDev& S, int img, int id) {
    return reinterpret_cast<__half*>(ib[img] + S.base + (int64_t)I_UHF * S.n) + (int64_t)(id - I_UHF) * S.n;
}
// A plane is FP16 when the form stores half bands and it is a UHF plane (ids are compile-time
// constants at every call site, so the test folds away).
__device__ __forceinline__ constexpr bool half_plane(bool hb, int id) { return hb && id >= I_UHF; }
template <bool HB>
__device__ __forceinline__ void band_store(float* const* ib, const BGeom& g, const BScaleDev& S, int img, int id,
                                           int64_t i, float v) {
    if (half_plane(HB, id))
        hplane(ib, S, img, id)[i] = __float2half_rn(v);
    else
        iplane(ib, g, S, img, id)[i] = v;
}
// Select a scale with constant indices only, so the parameter struct is never copied to the
// stack for a dynamic index.
__device__ __forceinline__ BScaleDev pick_scale(const BGeom& g, int s) { return s == 0 ? g.s[0] : g.s[1]; }

// ------------------------------------------------------------------------------------------
// Kernel: decode + linearise at full resolution + 2x2 box to half resolution.
// grid (ceil(w/32), ceil(h/32), nimages), 256 threads; frames[image].
template <int IT>
__global__ void __launch_bounds__(256, IT == IN_YUV ? 6 : 8) butter_decode_kernel(const FrameDesc* __restrict__ frames,
                                                            float* const* __restrict__ ib, BGeom g, YuvParams yp) {
    __shared__ float sm[3][32][33];
    const int img = blockIdx.z;
    const FrameDesc fd = frames[img];
    const BScaleDev F = g.s[0], Hs = g.s[1];
    const bool vec = rgb4_vectorizable<IT>(fd);
    if (IT == IN_YUV || vec) {
        // four adjacent pixels of one row per thread (load_rgb4), stored as one float4 per plane
        const int ly = threadIdx.x >> 3, lx = 4 * (threadIdx.x & 7);
        const int gx = blockIdx.x * 32 + lx, gy = blockIdx.y * 32 + ly;
        float v[3][4] = {};
        if (gx < F.w && gy < F.h) {
            load_rgb4<IT>(fd, yp, gx, gy, F.w, F.h, vec, v);
#pragma unroll
            for (int c = 0; c < 3; c++) {
#pragma unroll
                for (int i = 0; i < 4; i++)
                    if (!(IT == IN_YUV && yp.linear_out)) v[c][i] = gx + i < F.w ? to_linear_fast<IT>(v[c][i]) : 0.f;
                float* d = iplane(ib, g, F, img, I_LIN + c) + (int64_t)gy * F.p + gx;
                if (gx + 3 < F.w) {
                    *reinterpret_cast<float4*>(d) = make_float4(v[c][0], v[c][1], v[c][2], v[c][3]);
                } else {
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        if (gx + i < F.w) d[i] = v[c][i];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int i = 0; i < 4; i++) sm[c][ly][lx + i] = v[c][i];
    } else {
        const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int ly = ty + 8 * r;
            const int gx = blockIdx.x * 32 + tx, gy = blockIdx.y * 32 + ly;
            float v[3] = {0.f, 0.f, 0.f};
            if (gx < F.w && gy < F.h) {
                load_rgb<IT>(fd, yp, gx, gy, F.w, F.h, v[0], v[1], v[2]);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if (!(IT == IN_YUV && yp.linear_out)) v[c] = to_linear_fast<IT>(v[c]);
                    iplane(ib, g, F, img, I_LIN + c)[(int64_t)gy * F.p + gx] = v[c];
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) sm[c][ly][tx] = v[c];
        }
    }
    __syncthreads();
    const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;
    const int gx = blockIdx.x * 16 + lx, gy = blockIdx.y * 16 + ly;
    if (gx < Hs.w && gy < Hs.h) {
        const int x0 = 2 * lx, y0 = 2 * ly;
        const int x1 = min(2 * gx + 1, F.w - 1) - (int)blockIdx.x * 32;
        const int y1 = min(2 * gy + 1, F.h - 1) - (int)blockIdx.y * 32;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float s = sm[c][y0][x0];
            s += sm[c][y1][x0];
            s += sm[c][y0][x1];
            s += sm[c][y1][x1];
            iplane(ib, g, Hs, img, I_LIN + c)[(int64_t)gy * Hs.p + gx] = s * 0.25f;
        }
    }
}

// ------------------------------------------------------------------------------------------
// 2-D tile blur, radius 8: 32x48 outputs per 256-thread CTA. The 64x48 input tile (8-px halo,
// zero outside the image) is staged with cp.async into rows of TB_IP floats; the horizontal pass
// reads each thread's 24 inputs as six float4 (a warp takes 32 consecutive rows of one column
// group; pitch 52 = 13 quads: the 8 lanes of a quarter-warp phase hit distinct bank quads) and
// writes its 8 sums into the column-major buffer `hb` (column x at hb[x * TB_HC], pitch 66: the
// warp's stores hit 32 consecutive words); each thread then reads the 22 rows of column
// (tid & 31) it needs as 11 float2 (66 / 2 odd: a half-warp's 8-byte loads cover all 32 banks) and
// returns the 6 vertical outputs, rows 6*(tid>>5)+o, scaled by the product of both passes'
// border renormalisations (gaussianblur.hpp:94-186 divides after each pass).
constexpr int TB_TW = 32, TB_TH = 48, TB_R = 8;
constexpr int TB_IW = TB_TW + 2 * TB_R, TB_IH = TB_TH + 2 * TB_R;
constexpr int TB_IP = 52, TB_HC = 66;
constexpr int TB_RAW = TB_IH * TB_IP;
constexpr int TB_HPL = TB_TW * TB_HC;

__device__ __forceinline__ void tile_stage_r8(float* dst, const float* __restrict__ plane, int pitch, int w, int h,
                                              int x0, int y0) {
    stage_tile_t<TB_IH, TB_IW / 4>(dst, TB_IP, plane, pitch, w, h, x0 - TB_R, y0 - TB_R);
}

template <int KI>
__device__ __forceinline__ void tile_blur_r8(const float* in, float* hb, const float rxy[6], float out[6]) {
    const int tid = threadIdx.x;
    {
        const int hr = 32 * ((tid >> 5) & 1) + (tid & 31), hg = tid >> 6;
        const float* row = in + hr * TB_IP + 8 * hg;
        float v[24];
#pragma unroll
        for (int j4 = 0; j4 < 6; j4++) {
            const float4 q = *reinterpret_cast<const float4*>(row + 4 * j4);
            v[4 * j4] = q.x;
            v[4 * j4 + 1] = q.y;
            v[4 * j4 + 2] = q.z;
            v[4 * j4 + 3] = q.w;
        }
        float* dst = hb + (8 * hg) * TB_HC + hr;
#pragma unroll
        for (int o = 0; o < 8; o++) {
            float a = 0.f;
#pragma unroll
            for (int i = 0; i < 17; i++) a = fmaf(v[o + i], c_bk[KI][i], a);
            dst[o * TB_HC] = a;
        }
    }
    __syncthreads();
    {
        const int vc = tid & 31, vg = tid >> 5;
        const float2* col = reinterpret_cast<const float2*>(hb + vc * TB_HC + 6 * vg);
        float v[22];
#pragma unroll
        for (int j = 0; j < 11; j++) {
            const float2 q = col[j];
            v[2 * j] = q.x;
            v[2 * j + 1] = q.y;
        }
#pragma unroll
        for (int o = 0; o < 6; o++) {
            float a = 0.f;
#pragma unroll
            for (int i = 0; i < 17; i++) a = fmaf(v[o + i], c_bk[KI][i], a);
            out[o] = a * rxy[o];
        }
    }
}

// tile_blur_r8 on two planes at once, as f32x2 pairs (one instruction for both lanes, each
// rounded as the scalar FMA, so the values are those of two tile_blur_r8 calls). hb2 holds
// TB_TW x TB_HC {a, b} pairs, column-major (66 pairs = 33 quads per column, odd).
template <int KI>
__device__ __forceinline__ void tile_blur_r8_x2(const float* in0, const float* in1, float* hb2, const float rxy[6],
                                                float out0[6], float out1[6]) {
    const int tid = threadIdx.x;
    {
        const int hr = 32 * ((tid >> 5) & 1) + (tid & 31), hg = tid >> 6;
        const float* r0 = in0 + hr * TB_IP + 8 * hg;
        const float* r1 = in1 + hr * TB_IP + 8 * hg;
        float v0[24], v1[24];
#pragma unroll
        for (int j4 = 0; j4 < 6; j4++) {
            const float4 q0 = *reinterpret_cast<const float4*>(r0 + 4 * j4);
            const float4 q1 = *reinterpret_cast<const float4*>(r1 + 4 * j4);
            v0[4 * j4] = q0.x;
            v0[4 * j4 + 1] = q0.y;
            v0[4 * j4 + 2] = q0.z;
            v0[4 * j4 + 3] = q0.w;
            v1[4 * j4] = q1.x;
            v1[4 * j4 + 1] = q1.y;
            v1[4 * j4 + 2] = q1.z;
            v1[4 * j4 + 3] = q1.w;
        }
        f2_t a[8];
#pragma unroll
        for (int o = 0; o < 8; o++) a[o] = f2_pack(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 24; j++) {
            const f2_t p = f2_pack(v0[j], v1[j]);
#pragma unroll
            for (int o = 0; o < 8; o++) {
                const int i = j - o;  // tap index, ascending for each output
                if (i >= 0 && i < 17) a[o] = f2_fma(p, c_bk2_t[KI][i], a[o]);
            }
        }
        f2_t* dst = reinterpret_cast<f2_t*>(hb2) + (8 * hg) * TB_HC + hr;
#pragma unroll
        for (int o = 0; o < 8; o++) dst[o * TB_HC] = a[o];
    }
    __syncthreads();
    {
        const int vc = tid & 31, vg = tid >> 5;
        const ulonglong2* col = reinterpret_cast<const ulonglong2*>(reinterpret_cast<const f2_t*>(hb2) + vc * TB_HC + 6 * vg);
        f2_t a[6];
#pragma unroll
        for (int o = 0; o < 6; o++) a[o] = f2_pack(0.f, 0.f);
#pragma unroll
        for (int jj = 0; jj < 11; jj++) {
            const ulonglong2 q = col[jj];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = 2 * jj + h;
                const f2_t v = h ? q.y : q.x;
#pragma unroll
                for (int o = 0; o < 6; o++) {
                    const int i = j - o;
                    if (i >= 0 && i < 17) a[o] = f2_fma(v, c_bk2_t[KI][i], a[o]);
                }
            }
        }
#pragma unroll
        for (int o = 0; o < 6; o++) f2_unpack(f2_mul(a[o], f2_pack(rxy[o], rxy[o])), out0[o], out1[o]);
    }
}

template <int KI>
__device__ __forceinline__ void tile_masses_r8(int x0, int y0, int w, int h, float rxy[6]) {
    const int tid = threadIdx.x;
    const int x = x0 + (tid & 31);
    const float rx = (x >= 8 && x + 8 < w) ? c_bInvIn[KI] : b_inv_mass<KI, 8>(x, w);
    float ry[6];
    b_inv_mass_run<KI, 8, 6>(y0 + 6 * (tid >> 5), h, ry);
#pragma unroll
    for (int o = 0; o < 6; o++) rxy[o] = rx * ry[o];
}

// ------------------------------------------------------------------------------------------
// opsin dynamics (butter/colors.hpp:3-5,25-79)
__device__ __forceinline__ void b_opsin(float& x, float& y, float& z, bool clamp) {
    float ox = fmaf(0.29956550340058319f, x, fmaf(0.63373087833825936f, y, fmaf(0.077705617820981968f, z, 1.7557483643287353f)));
    float oy = fmaf(0.22158691104574774f, x, fmaf(0.69391388044116142f, y, fmaf(0.0987313588422f, z, 1.7557483643287353f)));
    float oz = fmaf(0.02f, x, fmaf(0.02f, y, fmaf(0.20480129041026129f, z, 12.226454707163354f)));
    if (clamp) {
        ox = fmaxf(ox, 1.7557483643287353f);
        oy = fmaxf(oy, 1.7557483643287353f);
        oz = fmaxf(oz, 12.226454707163354f);
    }
    x = ox;
    y = oy;
    z = oz;
}
__device__ __forceinline__ float b_gamma(float v) {
    // logf(x) as log2(x) * ln 2 (x >= 9.97 here, so the approximation's absolute log2 error of
    // ~2^-22 is ~1e-7 relative). The reference adds the double literal and rounds the sum to
    // float; the float sum here is at most 1 ulp from it, below the log approximation's error.
    return fmaf(19.245013259874995f, lg2_approx(v + 9.9710635769299145f) * 0.69314718055994531f,
                -23.16046239805755f);
}

// grid (ceil(w/32), ceil(h/48), nimages); the three channels' tiles are double-buffered.
__global__ void __launch_bounds__(256, 5) butter_opsin_kernel(float* const* __restrict__ ib, BGeom g, int s,
                                                              float intensity) {
    extern __shared__ __align__(16) float sm[];
    float* hb = sm + 2 * TB_RAW;
    const int img = blockIdx.z;
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * TB_TW, y0 = blockIdx.y * TB_TH;
    float rxy[6];
    tile_masses_r8<0>(x0, y0, S.w, S.h, rxy);
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    float src[3][6], blr[3][6];
    tile_stage_r8(sm, iplane(ib, g, S, img, I_LIN), S.p, S.w, S.h, x0, y0);
    cp_async_commit();
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float* in = sm + (c & 1) * TB_RAW;
        if (c < 2) {
            tile_stage_r8(sm + ((c + 1) & 1) * TB_RAW, iplane(ib, g, S, img, I_LIN + c + 1), S.p, S.w, S.h, x0,
                          y0);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        tile_blur_r8<0>(in, hb, rxy, blr[c]);
#pragma unroll
        for (int o = 0; o < 6; o++) src[c][o] = in[(6 * vg + o + TB_R) * TB_IP + vc + TB_R];
        __syncthreads();
    }
    float* ox = iplane(ib, g, S, img, I_XYB + 0);
    float* oy = iplane(ib, g, S, img, I_XYB + 1);
    float* oz = iplane(ib, g, S, img, I_XYB + 2);
#pragma unroll
    for (int o = 0; o < 6; o++) {
        const int x = x0 + vc, y = y0 + 6 * vg + o;
        if (x < S.w && y < S.h) {
            float sx = src[0][o] * intensity, sy = src[1][o] * intensity, sz = src[2][o] * intensity;
            float bx = blr[0][o] * intensity, by = blr[1][o] * intensity, bz = blr[2][o] * intensity;
            b_opsin(bx, by, bz, true);
            bx = fmaxf(bx, 1e-4f);
            by = fmaxf(by, 1e-4f);
            bz = fmaxf(bz, 1e-4f);
            const float ex = fmaxf(__fdividef(b_gamma(bx), bx), 1e-4f);
            const float ey = fmaxf(__fdividef(b_gamma(by), by), 1e-4f);
            const float ez = fmaxf(__fdividef(b_gamma(bz), bz), 1e-4f);
            b_opsin(sx, sy, sz, false);
            sx *= ex;
            sy *= ey;
            sz *= ez;
            sx = fmaxf(sx, 1.7557483643287353f);
            sy = fmaxf(sy, 1.7557483643287353f);
            sz = fmaxf(sz, 12.226454707163354f);
            const int64_t i = (int64_t)y * S.p + x;
            ox[i] = sx - sy;
            oy[i] = sx + sy;
            oz[i] = sz;
        }
    }
}

// ------------------------------------------------------------------------------------------
// Separable horizontal pass of radius R (R = 21: the LF band's 43 taps): 128x16 row tiles; each
// thread makes 8 consecutive outputs of a tile. The input rows start at x0 - RA (RA = R rounded
// up to a multiple of 4, so the cp.async chunks are 16-byte aligned) and are read back as float4
// (pitch 180 = 45 quads: conflict-free); the thread's window starts RA - R floats into its first
// quad. A CTA
// walks HB_NT row tiles down the column, staging tile t + 1 while it computes tile t, so the
// global-load latency hides behind the taps of the previous tile.
// grid (ceil(w/128), ceil(h/(16*HB_NT)), 3*nimages): z -> image = z/3, plane = src_id + z%3.
// HB_NT: 16 row tiles (256 rows) per CTA; 4 of them measured 4 % slower (more CTAs, each
// paying its first tile's staging latency unhidden)
constexpr int HB_TW = 128, HB_TH = 16, HB_P = 180, HB_NT = 16;

template <int KI, int R>
__global__ void __launch_bounds__(256, 3) butter_hblur_kernel(float* const* __restrict__ ib, BGeom g, int s,
                                                              int src_id, int dst_id) {
    __shared__ __align__(16) float in[2][HB_TH * HB_P];
    constexpr int RA = (R + 3) & ~3;
    constexpr int IW = HB_TW + 2 * RA;
    constexpr int OFF = RA - R;
    constexpr int NV4 = (OFF + 8 + 2 * R + 3) / 4;
    static_assert(IW <= HB_P && 120 + 4 * NV4 <= HB_P, "hblur tile");
    const int img = blockIdx.z / 3, pl = blockIdx.z % 3;
    const BScaleDev S = pick_scale(g, s);
    const float* src = iplane(ib, g, S, img, src_id + pl);
    float* dst = iplane(ib, g, S, img, dst_id + pl);
    const int x0 = blockIdx.x * HB_TW;
    const int yt0 = blockIdx.y * (HB_TH * HB_NT);
    const int nt = min(HB_NT, (S.h - yt0 + HB_TH - 1) / HB_TH);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = (warp >> 2) * 8 + (lane >> 2);
    const int col0 = (warp & 3) * 32 + 8 * (lane & 3);
    float rx[8];
    b_inv_mass_run<KI, R, 8>(x0 + col0, S.w, rx);
    stage_tile_t<HB_TH, IW / 4>(in[0], HB_P, src, S.p, S.w, S.h, x0 - RA, yt0);
    cp_async_commit();
#pragma unroll 1
    for (int t = 0; t < nt; t++) {
        if (t + 1 < nt) {
            stage_tile_t<HB_TH, IW / 4>(in[(t + 1) & 1], HB_P, src, S.p, S.w, S.h, x0 - RA, yt0 + (t + 1) * HB_TH);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int gy = yt0 + t * HB_TH + row;
        if (gy < S.h) {
            const float* tin = in[t & 1];
            float v[4 * NV4];
#pragma unroll
            for (int j4 = 0; j4 < NV4; j4++) {
                const float4 q = *reinterpret_cast<const float4*>(tin + row * HB_P + col0 + 4 * j4);
                v[4 * j4] = q.x;
                v[4 * j4 + 1] = q.y;
                v[4 * j4 + 2] = q.z;
                v[4 * j4 + 3] = q.w;
            }
            float out[8];
#pragma unroll
            for (int o = 0; o < 8; o++) {
                float a = 0.f;
#pragma unroll
                for (int i = 0; i < 2 * R + 1; i++) a = fmaf(v[OFF + o + i], c_bk[KI][i], a);
                out[o] = a * rx[o];
            }
            float* d = dst + (int64_t)gy * S.p + x0 + col0;
            if (x0 + col0 + 8 <= S.p) {  // rows are padded to a multiple of 8 floats
                *reinterpret_cast<float4*>(d) = make_float4(out[0], out[1], out[2], out[3]);
                *reinterpret_cast<float4*>(d + 4) = make_float4(out[4], out[5], out[6], out[7]);
            }
        }
        __syncthreads();  // every thread is done with in[t & 1] before tile t + 2 is staged into it
    }
}

// Separable vertical pass over the three channels of one image: 32x64 tile, each thread makes
// 8 consecutive rows of one column for every channel, then runs the fused epilogue.
// grid (ceil(w/32), ceil(h/64), nimages).
constexpr int VB_TW = 32, VB_TH = 64;

template <int KI, int R>
__device__ __forceinline__ void vblur3(float* in, float* ctr, float* const* __restrict__ ib, const BGeom& g, int img,
                                       int s, int src_id, int ctr_id, int nctr, float out[3][8]) {
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * VB_TW, y0 = blockIdx.y * VB_TH;
    constexpr int IH = VB_TH + 2 * R;
#pragma unroll
    for (int c = 0; c < 3; c++)
        stage_tile_t<IH, VB_TW / 4>(in + c * IH * VB_TW, VB_TW, iplane(ib, g, S, img, src_id + c), S.p, S.w, S.h, x0,
                                    y0 - R);
    // the epilogue's own-pixel planes, staged with the blur input so their latency overlaps
    for (int c = 0; c < nctr; c++)
        stage_tile_t<VB_TH, VB_TW / 4>(ctr + c * VB_TH * VB_TW, VB_TW, iplane(ib, g, S, img, ctr_id + c), S.p, S.w,
                                       S.h, x0, y0);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    float ry[8];
    b_inv_mass_run<KI, R, 8>(y0 + 8 * vg, S.h, ry);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float* col = in + c * IH * VB_TW + (8 * vg) * VB_TW + vc;
        float v[8 + 2 * R];
#pragma unroll
        for (int j = 0; j < 8 + 2 * R; j++) v[j] = col[j * VB_TW];
#pragma unroll
        for (int o = 0; o < 8; o++) {
            float a = 0.f;
#pragma unroll
            for (int i = 0; i < 2 * R + 1; i++) a = fmaf(v[o + i], c_bk[KI][i], a);
            out[c][o] = a * ry[o];
        }
    }
}

// LF vertical pass: D = XYB - LF (in place over XYB) and LF vals (separatefrequencies.hpp:3-12)
constexpr int kVLfSmem = (3 * (VB_TH + 42) * VB_TW + 3 * VB_TH * VB_TW) * 4;
__global__ void __launch_bounds__(256) butter_lf_v_kernel(float* const* __restrict__ ib, BGeom g, int s) {
    extern __shared__ __align__(16) float sm[];
    float* ctr = sm + 3 * (VB_TH + 42) * VB_TW;
    const int img = blockIdx.z;
    float lf[3][8];
    vblur3<4, 21>(sm, ctr, ib, g, img, s, I_TMP, I_XYB, 3, lf);
    const BScaleDev S = pick_scale(g, s);
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    const int x = blockIdx.x * VB_TW + vc;
    const int yb = blockIdx.y * VB_TH + 8 * vg;
    if (x >= S.w) return;
    float* xyb[3];
    float* lfv[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        xyb[c] = iplane(ib, g, S, img, I_XYB + c);
        lfv[c] = iplane(ib, g, S, img, I_LFV + c);
    }
#pragma unroll
    for (int o = 0; o < 8; o++) {
        const int y = yb + o;
        if (y < S.h) {
            const int64_t i = (int64_t)y * S.p + x;
#pragma unroll
            for (int c = 0; c < 3; c++) xyb[c][i] = ctr[(c * VB_TH + 8 * vg + o) * VB_TW + vc] - lf[c][o];
            float vx = lf[0][o], vy = lf[1][o], vb = lf[2][o];
            vb = vb + -0.362267051518f * vy;
            vb = vb * 49.87984651440f;
            vx = vx * 33.832837186260f;
            vy = vy * 14.458268100570f;
            lfv[0][i] = vx;
            lfv[1][i] = vy;
            lfv[2][i] = vb;
        }
    }
}

// The range operators (separatefrequencies.hpp) through the clamp c of x to [-w, w]: above w the
// reference's x + w / x - w, below -w its x - w / x + w (x + (-w), x - (-w): the same IEEE
// operations), inside 2x == x + x and x - x == 0. Same values for finite x, three instructions
// instead of six.
__device__ __forceinline__ float amplify_range(float x, float w) { return x + fminf(fmaxf(x, -w), w); }
__device__ __forceinline__ float remove_range(float x, float w) { return x - fminf(fmaxf(x, -w), w); }
// MaximumClamp (separatefrequencies.hpp) on the same clamp c: above maxval the reference's
// fma(v - maxval, kMul, maxval), below -maxval fma(v + maxval, kMul, -maxval) (v - (-maxval) is
// v + maxval), inside fma(0, kMul, v) == v (a zero's sign aside).
__device__ __forceinline__ float maximum_clamp(float v, float maxval) {
    const float kMul = 0.688059627878f;
    const float c = fminf(fmaxf(v, -maxval), maxval);
    return fmaf(v - c, kMul, c);
}

// MF band in one kernel: the separable 19-tap blur of the three D planes, then MF with the range
// operators and HF_pre = D - MF with X suppressed by Y (separatefrequencies.hpp:37-99,160-187).
// A CTA owns a 32-column strip of one image and walks MS_SEG rows of it in 64-row chunks. Per
// chunk the three channels' D rows are staged (cp.async, zeros outside the image), the horizontal
// pass writes its rows into a per-channel column-major buffer of 82 rows (the chunk's 64 and the
// 9-row halos) and keeps the X and Y values of the output pixels, the 18 rows a chunk shares with
// the next are carried over instead of blurred again, and the vertical pass runs the epilogue on
// all three channels while the next chunk's rows are being staged. The horizontal pass's rows
// never leave the SM: against a separate horizontal kernel (as the LF band still uses) this
// saves writing and re-reading three planes and the vertical pass's re-reads of its halo rows
// (201 -> 183 us per 3840x2160 pair). Taps, their order and the renormalisation are those of
// butter_hblur_kernel and vblur3 with the sigma-3.225 kernel, so the values are the same bit for
// bit as the two-pass form's. HF_pre goes to the dead TMP planes (I_HFP), not over D:
// neighbouring CTAs still read D in their halos.
// grid (ceil(w/32), ceil(h/MS_SEG), nimages)
constexpr int MS_TW = 32, MS_CH = 64, MS_R = 9, MS_RA = 12;  // RA: R rounded up to a multiple of 4
constexpr int MS_SEG = 8 * MS_CH;  // 512 rows: 2 % faster than 256 (fewer halo rows blurred twice)
constexpr int MS_HR = MS_CH + 2 * MS_R;   // 82 rows per chunk
constexpr int MS_IW = MS_TW + 2 * MS_RA;  // 56 staged columns, from x0 - 12
constexpr int MS_RP = 60;                 // staged row pitch: 15 quads (conflict-free float4 rows)
constexpr int MS_RAW = MS_HR * MS_RP;     // one channel's staged rows
// Horizontal-pass buffer, per channel column-major: column x starts at x * 84 + 8 * (x / 8). 84
// floats = 21 quads, odd, so the vertical pass's 16-byte loads of 8 neighbouring columns hit
// distinct bank quads; the 8-float step between column groups spreads the horizontal pass's
// stores of the four groups of a warp over all 32 banks.
constexpr int MS_HP = 84;
constexpr int MS_HPLANE = MS_TW * MS_HP + 8 * (MS_TW / 8 - 1);
// the X and Y D values of the chunk's own pixels (rows 0..63) and of the next chunk's first 9 rows
// (64..72), which only this chunk stages
constexpr int MS_CTRR = MS_CH + MS_R;
constexpr int MS_CTR = 2 * MS_CTRR * MS_TW;
constexpr int kMfSmem = (3 * MS_RAW + 3 * MS_HPLANE + MS_CTR) * 4;

__global__ void __launch_bounds__(256, 2) butter_mf_kernel(float* const* __restrict__ ib, BGeom g, int s) {
    extern __shared__ __align__(16) float sm[];
    float* raw = sm;                          // [channel][82 staged rows][60]
    float* hb = sm + 3 * MS_RAW;              // [channel][column-major buffer of 82 rows]
    float* ctr = hb + 3 * MS_HPLANE;          // [X, Y][73 rows][32 columns]
    const int img = blockIdx.z;
    const BScaleDev S = pick_scale(g, s);
    const int tx0 = blockIdx.x * MS_TW, sy0 = blockIdx.y * MS_SEG;
    const int nchunk = (min(MS_SEG, S.h - sy0) + MS_CH - 1) / MS_CH;
    const int tid = threadIdx.x, vc = tid & 31, vg = tid >> 5;
    // horizontal-pass tasks: output columns 8*hg .. 8*hg+7 of one staged row of one channel
    const int hg = tid & 3;
    float rx[8];
    b_inv_mass_run<3, MS_R, 8>(tx0 + 8 * hg, S.w, rx);
    const float sx = 0.653020556257f, yw = 46.0f;
    // staged row r is image row ty0 - 9 + r: a chunk's first staging takes rows 0..81, later ones
    // rows 18..81 (the new rows; rows 0..17 of the buffer are carried, and the epilogue's own
    // pixels are kept in ctr). The next chunk is staged as soon as this chunk's horizontal pass
    // is done, so its loads run under the vertical pass and the epilogue.
    auto stage = [&](int k) {
        const int ty0 = sy0 + k * MS_CH;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float* src = iplane(ib, g, S, img, I_XYB + c);
            if (k == 0)
                stage_tile_t<MS_HR, MS_IW / 4>(raw + c * MS_RAW, MS_RP, src, S.p, S.w, S.h, tx0 - MS_RA, ty0 - MS_R);
            else
                stage_tile_t<MS_CH, MS_IW / 4>(raw + c * MS_RAW + 2 * MS_R * MS_RP, MS_RP, src, S.p, S.w, S.h,
                                               tx0 - MS_RA, ty0 + MS_R);
        }
        cp_async_commit();
    };
    stage(0);
#pragma unroll 1
    for (int k = 0; k < nchunk; k++) {
        const int ty0 = sy0 + k * MS_CH;
        cp_async_wait<0>();
        __syncthreads();
        // horizontal pass: buffer rows 0..81 (first chunk) or 18..81, from the staged row of the
        // same index; the X and Y values of the output pixels (rows 9..72) go to ctr
        const int h0 = k == 0 ? 0 : 2 * MS_R;
        const int nrow = MS_HR - h0;
#pragma unroll 1
        for (int t = tid; t < 3 * nrow * 4; t += 256) {
            const int cr = t >> 2;
            const int c = cr / nrow, r = h0 + cr - c * nrow;
            const float* row = raw + c * MS_RAW + r * MS_RP + 8 * hg;
            float v[32];
#pragma unroll
            for (int j4 = 0; j4 < 8; j4++) {
                const float4 q = *reinterpret_cast<const float4*>(row + 4 * j4);
                v[4 * j4] = q.x;
                v[4 * j4 + 1] = q.y;
                v[4 * j4 + 2] = q.z;
                v[4 * j4 + 3] = q.w;
            }
            if (c < 2 && r >= MS_R) {
                float* cp = ctr + (c * MS_CTRR + r - MS_R) * MS_TW + 8 * hg;
                *reinterpret_cast<float4*>(cp) = make_float4(v[MS_RA], v[MS_RA + 1], v[MS_RA + 2], v[MS_RA + 3]);
                *reinterpret_cast<float4*>(cp + 4) = make_float4(v[MS_RA + 4], v[MS_RA + 5], v[MS_RA + 6], v[MS_RA + 7]);
            }
            float* d = hb + c * MS_HPLANE + 8 * hg * (MS_HP + 1) + r;
#pragma unroll
            for (int o = 0; o < 8; o++) {
                float a = 0.f;
#pragma unroll
                for (int i = 0; i < 2 * MS_R + 1; i++) a = fmaf(v[MS_RA - MS_R + o + i], c_bk[3][i], a);
                d[o * MS_HP] = a * rx[o];
            }
        }
        __syncthreads();
        if (k + 1 < nchunk) stage(k + 1);
        // vertical pass (column vc, rows 8*vg .. 8*vg+7 of the chunk, three channels) + epilogue
        float ry[8];
        b_inv_mass_run<3, MS_R, 8>(ty0 + 8 * vg, S.h, ry);
        float mf[3][8];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float4* col = reinterpret_cast<const float4*>(hb + c * MS_HPLANE + vc * MS_HP + 8 * (vc >> 3) + 8 * vg);
            float v[28];
#pragma unroll
            for (int j = 0; j < 7; j++) {
                const float4 q = col[j];
                v[4 * j] = q.x;
                v[4 * j + 1] = q.y;
                v[4 * j + 2] = q.z;
                v[4 * j + 3] = q.w;
            }
#pragma unroll
            for (int o = 0; o < 8; o++) {
                float a = 0.f;
#pragma unroll
                for (int i = 0; i < 2 * MS_R + 1; i++) a = fmaf(v[o + i], c_bk[3][i], a);
                mf[c][o] = a * ry[o];
            }
        }
        const int x = tx0 + vc;
        if (x < S.w) {
            float* h0p = iplane(ib, g, S, img, I_HFP + 0);
            float* h1p = iplane(ib, g, S, img, I_HFP + 1);
#pragma unroll
            for (int o = 0; o < 8; o++) {
                const int y = ty0 + 8 * vg + o;
                if (y < S.h) {
                    const int64_t i = (int64_t)y * S.p + x;
                    const int ci = (8 * vg + o) * MS_TW + vc;
                    float hx = ctr[ci] - mf[0][o];
                    const float hy = ctr[MS_CTRR * MS_TW + ci] - mf[1][o];
                    hx *= sx + div_nr(yw * (1.0f - sx), yw + hy * hy);
                    h0p[i] = hx;
                    h1p[i] = hy;
                    float* mfp = iplane(ib, g, S, img, I_MF);
                    mfp[i] = remove_range(mf[0][o], 0.29f);
                    mfp[S.n + i] = amplify_range(mf[1][o], 0.1f);
                    mfp[2 * S.n + i] = mf[2][o];
                }
            }
        }
        __syncthreads();  // buffer rows and ctr are rewritten for the next chunk
        if (k + 1 < nchunk) {
            // carry buffer rows 64..81 to rows 0..17: 3 channels x 32 columns x 9 row pairs
            for (int q = tid; q < 3 * MS_TW * 9; q += 256) {
                const int c = q / (MS_TW * 9), e = q - c * (MS_TW * 9), xx = e / 9, rp = e - xx * 9;
                float2* colp = reinterpret_cast<float2*>(hb + c * MS_HPLANE + xx * MS_HP + 8 * (xx >> 3));
                colp[rp] = colp[MS_CH / 2 + rp];
            }
            // and ctr rows 64..72 (the next chunk's first 9 rows) to rows 0..8
            for (int q = tid; q < 2 * MS_R * MS_TW; q += 256) {
                const int c = q / (MS_R * MS_TW), e = q - c * (MS_R * MS_TW);
                ctr[c * MS_CTRR * MS_TW + e] = ctr[(c * MS_CTRR + MS_CH) * MS_TW + e];
            }
        }
    }
}

// maskinit + diffPrecompute (maskPsycho.hpp:3-40) of one image: sqrt(m + b) - sqrt(b) evaluated as
// m / (sqrt(m + b) + sqrt(b)), the same value without the cancellation.
__device__ __forceinline__ float mask_precompute(float hf_x, float uhf_x, float hf_y, float uhf_y) {
    const float mul = 6.19424080439f;
    const float bias = mul * 12.61050594197f;
    const float xd = (uhf_x + hf_x) * 2.5f;
    const float yd = uhf_y * 0.4f + hf_y * 0.4f;
    const float mk = mul * sqrt_nr(xd * xd + yd * yd);
    return div_nr(mk, sqrt_nr(mk + bias) + sqrtf(bias));
}

// HF / UHF split (separatefrequencies.hpp:117-133,189-200) and the image's mask precompute, which
// depends on its own HF and UHF bands only (maskPsycho.hpp:3-40): computed here once per image
// from the FP32 band values (an image shared by several pairs is not recomputed per pair).
// grid (ceil(w/32), ceil(h/48), nimages)
template <bool HB>
__global__ void __launch_bounds__(256, 5) butter_hf_kernel(float* const* __restrict__ ib, BGeom g, int s) {
    extern __shared__ __align__(16) float sm[];
    float* hb2 = sm + 2 * TB_RAW;
    const int img = blockIdx.z;
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * TB_TW, y0 = blockIdx.y * TB_TH;
    float rxy[6];
    tile_masses_r8<1>(x0, y0, S.w, S.h, rxy);
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    tile_stage_r8(sm, iplane(ib, g, S, img, I_HFP), S.p, S.w, S.h, x0, y0);
    tile_stage_r8(sm + TB_RAW, iplane(ib, g, S, img, I_HFP + 1), S.p, S.w, S.h, x0, y0);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    float blr[2][6], pre[2][6];
    tile_blur_r8_x2<1>(sm, sm + TB_RAW, hb2, rxy, blr[0], blr[1]);
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
        for (int o = 0; o < 6; o++) pre[c][o] = sm[c * TB_RAW + (6 * vg + o + TB_R) * TB_IP + vc + TB_R];
#pragma unroll
    for (int o = 0; o < 6; o++) {
        const int x = x0 + vc, y = y0 + 6 * vg + o;
        float hfx = blr[0][o], uhfx = pre[0][o];
        uhfx -= hfx;
        hfx = remove_range(hfx, 1.5f);
        uhfx = remove_range(uhfx, 0.04f);
        float hf = blr[1][o], uhf = pre[1][o];
        hf = maximum_clamp(hf, 28.4691806922f);
        uhf -= hf;
        uhf = maximum_clamp(uhf, 5.19175294647f);
        uhf *= 2.69313763794f;
        hf *= 2.155f;
        hf = amplify_range(hf, 0.132f);
        if (x < S.w && y < S.h) {
            const int64_t i = (int64_t)y * S.p + x;
            band_store<HB>(ib, g, S, img, I_HF + 0, i, hfx);
            band_store<HB>(ib, g, S, img, I_UHF + 0, i, uhfx);
            band_store<HB>(ib, g, S, img, I_HF + 1, i, hf);
            band_store<HB>(ib, g, S, img, I_UHF + 1, i, uhf);
            iplane(ib, g, S, img, I_PRE)[i] = mask_precompute(hfx, uhfx, hf, uhf);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Malta difference (butter/maltaDiff.hpp). Parameters per map, derived on the host in float as
// MaltaDiffMap[_LF]_Kernel derives them (:528-535).
struct MaltaMap {
    float norm1, n2gt, n2lt;
};
struct DiffParams {
    MaltaMap mm[6];
    float l2asym_gt[2], l2asym_lt[2];  // already including the inner x0.8 (simplerdiff.hpp:297-298)
    float wmf[3], wlf[3];
};
__constant__ DiffParams c_dp;

__device__ __forceinline__ float malta_pre(float a, float b, const MaltaMap& m) {
    const float absval = 0.5f * fabsf(a) + 0.5f * fabsf(b);
    const float diff = a - b;
    const float inv = rcp_nr(m.norm1 + absval);  // one reciprocal for both scalers (norm1 >= 5)
    const float scaler = m.n2gt * inv;
    float v = scaler * diff;
    const float scaler2 = m.n2lt * inv;
    const float fabs0 = fabsf(a);
    const float too_small = 0.55f * fabs0, too_big = 1.05f * fabs0;
    // maltaDiff.hpp's two sign branches as one, on b mirrored to a's side: for a < 0 the
    // reference's b + too_small and -b - too_big are too_small - (-b) and (-b) - too_big, the same
    // IEEE operations, so the value is bitwise the same without divergent branches
    const float bm = a < 0.0f ? -b : b;
    // bm < too_small <= too_big gives (too_small - bm) + 0, bm > too_big gives 0 + (bm - too_big),
    // anything between 0 + 0: the reference's nested selects, term for term
    const float impact = (fmaxf(too_small - bm, 0.0f) + fmaxf(bm - too_big, 0.0f)) * scaler2;
    // v - impact for diff < 0, else v + impact, as one add of impact with diff's sign (impact >= 0;
    // the two forms differ only for diff == -0, where impact is 0 and only the sign of a zero
    // changes)
    return v + copysignf(impact, diff);
}

// The 16 line patterns, as (dx, dy) taps in the reference's order (maltaDiff.hpp:4-512, after
// google butteraugli). W(dx,dy) reads the register window at output row o. In the 5-tap bodies,
// parentheses group the centre triples that three patterns share, so each is formed once per
// output (14 of the 64 additions; the sums differ from the reference's left-to-right FP32 order
// by rounding only). The 9-tap bodies keep the reference's order: grouping their shared runs
// too holds more partial sums live than the 80 registers allow and measured slower.
#define W(dx, dy) win[(o) + 4 + (dy)][4 + (dx)]
#define SQ(expr)          \
    {                     \
        float s_ = (expr); \
        ret = fmaf(s_, s_, ret); \
    }
#define MALTA_HF_BODY                                                                                       \
    SQ(W(-4, 0) + W(-3, 0) + W(-2, 0) + W(-1, 0) + W(0, 0) + W(1, 0) + W(2, 0) + W(3, 0) + W(4, 0))        \
    SQ(W(0, -4) + W(0, -3) + W(0, -2) + W(0, -1) + W(0, 0) + W(0, 1) + W(0, 2) + W(0, 3) + W(0, 4))        \
    SQ(W(-3, -3) + W(-2, -2) + W(-1, -1) + W(0, 0) + W(1, 1) + W(2, 2) + W(3, 3))                          \
    SQ(W(3, -3) + W(2, -2) + W(1, -1) + W(0, 0) + W(-1, 1) + W(-2, 2) + W(-3, 3))                          \
    SQ(W(1, -4) + W(1, -3) + W(1, -2) + W(0, -1) + W(0, 0) + W(0, 1) + W(-1, 2) + W(-1, 3) + W(-1, 4))     \
    SQ(W(-1, -4) + W(-1, -3) + W(-1, -2) + W(0, -1) + W(0, 0) + W(0, 1) + W(1, 2) + W(1, 3) + W(1, 4))     \
    SQ(W(-4, -1) + W(-3, -1) + W(-2, -1) + W(-1, 0) + W(0, 0) + W(1, 0) + W(2, 1) + W(3, 1) + W(4, 1))     \
    SQ(W(-4, 1) + W(-3, 1) + W(-2, 1) + W(-1, 0) + W(0, 0) + W(1, 0) + W(2, -1) + W(3, -1) + W(4, -1))     \
    SQ(W(-2, -3) + W(-1, -2) + W(-1, -1) + W(0, 0) + W(1, 1) + W(1, 2) + W(2, 3))                          \
    SQ(W(2, -3) + W(1, -2) + W(1, -1) + W(0, 0) + W(-1, 1) + W(-1, 2) + W(-2, 3))                          \
    SQ(W(-3, -2) + W(-2, -1) + W(-1, -1) + W(0, 0) + W(1, 1) + W(2, 1) + W(3, 2))                          \
    SQ(W(3, -2) + W(2, -1) + W(1, -1) + W(0, 0) + W(-1, 1) + W(-2, 1) + W(-3, 2))                          \
    SQ(W(-4, 2) + W(-3, 2) + W(-2, 1) + W(-1, 1) + W(0, 0) + W(1, 0) + W(2, -1) + W(3, -1))                \
    SQ(W(-4, -2) + W(-3, -2) + W(-2, -1) + W(-1, -1) + W(0, 0) + W(1, 0) + W(2, 1) + W(3, 1))              \
    SQ(W(-2, -4) + W(-2, -3) + W(-1, -2) + W(-1, -1) + W(0, 0) + W(0, 1) + W(1, 2) + W(1, 3))              \
    SQ(W(2, -4) + W(2, -3) + W(1, -2) + W(1, -1) + W(0, 0) + W(0, 1) + W(-1, 2) + W(-1, 3))
#define MALTA_LF_BODY                                         \
    SQ(W(-4, 0) + W(-2, 0) + W(0, 0) + W(2, 0) + W(4, 0))     \
    SQ(W(0, -4) + W(0, -2) + W(0, 0) + W(0, 2) + W(0, 4))     \
    SQ(W(-3, -3) + W(-2, -2) + W(0, 0) + W(2, 2) + W(3, 3))   \
    SQ(W(3, -3) + W(2, -2) + W(0, 0) + W(-2, 2) + W(-3, 3))   \
    SQ(W(1, -4) + (W(1, -2) + W(0, 0) + W(-1, 2)) + W(-1, 4)) \
    SQ(W(-1, -4) + (W(-1, -2) + W(0, 0) + W(1, 2)) + W(1, 4)) \
    SQ(W(-4, -1) + (W(-2, -1) + W(0, 0) + W(2, 1)) + W(4, 1)) \
    SQ(W(-4, 1) + (W(-2, 1) + W(0, 0) + W(2, -1)) + W(4, -1)) \
    SQ(W(-2, -3) + (W(-1, -2) + W(0, 0) + W(1, 2)) + W(2, 3)) \
    SQ(W(2, -3) + (W(1, -2) + W(0, 0) + W(-1, 2)) + W(-2, 3)) \
    SQ(W(-3, -2) + (W(-2, -1) + W(0, 0) + W(2, 1)) + W(3, 2)) \
    SQ(W(3, -2) + W(2, -1) + W(0, 0) + W(-2, 1) + W(-3, 2))   \
    SQ(W(-4, 2) + (W(-2, 1) + W(0, 0) + W(2, -1)) + W(4, -2)) \
    SQ(W(-4, -2) + (W(-2, -1) + W(0, 0) + W(2, 1)) + W(4, 2)) \
    SQ(W(-2, -4) + (W(-1, -2) + W(0, 0) + W(1, 2)) + W(2, 4)) \
    SQ(W(2, -4) + (W(1, -2) + W(0, 0) + W(-1, 2)) + W(-2, 4))

constexpr int DF_TW = 32, DF_TH = 64, DF_H = 4;
constexpr int DF_IW = DF_TW + 2 * DF_H, DF_IH = DF_TH + 2 * DF_H;  // 40 x 72

// Sliding register window down one column. The patterns of both units reach columns
// -2..2 at rows -4 and +4 of the window, -3..3 at rows -3 and +3 and -4..4 in between, so each
// sample is loaded when the first output needs it and dies after the last: a row enters the
// window with its five central columns, gains the next two a row later and the outer two a row
// after that, and loses them in the reverse order, about 69 values live instead of 81.
__device__ __forceinline__ constexpr int malta_reach(int dy) {
    return (dy == 4 || dy == -4) ? 2 : (dy == 3 || dy == -3) ? 3 : 4;
}
template <bool HF>
__device__ __forceinline__ void malta_column(const float* __restrict__ Dt, int r0, int c, float* __restrict__ acc) {
    float win[16][9];
#pragma unroll
    for (int o = 0; o < 8; o++) {
#pragma unroll
        for (int r = o; r <= o + 8; r++) {
            const int dy = r - o - 4;
            const int reach = malta_reach(dy);
            // the reach this row had for the previous output (-1: not in that window)
            const int prev = (o == 0 || r == o + 8) ? -1 : malta_reach(dy + 1);
#pragma unroll
            for (int j = 0; j < 9; j++) {
                const int dx = j - 4 < 0 ? 4 - j : j - 4;
                if (dx <= reach && dx > prev) win[r][j] = Dt[(r0 + r) * DF_IW + c + j];
            }
        }
        float ret = 0.0f;
        if (HF) {
            MALTA_HF_BODY
        } else {
            MALTA_LF_BODY
        }
        acc[o * 256] += ret;
    }
}
#undef W
#undef SQ

// grid (ceil(w/32), ceil(h/64), npairs), 256 threads; column tid&31, rows 8*(tid>>5)..+7.
// pimg[pair] = (reference image, distorted image).
// The six maps' raw (l0, l1) tiles are staged with cp.async, double-buffered across maps;
// samples outside the image arrive as zeros, for which malta_pre returns exactly 0, the
// reference's padding value (maltaDiff.hpp:549-553).
// With half-band storage the UHF maps' raw tiles are FP16 rows of DFH_P halves staged from x0 - 8
// (16-byte chunks of 8 halves), in the same buffers, and the window's column c sits at half c + 4
// of its row.
constexpr int DF_RAW = DF_IH * DF_IW;
constexpr int kDiffSmem = (4 * DF_RAW + DF_RAW + 2 * 8 * 256) * 4;
constexpr int DFH_P = 56;  // 48 staged halves + 8 of padding (7 quads per row)
static_assert(DF_IH * DFH_P / 2 <= DF_RAW, "an FP16 raw tile fits an FP32 tile's buffer");

// L2AsymDiff's two terms for one pixel (simplerdiff.hpp:61-100), added to acc in the
// reference's order. The two sign branches are one, on s2 mirrored to s1's side (as in
// malta_pre): s2 + too_small == too_small - (-s2) and -s2 - too_big are the same IEEE operations;
// outside both ranges v = 0 adds exactly nothing.
__device__ __forceinline__ void l2asym_add(float& acc, float s1, float s2, float w_gt, float w_lt) {
    constexpr DConst k04 = dconst(0.4);
    const float diff = s1 - s2;
    acc += w_gt * diff * diff;
    const float fabs0 = fabsf(s1);
    const float too_small = mul_dc(fabs0, k04), too_big = fabs0;
    const float s2m = s1 < 0 ? -s2 : s2;
    const float v = s2m < too_small ? too_small - s2m : (s2m > too_big ? s2m - too_big : 0.0f);
    acc += w_lt * v * v;
}

template <bool HB>
__global__ void __launch_bounds__(256, 3) butter_diff_kernel(float* const* __restrict__ ib, const int2* __restrict__ pimg,
                                                             BGeom g, int s) {
    extern __shared__ __align__(16) float sm[];
    constexpr int RAWF = DF_RAW;  // floats per raw tile
    float* Dt = sm + 4 * RAWF;
    const int2 pi = pimg[blockIdx.z];
    const int i0 = pi.x, i1 = pi.y;
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * DF_TW, y0 = blockIdx.y * DF_TH;
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    // [channel Y, X][8 outputs][256 threads]: each thread's sums, kept in shared memory rather than
    // registers so that the Malta window has the register file to itself
    float* accs = Dt + DF_RAW + threadIdx.x;
#pragma unroll
    for (int o = 0; o < 16; o++) accs[o * 256] = 0.f;
    const DiffParams& P = c_dp;
    // maltaDiff order (main.hpp:57-79): UHF Y, UHF X, HF Y, HF X, MF Y, MF X, map m = 0..5. Each
    // channel's three maps (Y: m = 0, 2, 4; X: 1, 3, 5) are summed in that order into its own
    // accumulators. The two UHF maps (the 9-tap Malta unit, FP16 tiles with half-band storage) run
    // as one loop and the four HF and MF maps (the 5-tap unit, FP32 tiles) as another, so that
    // neither loop carries the other's staging and conversion paths.
    auto plane_id = [](int m) { return (m < 2 ? I_UHF : m < 4 ? I_HF : I_MF) + 1 - (m & 1); };
    auto stage = [&](float* dst, int img, int id, auto half) {
        if constexpr (decltype(half)::value)
            stage_tile_t<DF_IH, 6>(reinterpret_cast<__half*>(dst), DFH_P, (const __half*)hplane(ib, S, img, id), S.p,
                                   S.w, S.h, x0 - 8, y0 - DF_H);
        else
            stage_tile_t<DF_IH, DF_IW / 4>(dst, DF_IW, (const float*)iplane(ib, g, S, img, id), S.p, S.w, S.h,
                                           x0 - DF_H, y0 - DF_H);
    };
    // the staged sample at this thread's output (column vc, row 8*vg + o of an FP32 tile)
    auto center = [&](const float* tile, int o) { return tile[(8 * vg + o + DF_H) * DF_IW + vc + DF_H]; };
    // map m, whose raw tiles are staged in buffer pair m & 1; UHF: m < 2; next_half: the next
    // map's tiles are FP16 (UHF X after UHF Y with half-band storage)
    auto map_step = [&](int m, auto uhf, auto next_half) {
        constexpr bool UHF = decltype(uhf)::value;
        constexpr bool HALF = HB && UHF;
        const float* r0 = sm + (m & 1) * 2 * RAWF;
        const float* r1 = r0 + RAWF;
        if (m < 5) {
            float* n0 = sm + ((m + 1) & 1) * 2 * RAWF;
            const int id = plane_id(m + 1);
            stage(n0, i0, id, next_half);
            stage(n0 + RAWF, i1, id, next_half);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const MaltaMap mm = c_dp.mm[m];
        // four neighbouring samples per thread (rows of 40 floats hold 10 whole quads): one 16-byte
        // load per image (8 bytes of halves from an FP16 tile) and one 16-byte store
        constexpr int NQ = DF_IH * DF_IW / 4;
#pragma unroll
        for (int k = 0; k < (NQ + 255) / 256; k++) {
            const int q = threadIdx.x + 256 * k;
            if (q < NQ) {
                float4 a, b;
                if constexpr (HALF) {
                    const int r = q / (DF_IW / 4), c = 4 * (q - r * (DF_IW / 4));
                    const int hi = r * DFH_P + c + 4;  // a multiple of 4 halves: 8-byte aligned
                    const uint2 ua = *reinterpret_cast<const uint2*>(reinterpret_cast<const __half*>(r0) + hi);
                    const uint2 ub = *reinterpret_cast<const uint2*>(reinterpret_cast<const __half*>(r1) + hi);
                    const float2 a0 = __half22float2(*reinterpret_cast<const __half2*>(&ua.x));
                    const float2 a1 = __half22float2(*reinterpret_cast<const __half2*>(&ua.y));
                    const float2 b0 = __half22float2(*reinterpret_cast<const __half2*>(&ub.x));
                    const float2 b1 = __half22float2(*reinterpret_cast<const __half2*>(&ub.y));
                    a = make_float4(a0.x, a0.y, a1.x, a1.y);
                    b = make_float4(b0.x, b0.y, b1.x, b1.y);
                } else {
                    a = reinterpret_cast<const float4*>(r0)[q];
                    b = reinterpret_cast<const float4*>(r1)[q];
                }
                reinterpret_cast<float4*>(Dt)[q] = make_float4(malta_pre(a.x, b.x, mm), malta_pre(a.y, b.y, mm),
                                                               malta_pre(a.z, b.z, mm), malta_pre(a.w, b.w, mm));
            }
        }
        float* acc = accs + (m & 1) * 8 * 256;  // this map's channel
        if constexpr (!UHF) {
            // The HF and MF maps' own L2 terms (simplerdiff.hpp:41-100; channel X for odd m, Y for
            // even), from the bands already staged here, before the barrier after which the next
            // staging may overwrite this buffer: L2AsymDiff of HF, L2 of MF. The reference adds
            // them after all three maps of the channel; here they join the channel's sum between
            // maps, a different order of the same FP32 additions.
            const int c = (m & 1) ? 0 : 1;
#pragma unroll
            for (int o = 0; o < 8; o++) {
                const float s1 = center(r0, o), s2 = center(r1, o);
                float a = acc[o * 256];
                if (m < 4) {
                    l2asym_add(a, s1, s2, P.l2asym_gt[c], P.l2asym_lt[c]);
                } else {
                    const float dm = s1 - s2;
                    a += P.wmf[c] * dm * dm;
                }
                acc[o * 256] = a;
            }
        }
        __syncthreads();
        malta_column<UHF>(Dt, 8 * vg, vc, acc);
    };
    stage(sm, i0, plane_id(0), std::integral_constant<bool, HB>{});
    stage(sm + RAWF, i1, plane_id(0), std::integral_constant<bool, HB>{});
    cp_async_commit();
    if constexpr (HB) {
        // the UHF Y map stages FP16 tiles for UHF X, which stages FP32 tiles for HF Y
        map_step(0, std::true_type{}, std::integral_constant<bool, HB>{});
        map_step(1, std::true_type{}, std::false_type{});
    } else {
#pragma unroll 1
        for (int m = 0; m < 2; m++) map_step(m, std::true_type{}, std::false_type{});
    }
#pragma unroll 1
    for (int m = 2; m < 6; m++) map_step(m, std::false_type{}, std::false_type{});
    const int x = x0 + vc;
    if (x >= S.w) return;
    // What the staged tiles do not hold: MF of the B channel (no Malta map; L2 only) and the LF
    // values of all three channels (the DC terms).
#pragma unroll
    for (int o = 0; o < 8; o++) {
        const int y = y0 + 8 * vg + o;
        if (y < S.h) {
            const int64_t i = (int64_t)y * S.p + x;
            const float dmb = __ldg(iplane(ib, g, S, i0, I_MF + 2) + i) - __ldg(iplane(ib, g, S, i1, I_MF + 2) + i);
            const float acc_b = P.wmf[2] * dmb * dmb;
            float dc[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float dl = __ldg(iplane(ib, g, S, i0, I_LFV + c) + i) - __ldg(iplane(ib, g, S, i1, I_LFV + c) + i);
                dc[c] = P.wlf[c] * dl * dl;
            }
            iplane(ib, g, S, i1, Q_SAC)[i] = accs[(8 + o) * 256] + accs[o * 256] + acc_b;
            iplane(ib, g, S, i1, Q_SDC)[i] = dc[0] + dc[1] + dc[2];
        }
    }
}

// Blur both mask planes (sigma 2.7); store B0 and add 10*(B0-B1)^2 to the AC sum.
// grid (ceil(w/32), ceil(h/48), npairs)
__global__ void __launch_bounds__(256, 6) butter_mask_blur_kernel(float* const* __restrict__ ib,
                                                                  const int2* __restrict__ pimg, BGeom g, int s) {
    extern __shared__ __align__(16) float sm[];
    float* hb = sm + 2 * TB_RAW;
    const int2 pi = pimg[blockIdx.z];
    const int i1 = pi.y;
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * TB_TW, y0 = blockIdx.y * TB_TH;
    float rxy[6];
    tile_masses_r8<2>(x0, y0, S.w, S.h, rxy);
    // the two masks in two cp.async groups, so the second lands under the first one's blur
    tile_stage_r8(sm, iplane(ib, g, S, pi.x, I_PRE), S.p, S.w, S.h, x0, y0);
    cp_async_commit();
    tile_stage_r8(sm + TB_RAW, iplane(ib, g, S, i1, I_PRE), S.p, S.w, S.h, x0, y0);
    cp_async_commit();
    float b[2][6];
    cp_async_wait<1>();
    __syncthreads();
    tile_blur_r8<2>(sm, hb, rxy, b[0]);
    cp_async_wait<0>();
    __syncthreads();  // the second mask is staged and every thread is done with hb
    tile_blur_r8<2>(sm + TB_RAW, hb, rxy, b[1]);
    const int vc = threadIdx.x & 31, vg = threadIdx.x >> 5;
    float* b0 = iplane(ib, g, S, i1, Q_B0);
    float* sac = iplane(ib, g, S, i1, Q_SAC);
#pragma unroll
    for (int o = 0; o < 6; o++) {
        const int x = x0 + vc, y = y0 + 6 * vg + o;
        if (x < S.w && y < S.h) {
            const int64_t i = (int64_t)y * S.p + x;
            b0[i] = b[0][o];
            const float d = b[0][o] - b[1][o];
            sac[i] += 10.0f * d * d;
        }
    }
}


// combineMasks.hpp:3-19
__device__ __forceinline__ float mask_common(float c) {
    // the reference's (float)((1.0 + c) * K) in double, here in FP32: within 2 ulp of it
    constexpr float kK = (float)(1.0 / (double)(0.79079917404f * 17.83f));
    const float r = (1.0f + c) * kK;
    return r * r;
}
__device__ __forceinline__ float mask_y(float delta) {
    return mask_common(div_nr(2.5485944793f, (0.451936922203f * delta) + 0.829591754942f));
}
__device__ __forceinline__ float mask_dc_y(float delta) {
    return mask_common(div_nr(0.505054525019f, (3.87449418804f * delta) + 0.20025578522f));
}
// maskPsycho.hpp:42-55: keep the three smallest values, m0 <= m1 <= m2. As min/max insertion
// into the sorted triple: the same values as the reference's branches, ties included, and +inf
// leaves the triple unchanged.
__device__ __forceinline__ void store_min3(float v, float& m0, float& m1, float& m2) {
    const float n2 = fminf(m2, fmaxf(m1, v));
    const float n1 = fminf(m1, fmaxf(m0, v));
    m0 = fminf(m0, v);
    m1 = n1;
    m2 = n2;
}

// Fuzzy erosion + diffmap; FINAL also folds in the half-scale map, stores the distortion map
// (when distmap is not null) and emits norm partials. grid (ceil(w/32), ceil(h/32), npairs),
// 256 threads: thread (tx, ty) = (tid % 32, tid / 32) makes column x0 + tx, rows y0 + ty + 8k
// (k < 4). The blurred mask
// tile and its 3-px halo are staged in shared memory; neighbours outside the image are +inf,
// which store_min3 ignores, as the reference skips them (maskPsycho.hpp:57-110).
constexpr int DM_TW = 32, DM_TH = 32, DM_HX = 4, DM_HY = 3;
constexpr int DM_IW = DM_TW + 2 * DM_HX, DM_IH = DM_TH + 2 * DM_HY;  // 40 x 38

template <bool FINAL>
__global__ void __launch_bounds__(256) butter_diffmap_kernel(float* const* __restrict__ ib, const int2* __restrict__ pimg,
                                                             BGeom g, int s, float* __restrict__ distmap,
                                                             float* __restrict__ partials, float qnorm) {
    __shared__ __align__(16) float bt[DM_IH * DM_IW];
    const int pair = blockIdx.z;
    const int i1 = pimg[pair].y;
    const BScaleDev S = pick_scale(g, s);
    const int x0 = blockIdx.x * DM_TW, y0 = blockIdx.y * DM_TH;
    // 1-D block of 256 (stage_tile_t distributes chunks over threadIdx.x)
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const float* b0 = iplane(ib, g, S, i1, Q_B0);
    stage_tile_t<DM_IH, DM_IW / 4>(bt, DM_IW, b0, S.p, S.w, S.h, x0 - DM_HX, y0 - DM_HY);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    if (x0 < DM_HX || y0 < DM_HY || x0 + DM_TW + DM_HX > S.w || y0 + DM_TH + DM_HY > S.h) {
        for (int e = tid; e < DM_IH * DM_IW; e += 256) {
            const int r = e / DM_IW, c = e - r * DM_IW;
            const int gx = x0 - DM_HX + c, gy = y0 - DM_HY + r;
            if (gx < 0 || gx >= S.w || gy < 0 || gy >= S.h) bt[e] = __int_as_float(0x7f800000);
        }
        __syncthreads();
    }
    const float* sac = iplane(ib, g, S, i1, Q_SAC);
    const float* sdc = iplane(ib, g, S, i1, Q_SDC);
    float sq = 0.f, s3 = 0.f, mx = 0.f;
    const int x = x0 + tx;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int ly = ty + 8 * k, y = y0 + ly;
        if (x < S.w && y < S.h) {
            const float* c = bt + (ly + DM_HY) * DM_IW + tx + DM_HX;
            constexpr int K = 3, R = 3 * DM_IW;
            float m0 = c[0], m1 = 2.0f * m0, m2 = m1;
            store_min3(c[-K], m0, m1, m2);
            store_min3(c[-K - R], m0, m1, m2);
            store_min3(c[-K + R], m0, m1, m2);
            store_min3(c[K], m0, m1, m2);
            store_min3(c[K - R], m0, m1, m2);
            store_min3(c[K + R], m0, m1, m2);
            store_min3(c[-R], m0, m1, m2);
            store_min3(c[R], m0, m1, m2);
            const float mask = 0.45f * m0 + 0.3f * m1 + 0.25f * m2;
            const int64_t i = (int64_t)y * S.p + x;
            float d = sqrt_nr(mask_y(mask) * __ldg(sac + i) + mask_dc_y(mask) * __ldg(sdc + i));
            if (!FINAL) {
                iplane(ib, g, S, i1, Q_DIFF)[i] = d;
            } else {
                constexpr DConst k085 = dconst(1.0 - 0.3 * (double)0.5f);
                const BScaleDev Hs = g.s[1];
                const float small = iplane(ib, g, Hs, i1, Q_DIFF)[(int64_t)(y / 2) * Hs.p + x / 2];
                d = fmaf(0.5f, small, mul_dc(d, k085));
                if (distmap) distmap[(int64_t)pair * S.w * S.h + (int64_t)y * S.w + x] = d;
                sq += qnorm == 2.0f ? d * d : powf(d, qnorm);  // diffnorms.hpp:63
                s3 += fabsf(d) * d * d;
                mx = fmaxf(mx, fabsf(d));
            }
        }
    }
    if (FINAL) {
        __shared__ float red[3][8];
        const int lane = tx, warp = ty;
        sq = warp_sum(sq);
        s3 = warp_sum(s3);
        mx = warp_max(mx);
        if (lane == 0) {
            red[0][warp] = sq;
            red[1][warp] = s3;
            red[2][warp] = mx;
        }
        __syncthreads();
        if (warp == 0 && lane < 3) {
            float v = red[lane][0];
            for (int w = 1; w < 8; w++) v = lane == 2 ? fmaxf(v, red[lane][w]) : v + red[lane][w];
            const int blk = blockIdx.y * gridDim.x + blockIdx.x;
            partials[((int64_t)pair * 3 + lane) * g.norm_tiles + blk] = v;
        }
    }
}

// Norm combine, one CTA per pair (diffnorms.hpp:263-306): the per-tile sums reduced as
// float-float sums on the FP32 pipe (eight loads in flight per thread), then the two roots in
// FP64 by two warps at once. On this GPU a dependent FP64 operation takes about 60 cycles and
// pow() several thousand, so the common norms take the cheaper library roots: the 3-norm cbrt,
// a Q-norm of 2 sqrt (1 none), other Q pow.
__device__ __forceinline__ double root_q(double x, int q) {
    return q == 1 ? x : q == 2 ? sqrt(x) : q == 3 ? cbrt(x) : pow(x, 1.0 / (double)q);
}

__global__ void __launch_bounds__(256) butter_finalize_kernel(const float* __restrict__ partials,
                                                              double* __restrict__ norms, BGeom g, int qnorm) {
    __shared__ FSum red[2][8];
    __shared__ float redmx[8];
    const int pair = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    FSum sq{0.f, 0.f}, s3{0.f, 0.f};
    float mx = 0.f;
    const float* p = partials + (int64_t)pair * 3 * g.norm_tiles;
    for (int t0 = tid; t0 < g.norm_tiles; t0 += 256 * 8) {
        float a[8], b[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int t = t0 + 256 * k;
            a[k] = t < g.norm_tiles ? __ldg(p + t) : 0.f;
            b[k] = t < g.norm_tiles ? __ldg(p + g.norm_tiles + t) : 0.f;
            if (t < g.norm_tiles) mx = fmaxf(mx, __ldg(p + 2 * g.norm_tiles + t));
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sq.add(a[k]);
            s3.add(b[k]);
        }
    }
    sq = warp_sum(sq);
    s3 = warp_sum(s3);
    mx = warp_max(mx);
    if (lane == 0) {
        red[0][warp] = sq;
        red[1][warp] = s3;
        redmx[warp] = mx;
    }
    __syncthreads();
    if (lane == 0 && warp < 2) {
        FSum a = red[warp][0];
        for (int w = 1; w < 8; w++) a.add(red[warp][w]);
        const double n = (double)g.s[0].w * (double)g.s[0].h;
        norms[pair * 3 + warp] = root_q(a.value() / n, warp == 0 ? qnorm : 3);
        if (warp == 1) {
            float c = redmx[0];
            for (int w = 1; w < 8; w++) c = fmaxf(c, redmx[w]);
            norms[pair * 3 + 2] = (double)c;
        }
    }
}

// ------------------------------------------------------------------------------------------
// Host side

static BGeom make_bgeom(int64_t w, int64_t h, bool half_bands) {
    BGeom g{};
    g.half_bands = half_bands ? 1 : 0;
    int64_t off = 0;
    int64_t cw = w, ch = h;
    for (int s = 0; s < 2; s++) {
        BScaleDev& S = g.s[s];
        S.w = (int)cw;
        S.h = (int)ch;
        S.p = (int)round_up(cw, 8);
        S.n = round_up((int64_t)S.p * ch, 64);
        S.base = off;
        // S.n is a multiple of 64, so the FP16 block (NIMG - I_UHF half planes) keeps the next
        // scale's base 256-byte aligned
        off += half_bands ? S.n * I_UHF + S.n * (NIMG - I_UHF) / 2 : S.n * NIMG;
        cw = half_dim(cw);
        ch = half_dim(ch);
    }
    g.img_floats = off;
    g.norm_tiles_x = (int)ceil_div(w, DM_TW);
    g.norm_tiles = g.norm_tiles_x * (int)ceil_div(h, DM_TH);
    return g;
}

static DiffParams make_diff_params() {
    DiffParams P{};
    const float hf_asym = 0.8f;
    const float sq = std::sqrt(hf_asym);
    struct In {
        float w_gt, w_lt, norm1;
        bool hf;
    };
    const In in[6] = {
        {1.10039032555f * hf_asym, 1.10039032555f / hf_asym, 71.7800275169f, true},
        {173.5f * hf_asym, 173.5f / hf_asym, 5.0f, true},
        {18.7237414387f * sq, 18.7237414387f / sq, 4498534.45232f, false},
        {6923.99476109f * sq, 6923.99476109f / sq, 8051.15833247f, false},
        {37.0819870399f, 37.0819870399f, 130262059.556f, false},
        {8246.75321353f, 8246.75321353f, 1009002.70582f, false},
    };
    for (int m = 0; m < 6; m++) {
        const float mulli = in[m].hf ? 0.39905817637f : 0.611612573796f;
        const float len2 = 3.75f * 2.0f + 1.0f;
        const float wpg = mulli * std::sqrt(0.5f * in[m].w_gt) / len2;
        const float wpl = mulli * std::sqrt(0.33f * in[m].w_lt) / len2;
        P.mm[m].norm1 = in[m].norm1;
        P.mm[m].n2gt = wpg * in[m].norm1;
        P.mm[m].n2lt = wpl * in[m].norm1;
    }
    const float wmul[9] = {400.0f, 1.50815703118f, 0.0f, 2150.0f, 10.6195433239f, 16.2176043152f,
                           29.2353797994f, 0.844626970982f, 0.703646627719f};
    for (int c = 0; c < 2; c++) {
        float gt = wmul[c] * hf_asym, lt = wmul[c] / hf_asym;
        P.l2asym_gt[c] = (float)((double)gt * 0.8);
        P.l2asym_lt[c] = (float)((double)lt * 0.8);
    }
    for (int c = 0; c < 3; c++) {
        P.wmf[c] = wmul[3 + c];
        P.wlf[c] = wmul[6 + c];
    }
    return P;
}

constexpr int kTileSmem = (2 * TB_RAW + TB_HPL) * 4;
constexpr int kTileSmem2 = (2 * TB_RAW + 2 * TB_HPL) * 4;  // with a pair buffer (tile_blur_r8_x2)

__global__ void butter_identity_pairs_kernel(int2* pimg, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pimg[i] = make_int2(2 * i, 2 * i + 1);
}

int butter_prepare_device() {
    int rc = upload_butter_tables();
    if (rc) return rc;
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(butter_lf_v_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kVLfSmem));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(butter_mf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMfSmem));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(butter_diff_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kDiffSmem));
    VSHIP_CUDA_TRY(cudaFuncSetAttribute(butter_diff_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kDiffSmem));
    const DiffParams P = make_diff_params();
    VSHIP_CUDA_TRY(cudaMemcpyToSymbol(c_dp, &P, sizeof(P)));
    return E_OK;
}

size_t butter_image_floats(int64_t w, int64_t h, bool half_bands) {
    return (size_t)make_bgeom(w, h, half_bands).img_floats;
}
int butter_norm_tiles(int64_t w, int64_t h) { return make_bgeom(w, h, false).norm_tiles; }

int ButterEngine::init(int64_t width, int64_t height, int qnorm_, float intensity_, int max_pairs_) {
    int rc = init_images(width, height, qnorm_, intensity_, 2 * max_pairs_, max_pairs_, true);
    if (rc) return rc;
    VSHIP_CUDA_TRY(vship_malloc((void**)&pimg_identity, sizeof(int2) * max_pairs));
    butter_identity_pairs_kernel<<<(unsigned)ceil_div(max_pairs, 256), 256>>>(pimg_identity, max_pairs);
    VSHIP_CUDA_TRY(cudaGetLastError());
    VSHIP_CUDA_TRY(cudaDeviceSynchronize());
    return E_OK;
}

int ButterEngine::init_images(int64_t width, int64_t height, int qnorm_, float intensity_, int max_images_,
                              int max_pairs_, bool keep_distmap) {
    w = width;
    h = height;
    qnorm = qnorm_;
    intensity = intensity_;
    max_images = max_images_;
    max_pairs = max_pairs_;
    if (max_images <= 0 || max_pairs <= 0) return E_BAD_POINTER;
    BGeom g = make_bgeom(w, h, half_bands);
    for (int s = 0; s < 2; s++) {
        sc[s].w = g.s[s].w;
        sc[s].h = g.s[s].h;
        sc[s].n = g.s[s].n;
    }
    img_floats = g.img_floats;
    norm_blocks = g.norm_tiles;
    int rc = butter_prepare_device();
    if (rc) return rc;
    VSHIP_CUDA_TRY(vship_malloc((void**)&work, sizeof(float) * img_floats * max_images));
    VSHIP_CUDA_TRY(vship_malloc((void**)&partials, sizeof(float) * 3 * (size_t)norm_blocks * max_pairs));
    if (keep_distmap) VSHIP_CUDA_TRY(vship_malloc((void**)&distmap, sizeof(float) * (size_t)w * h * max_pairs));
    VSHIP_CUDA_TRY(vship_malloc((void**)&norms, sizeof(double) * 3 * max_pairs));
    std::vector<float*> bases(max_images);
    for (int i = 0; i < max_images; i++) bases[i] = work + (size_t)i * img_floats;
    VSHIP_CUDA_TRY(vship_malloc((void**)&ibase, sizeof(float*) * max_images));
    VSHIP_CUDA_TRY(cudaMemcpy(ibase, bases.data(), sizeof(float*) * max_images, cudaMemcpyHostToDevice));
    VSHIP_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    return E_OK;
}

void ButterEngine::destroy() {
    if (work) cudaFree(work);
    if (partials) cudaFree(partials);
    if (distmap) cudaFree(distmap);
    if (norms) cudaFree(norms);
    if (pimg_identity) cudaFree(pimg_identity);
    if (ibase) cudaFree(ibase);
    work = nullptr;
    partials = nullptr;
    distmap = nullptr;
    norms = nullptr;
    pimg_identity = nullptr;
    ibase = nullptr;
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    side = nullptr;
    ev_fork = ev_join = nullptr;
}

size_t ButterEngine::image_bytes(int64_t w, int64_t h, bool half_bands) {
    return sizeof(float) * (size_t)make_bgeom(w, h, half_bands).img_floats;
}

size_t ButterEngine::device_bytes(int64_t w, int64_t h, int pairs, bool half_bands) {
    BGeom g = make_bgeom(w, h, half_bands);
    return (sizeof(float) * 2 * (size_t)g.img_floats + sizeof(float) * 3 * (size_t)g.norm_tiles +
            sizeof(float) * (size_t)w * h + sizeof(double) * 3 + sizeof(int2) + 2 * sizeof(float*)) *
           pairs;
}

int ButterEngine::launch(const FrameDesc* frames_dev, int intype, int npairs, double* norms_out, cudaStream_t st,
                         const YuvParams* yuv) {
    if (npairs <= 0 || npairs > max_pairs || !pimg_identity) return E_BAD_POINTER;
    return launch_images(frames_dev, 2 * npairs, pimg_identity, npairs, intype, norms_out, distmap, st, yuv);
}

int ButterEngine::launch_images(const FrameDesc* frames_dev, int nimages, const int2* pimg, int npairs, int intype,
                                double* norms_out, float* distmap_out, cudaStream_t st, const YuvParams* yuv) {
    if (nimages <= 0 || nimages > max_images || npairs <= 0 || npairs > max_pairs) return E_BAD_POINTER;
    return butter_enqueue(w, h, qnorm, intensity, ibase, frames_dev, nimages, pimg, npairs, intype, partials,
                          norms_out ? norms_out : norms, distmap_out, st, yuv, half_bands, side, ev_fork, ev_join);
}

int butter_enqueue(int64_t w, int64_t h, int qnorm, float intensity, float* const* ib, const FrameDesc* frames_dev,
                   int nstage, const int2* pimg, int npairs, int intype, float* partials, double* norms_out,
                   float* distmap_out, cudaStream_t st, const YuvParams* yuv, bool half_bands, cudaStream_t side,
                   cudaEvent_t ev_fork, cudaEvent_t ev_join) {
    if (npairs <= 0 || nstage < 0) return E_BAD_POINTER;
    const YuvParams yp = yuv ? *yuv : yuv420p10_params();
    const BGeom g = make_bgeom(w, h, half_bands);
    const unsigned ni = (unsigned)nstage, np = (unsigned)npairs;
    if (ni) {
        dim3 gr((unsigned)ceil_div(w, 32), (unsigned)ceil_div(h, 32), ni);
        ProfScope ps_("butter_decode", st);
        switch (intype) {
            case IN_UINT8: butter_decode_kernel<IN_UINT8><<<gr, 256, 0, st>>>(frames_dev, ib, g, yp); break;
            case IN_UINT16: butter_decode_kernel<IN_UINT16><<<gr, 256, 0, st>>>(frames_dev, ib, g, yp); break;
            case IN_HALF: butter_decode_kernel<IN_HALF><<<gr, 256, 0, st>>>(frames_dev, ib, g, yp); break;
            case IN_YUV: butter_decode_kernel<IN_YUV><<<gr, 256, 0, st>>>(frames_dev, ib, g, yp); break;
            default: butter_decode_kernel<IN_FLOAT><<<gr, 256, 0, st>>>(frames_dev, ib, g, yp); break;
        }
    }
    // With a side stream the half scale's chain runs beside the full scale's: they share nothing
    // until the full-scale diffmap adds the half-scale map (1 % more pairs/s at 3840x2160, in the
    // batched form and end to end). Per-kernel profiling keeps everything on st.
    const bool fork = side && ev_fork && ev_join && !prof_enabled();
    if (fork) {
        VSHIP_CUDA_TRY(cudaEventRecord(ev_fork, st));
        VSHIP_CUDA_TRY(cudaStreamWaitEvent(side, ev_fork, 0));
    }
    const cudaStream_t st_full = st;
    for (int s = 1; s >= 0; s--) {
        const int64_t sw = g.s[s].w, sh = g.s[s].h;
        const cudaStream_t st = s == 1 && fork ? side : st_full;
        if (ni) {
            const dim3 gt((unsigned)ceil_div(sw, TB_TW), (unsigned)ceil_div(sh, TB_TH), ni);
            const dim3 gh((unsigned)ceil_div(sw, HB_TW), (unsigned)ceil_div(sh, HB_TH * HB_NT), 3 * ni);
            const dim3 gv((unsigned)ceil_div(sw, VB_TW), (unsigned)ceil_div(sh, VB_TH), ni);
            { ProfScope ps_("butter_opsin", st); butter_opsin_kernel<<<gt, 256, kTileSmem, st>>>(ib, g, s, intensity); }
            { ProfScope ps_("butter_hblur_lf", st); butter_hblur_kernel<4, 21><<<gh, 256, 0, st>>>(ib, g, s, I_XYB, I_TMP); }
            { ProfScope ps_("butter_lf_v", st); butter_lf_v_kernel<<<gv, 256, kVLfSmem, st>>>(ib, g, s); }
            {
                ProfScope ps_("butter_mf", st);
                const dim3 gmf((unsigned)ceil_div(sw, MS_TW), (unsigned)ceil_div(sh, MS_SEG), ni);
                butter_mf_kernel<<<gmf, 256, kMfSmem, st>>>(ib, g, s);
            }
            {
                ProfScope ps_("butter_hf", st);
                if (half_bands) butter_hf_kernel<true><<<gt, 256, kTileSmem2, st>>>(ib, g, s);
                else butter_hf_kernel<false><<<gt, 256, kTileSmem2, st>>>(ib, g, s);
            }
        }
        const dim3 gd((unsigned)ceil_div(sw, DF_TW), (unsigned)ceil_div(sh, DF_TH), np);
        {
            ProfScope ps_("butter_diff", st);
            if (half_bands) butter_diff_kernel<true><<<gd, 256, kDiffSmem, st>>>(ib, pimg, g, s);
            else butter_diff_kernel<false><<<gd, 256, kDiffSmem, st>>>(ib, pimg, g, s);
        }
        const dim3 gm((unsigned)ceil_div(sw, TB_TW), (unsigned)ceil_div(sh, TB_TH), np);
        { ProfScope ps_("butter_mask_blur", st); butter_mask_blur_kernel<<<gm, 256, kTileSmem, st>>>(ib, pimg, g, s); }
        const dim3 gf((unsigned)ceil_div(sw, DM_TW), (unsigned)ceil_div(sh, DM_TH), np);
        if (s == 1) {
            { ProfScope ps_("butter_diffmap", st); butter_diffmap_kernel<false><<<gf, 256, 0, st>>>(ib, pimg, g, s, nullptr, partials, (float)qnorm); }
            if (fork) VSHIP_CUDA_TRY(cudaEventRecord(ev_join, side));
        } else {
            if (fork) VSHIP_CUDA_TRY(cudaStreamWaitEvent(st, ev_join, 0));
            { ProfScope ps_("butter_diffmap", st); butter_diffmap_kernel<true><<<gf, 256, 0, st>>>(ib, pimg, g, s, distmap_out, partials, (float)qnorm); }
        }
    }
    { ProfScope ps_("butter_finalize", st); butter_finalize_kernel<<<np, 256, 0, st>>>(partials, norms_out, g, qnorm); }
    VSHIP_CUDA_TRY(cudaGetLastError());
    return E_OK;
}

}  // namespace vship
