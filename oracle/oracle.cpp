// oracle.cpp -- CPU restatement of Vship's per-frame-pair scoring math (SSIMULACRA2 and
// Butteraugli).
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py load it; the product library (vship_gb300/libvship.so) never
// links, loads or calls it.
//
// It is written from the reference's kernels, one function per reference step, each citing the
// file:line it follows (paths relative to the Vship source tree). It is instantiated twice:
//   * T = float  : follows the reference's FP32 evaluation order, including the places where a
//                  double literal promotes a float expression to double (e.g. `+ 0.55`).
//   * T = double : the FP64 error reference ("the same pipeline in FP64").
// Reductions accumulate in double in both instantiations (the math, not the reference's
// per-block tree order).
//
// Pins: the reference's only known-answer test (test/basic_metric_math_test.cpp:40-79) --
// identical frames give SSIMU2 == 100 exactly, Butteraugli norms (0,0,0) and an all-zero
// distortion map, with 0xFF bytes in the stride padding ignored -- is checked against this
// oracle in tests/test_oracle_pins.py, together with a check of every constant table below
// against the reference source text when the reference tree is present.
//
// Build: g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off (contraction off so x86 and Arm
// hosts round identically).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

enum InType { IN_UINT8 = 0, IN_UINT16 = 1, IN_HALF = 2, IN_FLOAT = 3 };  // util/preprocessor.hpp:94

constexpr double kTau = 6.28318530718;  // util/preprocessor.hpp:92

// ---------------------------------------------------------------------------------------------
// small helpers

// `a + c` where c is a double literal: the reference promotes to double and rounds back to T.
template <typename T> inline T addD(T a, double c) { return (T)((double)a + c); }
template <typename T> inline T mulD(T a, double c) { return (T)((double)a * c); }

template <typename F>
void parallel_rows(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 32) {
        f((int64_t)0, n);
        return;
    }
    int nt = (int)std::min<int64_t>(nthreads, n);
    std::vector<std::thread> th;
    th.reserve(nt);
    for (int t = 0; t < nt; t++) {
        int64_t b = n * t / nt, e = n * (t + 1) / nt;
        th.emplace_back([=]() { f(b, e); });
    }
    for (auto& x : th) x.join();
}

float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h >> 15) << 31;
    uint32_t exp = (h >> 10) & 0x1f;
    uint32_t man = h & 0x3ff;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal
            int e = -1;
            do { e++; man <<= 1; } while (!(man & 0x400));
            man &= 0x3ff;
            bits = sign | (uint32_t)(127 - 15 - e) << 23 | man << 13;
        }
    } else if (exp == 31) {
        bits = sign | 0x7f800000u | man << 13;
    } else {
        bits = sign | (exp + 112) << 23 | man << 13;
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// util/float3operations.hpp:197-218 (convertPointer<InputMemType>)
template <typename T>
inline T decode(const uint8_t* plane, int64_t stride, int64_t x, int64_t y, int intype) {
    const uint8_t* row = plane + y * stride;
    switch (intype) {
        case IN_UINT8: return (T)row[x] / (T)255;
        case IN_UINT16: { uint16_t v; std::memcpy(&v, row + 2 * x, 2); return (T)v / (T)65535; }
        case IN_HALF: { uint16_t v; std::memcpy(&v, row + 2 * x, 2); return (T)half_to_float(v); }
        default: { float v; std::memcpy(&v, row + 4 * x, 4); return (T)v; }
    }
}

// Round to the nearest IEEE half-precision value (ties to even), returned as T. Used to model
// FP16 storage of intermediate planes.
template <typename T> T round_half(T v) {
    float f = (float)v;
    uint32_t b;
    std::memcpy(&b, &f, 4);
    const uint32_t sign = b & 0x80000000u;
    const float a = std::fabs(f);
    if (!(a < 65520.f)) return (T)(sign ? -INFINITY : INFINITY);
    if (a < 6.103515625e-05f) {  // subnormal half: quantum 2^-24
        const float q = std::nearbyint(a * 16777216.f) / 16777216.f;
        return (T)(sign ? -q : q);
    }
    int e;
    std::frexp(a, &e);  // a = m * 2^e, m in [0.5, 1)
    const double quantum = std::ldexp(1.0, e - 11);
    const double q = std::nearbyint((double)a / quantum) * quantum;
    return (T)(sign ? -q : q);
}

// ssimu2/makeXYB.hpp:52-58 and butter/colors.hpp:7-13: sign-preserving x^2.4
template <typename T> inline T to_linear(T a) {
    return a < 0 ? -std::pow(-a, (T)2.4) : std::pow(a, (T)2.4);
}

struct Dims { int64_t w, h; };
inline int64_t half_dim(int64_t v) { return (v - 1) / 2 + 1; }

// ssimu2/downsample.hpp:3-19, butter/downupsample.hpp:3-20: 2x2 box with edge clamp
template <typename T>
void downsample(const T* src, T* dst, int64_t w, int64_t h) {
    int64_t nw = half_dim(w), nh = half_dim(h);
    for (int64_t y = 0; y < nh; y++) {
        int64_t y0 = std::min(2 * y, h - 1), y1 = std::min(2 * y + 1, h - 1);
        for (int64_t x = 0; x < nw; x++) {
            int64_t x0 = std::min(2 * x, w - 1), x1 = std::min(2 * x + 1, w - 1);
            T s = src[y0 * w + x0];
            s += src[y1 * w + x0];
            s += src[y0 * w + x1];
            s += src[y1 * w + x1];
            dst[y * nw + x] = s * (T)0.25;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Gaussian tables. A table holds 2R+1 taps followed by the 2R+2-entry prefix integral
// (I[0] = 0, I[i+1] = I[i] + k[i]) used for border renormalisation.

template <typename T> struct Kernel {
    int R;
    std::vector<T> k;  // 2R+1
    std::vector<T> I;  // 2R+2
};

// ssimu2/gaussianblur.hpp:7-18 (sigma 1.5, radius 8; util/preprocessor.hpp:89-90)
template <typename T> Kernel<T> ssimu2_kernel();
template <> Kernel<float> ssimu2_kernel<float>() {
    Kernel<float> g;
    g.R = 8;
    g.k.resize(17);
    g.I.assign(18, 0.f);
    const float sigma = 1.5f;
    for (int i = 0; i < 17; i++) {
        float e = std::exp((float)(-(8 - i) * (8 - i)) / (2 * sigma * sigma));
        g.k[i] = (float)((double)e / std::sqrt(kTau * sigma * sigma));
        g.I[i + 1] = g.I[i] + g.k[i];
    }
    return g;
}
template <> Kernel<double> ssimu2_kernel<double>() {
    Kernel<double> g;
    g.R = 8;
    g.k.resize(17);
    g.I.assign(18, 0.0);
    for (int i = 0; i < 17; i++) {
        g.k[i] = std::exp(-(double)((8 - i) * (8 - i)) / (2 * 1.5 * 1.5)) / std::sqrt(kTau * 1.5 * 1.5);
        g.I[i + 1] = g.I[i] + g.k[i];
    }
    return g;
}

// butter/gaussianblur.hpp:3-14,21-42: sigma list and window max(int(3 sigma), 8)
const double kButterSigmas[5] = {1.2, 1.56416327805, 2.7, 3.22489901262, 7.15593339443};

template <typename T> Kernel<T> butter_kernel(int idx);
template <> Kernel<float> butter_kernel<float>(int idx) {
    const double sigma = kButterSigmas[idx];
    Kernel<float> g;
    g.R = std::max((int)(sigma * 3), 8);
    int n = 2 * g.R + 1;
    g.k.resize(n);
    g.I.resize(n + 1);
    float acc = 0.f;
    for (int i = 0; i <= n; i++) {
        double q = (double)std::exp((float)(-(g.R - i) * (g.R - i) / (2 * sigma * sigma))) /
                   std::sqrt(kTau * sigma * sigma);
        if (i < n) g.k[i] = (float)q;
        g.I[i] = acc;
        acc = (float)((double)acc + q);
    }
    return g;
}
template <> Kernel<double> butter_kernel<double>(int idx) {
    const double sigma = kButterSigmas[idx];
    Kernel<double> g;
    g.R = std::max((int)(sigma * 3), 8);
    int n = 2 * g.R + 1;
    g.k.resize(n);
    g.I.assign(n + 1, 0.0);
    for (int i = 0; i < n; i++) {
        g.k[i] = std::exp(-(double)((g.R - i) * (g.R - i)) / (2 * sigma * sigma)) / std::sqrt(kTau * sigma * sigma);
        g.I[i + 1] = g.I[i] + g.k[i];
    }
    return g;
}

// Separable FIR with zero outside the image, each pass divided by the in-bounds kernel mass.
// ssimu2/gaussianblur.hpp:63-92 (tile form), butter/gaussianblur.hpp:58-92 and :94-186.
template <typename T>
void blur(const T* src, T* dst, T* tmp, int64_t w, int64_t h, const Kernel<T>& g, int nthreads) {
    const int R = g.R;
    parallel_rows(h, nthreads, [&](int64_t y0, int64_t y1) {
        for (int64_t y = y0; y < y1; y++) {
            const T* row = src + y * w;
            for (int64_t x = 0; x < w; x++) {
                int64_t beg = std::max<int64_t>(0, x - R) - (x - R);
                int64_t end = std::min<int64_t>(w, x + R + 1) - (x - R);
                T tot = g.I[end] - g.I[beg];
                T out = 0;
                for (int64_t i = beg; i < end; i++) out += row[x - R + i] * g.k[i];
                tmp[y * w + x] = out / tot;
            }
        }
    });
    parallel_rows(h, nthreads, [&](int64_t y0, int64_t y1) {
        std::vector<T> acc(w);
        for (int64_t y = y0; y < y1; y++) {
            int64_t beg = std::max<int64_t>(0, y - R) - (y - R);
            int64_t end = std::min<int64_t>(h, y + R + 1) - (y - R);
            T tot = g.I[end] - g.I[beg];
            std::fill(acc.begin(), acc.end(), (T)0);
            for (int64_t i = beg; i < end; i++) {
                const T* row = tmp + (y - R + i) * w;
                T k = g.k[i];
                for (int64_t x = 0; x < w; x++) acc[x] += row[x] * k;
            }
            for (int64_t x = 0; x < w; x++) dst[y * w + x] = acc[x] / tot;
        }
    });
}

// =============================================================================================
// SSIMULACRA2

// ssimu2/makeXYB.hpp:4-50 (opsin_absorbance, linear_rgb_to_xyb, mixed_to_xyb, make_positive_xyb)
template <typename T>
inline void positive_xyb(T& r, T& g, T& b) {
    const T bias = (T)0.0037930734f;
    T ox = std::fma((T)0.30f, r, std::fma((T)0.622f, g, std::fma((T)0.078f, b, bias)));
    T oy = std::fma((T)0.23f, r, std::fma((T)0.692f, g, std::fma((T)0.078f, b, bias)));
    T oz = std::fma((T)0.24342269f, r, std::fma((T)0.20476745f, g, std::fma((T)0.55180986f, b, bias)));
    const T abs_bias = (T)-0.1559542025327239f;
    ox = std::cbrt(ox * (T)(ox >= 0)) + abs_bias;
    oy = std::cbrt(oy * (T)(oy >= 0)) + abs_bias;
    oz = std::cbrt(oz * (T)(oz >= 0)) + abs_bias;
    T X = (T)0.5f * (ox - oy);
    T Y = X + oy;
    T B = oz;
    B = addD(B - Y, 0.55);
    X = addD(X * (T)14.0f, 0.42);
    Y = addD(Y, 0.01);
    r = X;
    g = Y;
    b = B;
}

// ssimu2/score.hpp:272-379: the 108 SSIMULACRA2 feature weights (the published SSIMULACRA2
// model). Order: plane*36 + scale*6 + norm*3 + map.
const double kSsimu2Weights[108] = {
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

// ssimu2/score.hpp:383-401 (final_score). The FP32 instantiation keeps the reference's float
// accumulator and its double-promoted polynomial; the FP64 one is all double.
template <typename T> double final_score(const T* s108);
template <> double final_score<float>(const float* s) {
    float ssim = 0.0f;
    for (int i = 0; i < 108; i++) ssim = std::fma((float)kSsimu2Weights[i], s[i], ssim);
    ssim = (float)((double)ssim * 0.9562382616834844);
    double x = ssim;
    ssim = (float)((6.248496625763138e-5 * x * x) * x + 2.326765642916932 * x - 0.020884521182843837 * x * x);
    if (ssim > 0.0) ssim = (float)(std::pow((double)ssim, 0.6276336467831387) * -10.0 + 100.0);
    else ssim = 100.0f;
    return ssim;
}
template <> double final_score<double>(const double* s) {
    double ssim = 0.0;
    for (int i = 0; i < 108; i++) ssim = std::fma(kSsimu2Weights[i], s[i], ssim);
    ssim *= 0.9562382616834844;
    ssim = (6.248496625763138e-5 * ssim * ssim) * ssim + 2.326765642916932 * ssim - 0.020884521182843837 * ssim * ssim;
    if (ssim > 0.0) return std::pow(ssim, 0.6276336467831387) * -10.0 + 100.0;
    return 100.0;
}

// ssimu2/score.hpp:95-196 (allscore_map_Kernel) for one scale and one channel: returns the six
// means {ssim, ssim^4, artifact, artifact^4, detail, detail^4} over the scale.
template <typename T>
void ssimu2_channel_stats(const T* i1, const T* i2, int64_t w, int64_t h, const Kernel<T>& g,
                          int nthreads, double out[6]) {
    const int64_t n = w * h;
    std::vector<T> p11(n), p22(n), p12(n), tmp(n);
    std::vector<T> m1(n), m2(n), s11(n), s22(n), s12(n);
    for (int64_t i = 0; i < n; i++) {
        p11[i] = i1[i] * i1[i];
        p22[i] = i2[i] * i2[i];
        p12[i] = i1[i] * i2[i];
    }
    blur(i1, m1.data(), tmp.data(), w, h, g, nthreads);
    blur(i2, m2.data(), tmp.data(), w, h, g, nthreads);
    blur(p11.data(), s11.data(), tmp.data(), w, h, g, nthreads);
    blur(p22.data(), s22.data(), tmp.data(), w, h, g, nthreads);
    blur(p12.data(), s12.data(), tmp.data(), w, h, g, nthreads);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < n; i++) {
        T a = m1[i], b = m2[i];
        T m11 = a * a, m22 = b * b, m12 = a * b, md = a - b;
        T num_m = std::fma(md, -md, (T)1);
        T num_s = std::fma(s12[i] - m12, (T)2, (T)0.0009f);
        T denom = (s11[i] - m11) + (s22[i] - m22) + (T)0.0009f;
        T d0 = std::max((T)1 - (num_m * num_s) / denom, (T)0);
        T v1 = (std::fabs(i2[i] - b) + (T)1) / (std::fabs(i1[i] - a) + (T)1) - (T)1;
        T d1 = std::max(v1, (T)0), d2 = std::max(-v1, (T)0);
        T q0 = d0 * d0, q1 = d1 * d1, q2 = d2 * d2;
        acc[0] += d0; acc[1] += q0 * q0;
        acc[2] += d1; acc[3] += q1 * q1;
        acc[4] += d2; acc[5] += q2 * q2;
    }
    for (int k = 0; k < 6; k++) out[k] = acc[k] / (double)n;
}

// ssimu2/main.hpp:34-151 (getTotalScaleSize, ssimu2GPUProcess, ssimu2process)
// FP16 storage model for the XYB pyramid: each value is stored as half(v - offset[c]).
const double kXybHalfOffset[3] = {0.42, 0.45, 0.55};

template <typename T>
double ssimu2(const uint8_t* const* src1, const uint8_t* const* src2, int64_t stride1, int64_t stride2,
              int64_t w, int64_t h, int intype, int nthreads, T* measure_out, int storage16 = 0) {
    const Kernel<T> g = ssimu2_kernel<T>();
    // planar linear RGB at every scale, both images
    std::vector<Dims> dims;
    int64_t cw = w, ch = h;
    for (int s = 0; s < 6; s++) {
        dims.push_back({cw, ch});
        cw = half_dim(cw);
        ch = half_dim(ch);
    }
    std::vector<std::vector<T>> img[2];
    for (int m = 0; m < 2; m++) {
        img[m].resize(6 * 3);
        const uint8_t* const* src = m == 0 ? src1 : src2;
        int64_t stride = m == 0 ? stride1 : stride2;
        for (int c = 0; c < 3; c++) {
            std::vector<T>& p = img[m][c];
            p.resize(w * h);
            for (int64_t y = 0; y < h; y++)
                for (int64_t x = 0; x < w; x++) p[y * w + x] = to_linear(decode<T>(src[c], stride, x, y, intype));
        }
        for (int s = 1; s < 6; s++)
            for (int c = 0; c < 3; c++) {
                img[m][s * 3 + c].resize(dims[s].w * dims[s].h);
                downsample(img[m][(s - 1) * 3 + c].data(), img[m][s * 3 + c].data(), dims[s - 1].w, dims[s - 1].h);
            }
        for (int s = 0; s < 6; s++) {
            int64_t n = dims[s].w * dims[s].h;
            T* r = img[m][s * 3 + 0].data();
            T* gg = img[m][s * 3 + 1].data();
            T* b = img[m][s * 3 + 2].data();
            for (int64_t i = 0; i < n; i++) {
                positive_xyb(r[i], gg[i], b[i]);
                if (storage16 == 1) {
                    r[i] = round_half(r[i] - (T)kXybHalfOffset[0]) + (T)kXybHalfOffset[0];
                    gg[i] = round_half(gg[i] - (T)kXybHalfOffset[1]) + (T)kXybHalfOffset[1];
                    b[i] = round_half(b[i] - (T)kXybHalfOffset[2]) + (T)kXybHalfOffset[2];
                }
            }
        }
        if (storage16 == 2 && m == 1) {  // distorted pyramid stored as FP16 differences
            for (int k = 0; k < 18; k++) {
                std::vector<T>& d = img[1][k];
                const std::vector<T>& r = img[0][k];
                for (size_t i = 0; i < d.size(); i++) d[i] = r[i] + round_half(d[i] - r[i]);
            }
        }
    }
    // res[scale][channel][6]
    double res[6][3][6];
    for (int s = 0; s < 6; s++)
        for (int c = 0; c < 3; c++)
            ssimu2_channel_stats(img[0][s * 3 + c].data(), img[1][s * 3 + c].data(), dims[s].w, dims[s].h, g,
                                 nthreads, res[s][c]);
    // ssimu2/score.hpp:263-267: 4th root of the 4-norm means; ssimu2/main.hpp:83-95 permutation
    T measure[108];
    for (int plane = 0; plane < 3; plane++)
        for (int s = 0; s < 6; s++)
            for (int nrm = 0; nrm < 2; nrm++)
                for (int i = 0; i < 3; i++) {
                    double v = res[s][plane][i * 2 + nrm];
                    T tv = (T)v;
                    if (nrm == 1) tv = std::sqrt(std::sqrt(tv));
                    measure[plane * 36 + s * 6 + nrm * 3 + i] = tv;
                }
    if (measure_out) std::memcpy(measure_out, measure, sizeof(measure));
    return final_score<T>(measure);
}

// =============================================================================================
// Butteraugli

// butter/colors.hpp:3-5
template <typename T> inline T gamma_fn(T v) {
    return std::fma((T)19.245013259874995f, std::log(addD(v, 9.9710635769299145)), (T)-23.16046239805755f);
}

// butter/colors.hpp:25-49
template <typename T> inline void butter_opsin(T& x, T& y, T& z, bool clamp) {
    T ox = std::fma((T)0.29956550340058319f, x, std::fma((T)0.63373087833825936f, y,
           std::fma((T)0.077705617820981968f, z, (T)1.7557483643287353f)));
    T oy = std::fma((T)0.22158691104574774f, x, std::fma((T)0.69391388044116142f, y,
           std::fma((T)0.0987313588422f, z, (T)1.7557483643287353f)));
    T oz = std::fma((T)0.02f, x, std::fma((T)0.02f, y, std::fma((T)0.20480129041026129f, z, (T)12.226454707163354f)));
    if (clamp) {
        ox = std::max(ox, (T)1.7557483643287353f);
        oy = std::max(oy, (T)1.7557483643287353f);
        oz = std::max(oz, (T)12.226454707163354f);
    }
    x = ox; y = oy; z = oz;
}

// butter/separatefrequencies.hpp:24-51
template <typename T> inline T maximum_clamp(T v, T maxval) {
    const T kMul = (T)0.688059627878f;
    if (v >= maxval) { v -= maxval; v *= kMul; v += maxval; }
    else if (v < -maxval) { v += maxval; v *= kMul; v -= maxval; }
    return v;
}
template <typename T> inline T amplify_range(T x, T w) { return x > w ? x + w : x < -w ? x - w : (T)2 * x; }
template <typename T> inline T remove_range(T x, T w) { return x > w ? x - w : x < -w ? x + w : (T)0; }

// Malta line patterns (butter/maltaDiff.hpp:4-512, after google butteraugli): 16 oriented lines
// through the centre, given as (dx, dy) offsets in summation order. "HF" is the long-tap unit
// (MaltaUnit), "LF" the 5-tap unit (MaltaUnitLF).
struct Tap { int dx, dy; };
struct Pattern { int n; Tap t[9]; };

const Pattern kMaltaHF[16] = {
    {9, {{-4, 0}, {-3, 0}, {-2, 0}, {-1, 0}, {0, 0}, {1, 0}, {2, 0}, {3, 0}, {4, 0}}},
    {9, {{0, -4}, {0, -3}, {0, -2}, {0, -1}, {0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}}},
    {7, {{-3, -3}, {-2, -2}, {-1, -1}, {0, 0}, {1, 1}, {2, 2}, {3, 3}}},
    {7, {{3, -3}, {2, -2}, {1, -1}, {0, 0}, {-1, 1}, {-2, 2}, {-3, 3}}},
    {9, {{1, -4}, {1, -3}, {1, -2}, {0, -1}, {0, 0}, {0, 1}, {-1, 2}, {-1, 3}, {-1, 4}}},
    {9, {{-1, -4}, {-1, -3}, {-1, -2}, {0, -1}, {0, 0}, {0, 1}, {1, 2}, {1, 3}, {1, 4}}},
    {9, {{-4, -1}, {-3, -1}, {-2, -1}, {-1, 0}, {0, 0}, {1, 0}, {2, 1}, {3, 1}, {4, 1}}},
    {9, {{-4, 1}, {-3, 1}, {-2, 1}, {-1, 0}, {0, 0}, {1, 0}, {2, -1}, {3, -1}, {4, -1}}},
    {7, {{-2, -3}, {-1, -2}, {-1, -1}, {0, 0}, {1, 1}, {1, 2}, {2, 3}}},
    {7, {{2, -3}, {1, -2}, {1, -1}, {0, 0}, {-1, 1}, {-1, 2}, {-2, 3}}},
    {7, {{-3, -2}, {-2, -1}, {-1, -1}, {0, 0}, {1, 1}, {2, 1}, {3, 2}}},
    {7, {{3, -2}, {2, -1}, {1, -1}, {0, 0}, {-1, 1}, {-2, 1}, {-3, 2}}},
    {8, {{-4, 2}, {-3, 2}, {-2, 1}, {-1, 1}, {0, 0}, {1, 0}, {2, -1}, {3, -1}}},
    {8, {{-4, -2}, {-3, -2}, {-2, -1}, {-1, -1}, {0, 0}, {1, 0}, {2, 1}, {3, 1}}},
    {8, {{-2, -4}, {-2, -3}, {-1, -2}, {-1, -1}, {0, 0}, {0, 1}, {1, 2}, {1, 3}}},
    {8, {{2, -4}, {2, -3}, {1, -2}, {1, -1}, {0, 0}, {0, 1}, {-1, 2}, {-1, 3}}},
};
const Pattern kMaltaLF[16] = {
    {5, {{-4, 0}, {-2, 0}, {0, 0}, {2, 0}, {4, 0}}},
    {5, {{0, -4}, {0, -2}, {0, 0}, {0, 2}, {0, 4}}},
    {5, {{-3, -3}, {-2, -2}, {0, 0}, {2, 2}, {3, 3}}},
    {5, {{3, -3}, {2, -2}, {0, 0}, {-2, 2}, {-3, 3}}},
    {5, {{1, -4}, {1, -2}, {0, 0}, {-1, 2}, {-1, 4}}},
    {5, {{-1, -4}, {-1, -2}, {0, 0}, {1, 2}, {1, 4}}},
    {5, {{-4, -1}, {-2, -1}, {0, 0}, {2, 1}, {4, 1}}},
    {5, {{-4, 1}, {-2, 1}, {0, 0}, {2, -1}, {4, -1}}},
    {5, {{-2, -3}, {-1, -2}, {0, 0}, {1, 2}, {2, 3}}},
    {5, {{2, -3}, {1, -2}, {0, 0}, {-1, 2}, {-2, 3}}},
    {5, {{-3, -2}, {-2, -1}, {0, 0}, {2, 1}, {3, 2}}},
    {5, {{3, -2}, {2, -1}, {0, 0}, {-2, 1}, {-3, 2}}},
    {5, {{-4, 2}, {-2, 1}, {0, 0}, {2, -1}, {4, -2}}},
    {5, {{-4, -2}, {-2, -1}, {0, 0}, {2, 1}, {4, 2}}},
    {5, {{-2, -4}, {-1, -2}, {0, 0}, {1, 2}, {2, 4}}},
    {5, {{2, -4}, {1, -2}, {0, 0}, {-1, 2}, {-2, 4}}},
};

// butter/maltaDiff.hpp:514-600 (diff precompute of MaltaDiffMap[_LF]_Kernel) and :602-660
// (pattern sum), accumulated into ac.
template <typename T>
void malta_diff(const T* l0, const T* l1, T* ac, int64_t w, int64_t h, T w_0gt1, T w_0lt1, T norm1,
                bool hf_unit, int nthreads) {
    const T mulli = hf_unit ? (T)0.39905817637f : (T)0.611612573796f;
    const T kWeight0 = (T)0.5f, kWeight1 = (T)0.33f;
    const T len2 = (T)3.75f * (T)2.0f + (T)1.0f;
    const T w_pre0gt1 = mulli * std::sqrt(kWeight0 * w_0gt1) / len2;
    const T w_pre0lt1 = mulli * std::sqrt(kWeight1 * w_0lt1) / len2;
    const T norm2_0gt1 = w_pre0gt1 * norm1;
    const T norm2_0lt1 = w_pre0lt1 * norm1;
    const int64_t n = w * h;
    std::vector<T> d(n);
    for (int64_t i = 0; i < n; i++) {
        T a = l0[i], b = l1[i];
        T absval = (T)0.5f * std::fabs(a) + (T)0.5f * std::fabs(b);
        T diff = a - b;
        T scaler = norm2_0gt1 / (norm1 + absval);
        T v = scaler * diff;
        T scaler2 = norm2_0lt1 / (norm1 + absval);
        T fabs0 = std::fabs(a);
        T too_small = (T)0.55f * fabs0, too_big = (T)1.05f * fabs0;
        T impact = 0;
        if (a < (T)0) {
            if (b > -too_small) impact = b + too_small;
            else if (b < -too_big) impact = -b - too_big;
        } else {
            if (b < too_small) impact = -b + too_small;
            else if (b > too_big) impact = b - too_big;
        }
        impact *= scaler2;
        if (diff < (T)0) v -= impact;
        else v += impact;
        d[i] = v;
    }
    const Pattern* pats = hf_unit ? kMaltaHF : kMaltaLF;
    parallel_rows(h, nthreads, [&](int64_t y0, int64_t y1) {
        for (int64_t y = y0; y < y1; y++)
            for (int64_t x = 0; x < w; x++) {
                T ret = 0;
                for (int p = 0; p < 16; p++) {
                    T sum = 0;
                    for (int t = 0; t < pats[p].n; t++) {
                        int64_t xx = x + pats[p].t[t].dx, yy = y + pats[p].t[t].dy;
                        T v = (xx >= 0 && xx < w && yy >= 0 && yy < h) ? d[yy * w + xx] : (T)0;
                        sum = t == 0 ? v : sum + v;
                    }
                    ret += sum * sum;
                }
                ac[y * w + x] += ret;
            }
    });
}

// butter/simplerdiff.hpp:41-59 (L2diff_Kernel, L2diff)
template <typename T> void l2diff(const T* a, const T* b, T* dst, int64_t n, T w) {
    if (w == (T)0) return;
    for (int64_t i = 0; i < n; i++) {
        T diff = a[i] - b[i];
        dst[i] += w * diff * diff;
    }
}

// butter/simplerdiff.hpp:61-100 (L2AsymDiff_Kernel, L2AsymDiff; including the extra x0.8 applied to
// both weights at :94-95)
template <typename T> void l2asym(const T* a, const T* b, T* dst, int64_t n, T w_gt, T w_lt) {
    if (w_gt == (T)0 && w_lt == (T)0) return;
    w_gt = mulD(w_gt, 0.8);
    w_lt = mulD(w_lt, 0.8);
    for (int64_t i = 0; i < n; i++) {
        T s1 = a[i], s2 = b[i];
        T diff = s1 - s2;
        dst[i] += w_gt * diff * diff;
        T fabs0 = std::fabs(s1);
        T too_small = mulD(fabs0, 0.4), too_big = fabs0;
        if (s1 < (T)0) {
            if (s2 > -too_small) { T v = s2 + too_small; dst[i] += w_lt * v * v; }
            else if (s2 < -too_big) { T v = -s2 - too_big; dst[i] += w_lt * v * v; }
        } else {
            if (s2 < too_small) { T v = too_small - s2; dst[i] += w_lt * v * v; }
            else if (s2 > too_big) { T v = s2 - too_big; dst[i] += w_lt * v * v; }
        }
    }
}

// butter/maskPsycho.hpp:42-104
template <typename T> inline void store_min3(T v, T& m0, T& m1, T& m2) {
    if (v < m2) {
        if (v < m0) { m2 = m1; m1 = m0; m0 = v; }
        else if (v < m1) { m2 = m1; m1 = v; }
        else m2 = v;
    }
}
template <typename T> void fuzzy_erosion(const T* src, T* dst, int64_t w, int64_t h) {
    const int64_t k = 3;
    for (int64_t y = 0; y < h; y++)
        for (int64_t x = 0; x < w; x++) {
            T m0 = src[y * w + x], m1 = (T)2 * m0, m2 = m1;
            if (x >= k) {
                store_min3(src[y * w + x - k], m0, m1, m2);
                if (y >= k) store_min3(src[(y - k) * w + x - k], m0, m1, m2);
                if (y < h - k) store_min3(src[(y + k) * w + x - k], m0, m1, m2);
            }
            if (x < w - k) {
                store_min3(src[y * w + x + k], m0, m1, m2);
                if (y >= k) store_min3(src[(y - k) * w + x + k], m0, m1, m2);
                if (y < h - k) store_min3(src[(y + k) * w + x + k], m0, m1, m2);
            }
            if (y >= k) store_min3(src[(y - k) * w + x], m0, m1, m2);
            if (y < h - k) store_min3(src[(y + k) * w + x], m0, m1, m2);
            dst[y * w + x] = (T)0.45f * m0 + (T)0.3f * m1 + (T)0.25f * m2;
        }
}

// butter/combineMasks.hpp:3-19
template <typename T> inline T mask_y(T delta) {
    const T c = (T)2.5485944793f / (((T)0.451936922203f * delta) + (T)0.829591754942f);
    T r = (T)((1.0 + (double)c) * (1.0 / (double)(0.79079917404f * 17.83f)));
    return r * r;
}
template <typename T> inline T mask_dc_y(T delta) {
    const T c = (T)0.505054525019f / (((T)3.87449418804f * delta) + (T)0.20025578522f);
    T r = (T)((1.0 + (double)c) * (1.0 / (double)(0.79079917404f * 17.83f)));
    return r * r;
}

template <typename T> struct ButterKernels { Kernel<T> k[5]; };

// Per-image bands of butter/separatefrequencies.hpp:160-203.
template <typename T> struct Bands {
    std::vector<T> lf[3], mf[3], hf[2], uhf[2];
};

// butter/colors.hpp:51-91 (opsinDynamicsImage) then separatefrequencies.hpp:160-203
template <typename T>
void psycho_image(std::vector<T> src[3], int64_t w, int64_t h, float intensity, const ButterKernels<T>& K,
                  int nthreads, Bands<T>& out) {
    const int64_t n = w * h;
    std::vector<T> tmp(n), blurred[3];
    for (int c = 0; c < 3; c++) {
        blurred[c].resize(n);
        blur(src[c].data(), blurred[c].data(), tmp.data(), w, h, K.k[0], nthreads);
    }
    const T im = (T)intensity;
    for (int64_t i = 0; i < n; i++) {
        T sx = src[0][i] * im, sy = src[1][i] * im, sz = src[2][i] * im;
        T bx = blurred[0][i] * im, by = blurred[1][i] * im, bz = blurred[2][i] * im;
        butter_opsin(bx, by, bz, true);
        bx = std::max(bx, (T)1e-4f); by = std::max(by, (T)1e-4f); bz = std::max(bz, (T)1e-4f);
        T ex = std::max(gamma_fn(bx) / bx, (T)1e-4f);
        T ey = std::max(gamma_fn(by) / by, (T)1e-4f);
        T ez = std::max(gamma_fn(bz) / bz, (T)1e-4f);
        butter_opsin(sx, sy, sz, false);
        sx *= ex; sy *= ey; sz *= ez;
        sx = std::max(sx, (T)1.7557483643287353f);
        sy = std::max(sy, (T)1.7557483643287353f);
        sz = std::max(sz, (T)12.226454707163354f);
        src[0][i] = sx - sy;
        src[1][i] = sx + sy;
        src[2][i] = sz;
    }
    // frequency separation
    for (int c = 0; c < 3; c++) {
        out.lf[c].resize(n);
        out.mf[c].resize(n);
        blur(src[c].data(), out.lf[c].data(), tmp.data(), w, h, K.k[4], nthreads);
    }
    std::vector<T> hf_pre[2];
    for (int c = 0; c < 3; c++) {
        std::vector<T> d(n);
        for (int64_t i = 0; i < n; i++) d[i] = src[c][i] - out.lf[c][i];
        blur(d.data(), out.mf[c].data(), tmp.data(), w, h, K.k[3], nthreads);
        if (c == 2) break;
        hf_pre[c].resize(n);
        for (int64_t i = 0; i < n; i++) {
            hf_pre[c][i] = d[i] - out.mf[c][i];
            out.mf[c][i] = c == 0 ? remove_range(out.mf[c][i], (T)0.29f) : amplify_range(out.mf[c][i], (T)0.1f);
        }
    }
    // separatefrequencies.hpp:37-41 (supressXbyY, yw = 46)
    const T s = (T)0.653020556257f, yw = (T)46.0f;
    for (int64_t i = 0; i < n; i++) {
        T yv = hf_pre[1][i];
        hf_pre[0][i] *= s + (yw * ((T)1.0f - s)) / (yw + yv * yv);
    }
    for (int c = 0; c < 2; c++) {
        out.hf[c].resize(n);
        out.uhf[c].resize(n);
        blur(hf_pre[c].data(), out.hf[c].data(), tmp.data(), w, h, K.k[1], nthreads);
        for (int64_t i = 0; i < n; i++) {
            T hf = out.hf[c][i], uhf = hf_pre[c][i];
            if (c == 0) {
                uhf -= hf;
                hf = remove_range(hf, (T)1.5f);
                uhf = remove_range(uhf, (T)0.04f);
            } else {  // separatefrequencies.hpp:117-133
                hf = maximum_clamp(hf, (T)28.4691806922f);
                uhf -= hf;
                uhf = maximum_clamp(uhf, (T)5.19175294647f);
                uhf *= (T)2.69313763794f;
                hf *= (T)2.155f;
                hf = amplify_range(hf, (T)0.132f);
            }
            out.hf[c][i] = hf;
            out.uhf[c][i] = uhf;
        }
    }
    // separatefrequencies.hpp:3-12 (XybLowFreqToVals)
    for (int64_t i = 0; i < n; i++) {
        T x = out.lf[0][i], y = out.lf[1][i], b = out.lf[2][i];
        b = b + (T)-0.362267051518f * y;
        b = b * (T)49.87984651440f;
        x = x * (T)33.832837186260f;
        y = y * (T)14.458268100570f;
        out.lf[0][i] = x; out.lf[1][i] = y; out.lf[2][i] = b;
    }
}

// butter/main.hpp:23-113 (getdiffmap) for one scale
// half_bands models FP16 storage of the frequency bands that the pair stage reads: 1 = every
// band of both images rounded to half; 2 = reference bands exact, distorted bands stored as
// half(distorted - reference) and read back as reference + delta; 3 = as 2 but the LF bands
// kept exact; 4 = the UHF bands of both images rounded to half, the others exact (the CUDA
// path's half-band storage).
template <typename T>
void store_bands_half(Bands<T>& b1, Bands<T>& b2, int half_bands) {
    auto each = [&](std::vector<T>& a, std::vector<T>& b) {
        for (size_t i = 0; i < a.size(); i++) {
            if (half_bands == 1 || half_bands == 4) {
                a[i] = round_half(a[i]);
                b[i] = round_half(b[i]);
            } else {
                b[i] = a[i] + round_half(b[i] - a[i]);
            }
        }
    };
    if (half_bands != 4) {
        for (int c = 0; c < 3; c++) {
            if (half_bands != 3) each(b1.lf[c], b2.lf[c]);
            each(b1.mf[c], b2.mf[c]);
        }
        for (int c = 0; c < 2; c++) each(b1.hf[c], b2.hf[c]);
    }
    for (int c = 0; c < 2; c++) each(b1.uhf[c], b2.uhf[c]);
}

template <typename T>
std::vector<T> butter_diffmap(std::vector<T> src1[3], std::vector<T> src2[3], int64_t w, int64_t h, float intensity,
                              const ButterKernels<T>& K, int nthreads, int half_bands = 0) {
    const int64_t n = w * h;
    Bands<T> b1, b2;
    psycho_image(src1, w, h, intensity, K, nthreads, b1);
    psycho_image(src2, w, h, intensity, K, nthreads, b2);
    if (half_bands) store_bands_half(b1, b2, half_bands);
    std::vector<T> ac[3], dc[3];
    for (int c = 0; c < 3; c++) { ac[c].assign(n, (T)0); dc[c].assign(n, (T)0); }
    const T hf_asym = (T)0.8f;
    const T sq = std::sqrt(hf_asym);
    malta_diff(b1.uhf[1].data(), b2.uhf[1].data(), ac[1].data(), w, h, (T)1.10039032555f * hf_asym,
               (T)1.10039032555f / hf_asym, (T)71.7800275169f, true, nthreads);
    malta_diff(b1.uhf[0].data(), b2.uhf[0].data(), ac[0].data(), w, h, (T)173.5f * hf_asym, (T)173.5f / hf_asym,
               (T)5.0f, true, nthreads);
    malta_diff(b1.hf[1].data(), b2.hf[1].data(), ac[1].data(), w, h, (T)18.7237414387f * sq, (T)18.7237414387f / sq,
               (T)4498534.45232f, false, nthreads);
    malta_diff(b1.hf[0].data(), b2.hf[0].data(), ac[0].data(), w, h, (T)6923.99476109f * sq, (T)6923.99476109f / sq,
               (T)8051.15833247f, false, nthreads);
    malta_diff(b1.mf[1].data(), b2.mf[1].data(), ac[1].data(), w, h, (T)37.0819870399f, (T)37.0819870399f,
               (T)130262059.556f, false, nthreads);
    malta_diff(b1.mf[0].data(), b2.mf[0].data(), ac[0].data(), w, h, (T)8246.75321353f, (T)8246.75321353f,
               (T)1009002.70582f, false, nthreads);
    const T wmul[9] = {(T)400.0f, (T)1.50815703118f, (T)0.0f, (T)2150.0f, (T)10.6195433239f,
                       (T)16.2176043152f, (T)29.2353797994f, (T)0.844626970982f, (T)0.703646627719f};
    for (int c = 0; c < 3; c++) {
        if (c < 2) l2asym(b1.hf[c].data(), b2.hf[c].data(), ac[c].data(), n, wmul[c] * hf_asym, wmul[c] / hf_asym);
        l2diff(b1.mf[c].data(), b2.mf[c].data(), ac[c].data(), n, wmul[3 + c]);
        l2diff(b1.lf[c].data(), b2.lf[c].data(), dc[c].data(), n, wmul[6 + c]);
    }
    // butter/maskPsycho.hpp:113-135 (MaskPsychoImage)
    std::vector<T> mxyb[2], pre[2], blurred[2], tmp(n), mask(n);
    const Bands<T>* bb[2] = {&b1, &b2};
    const T mul = (T)6.19424080439f, bias = mul * (T)12.61050594197f, sqb = std::sqrt(bias);
    for (int m = 0; m < 2; m++) {
        mxyb[m].resize(n);
        pre[m].resize(n);
        blurred[m].resize(n);
        for (int64_t i = 0; i < n; i++) {
            T xd = (bb[m]->uhf[0][i] + bb[m]->hf[0][i]) * (T)2.5f;
            T yd = bb[m]->uhf[1][i] * (T)0.4f + bb[m]->hf[1][i] * (T)0.4f;
            mxyb[m][i] = std::sqrt(xd * xd + yd * yd);
            pre[m][i] = std::sqrt(mul * std::fabs(mxyb[m][i]) + bias) - sqb;
        }
        blur(pre[m].data(), blurred[m].data(), tmp.data(), w, h, K.k[2], nthreads);
    }
    fuzzy_erosion(blurred[0].data(), mask.data(), w, h);
    l2diff(blurred[0].data(), blurred[1].data(), ac[1].data(), n, (T)10.0f);
    // butter/combineMasks.hpp:21-40 (computeDiffmap_Kernel, computeDiffmap)
    std::vector<T> diffmap(n);
    for (int64_t i = 0; i < n; i++) {
        T v = mask[i];
        T sac = ac[0][i] + ac[1][i] + ac[2][i];
        T sdc = dc[0][i] + dc[1][i] + dc[2][i];
        diffmap[i] = std::sqrt(mask_y(v) * sac + mask_dc_y(v) * sdc);
    }
    return diffmap;
}

// butter/main.hpp:116-195 (getmultiscalediffmap, butterprocess) and diffnorms.hpp:86-129 (diffmapscore)
template <typename T>
void butteraugli(const uint8_t* const* src1, const uint8_t* const* src2, int64_t stride1, int64_t stride2, int64_t w,
                 int64_t h, int intype, int qnorm, float intensity, int nthreads, double norms[3], float* distmap,
                 int half_bands = 0) {
    ButterKernels<T> K;
    for (int i = 0; i < 5; i++) K.k[i] = butter_kernel<T>(i);
    const int64_t n = w * h, nw = half_dim(w), nh = half_dim(h);
    std::vector<T> full[2][3], half[2][3];
    for (int m = 0; m < 2; m++) {
        const uint8_t* const* src = m == 0 ? src1 : src2;
        int64_t stride = m == 0 ? stride1 : stride2;
        for (int c = 0; c < 3; c++) {
            full[m][c].resize(n);
            for (int64_t y = 0; y < h; y++)
                for (int64_t x = 0; x < w; x++) full[m][c][y * w + x] = to_linear(decode<T>(src[c], stride, x, y, intype));
            half[m][c].resize(nw * nh);
            downsample(full[m][c].data(), half[m][c].data(), w, h);
        }
    }
    std::vector<T> dm = butter_diffmap(full[0], full[1], w, h, intensity, K, nthreads, half_bands);
    std::vector<T> dms = butter_diffmap(half[0], half[1], nw, nh, intensity, K, nthreads, half_bands);
    // butter/downupsample.hpp:34-56 (addsupersample2X_kernel, addsupersample2X; w = 0.5)
    const T wsup = (T)0.5f;
    for (int64_t y = 0; y < h; y++)
        for (int64_t x = 0; x < w; x++) {
            T d = mulD(dm[y * w + x], 1.0 - 0.3 * (double)wsup);
            d += wsup * dms[(y / 2) * nw + x / 2];
            dm[y * w + x] = d;
        }
    double sq = 0, s3 = 0, mx = 0;
    for (int64_t i = 0; i < n; i++) {
        T d = dm[i];
        sq += (double)std::pow(d, (T)qnorm);
        s3 += (double)(std::fabs(d) * d * d);
        mx = std::max(mx, (double)std::fabs(d));
    }
    norms[0] = std::pow(sq / (double)n, 1.0 / (double)qnorm);
    norms[1] = std::pow(s3 / (double)n, 1.0 / 3.0);
    norms[2] = mx;
    if (distmap)
        for (int64_t i = 0; i < n; i++) distmap[i] = (float)dm[i];
}

}  // namespace

// =============================================================================================
// C entry points used by the Python test/bench harness (ctypes). precision: 32 or 64.

extern "C" {

int oracle_ssimu2(const uint8_t* const* src1, const uint8_t* const* src2, int64_t stride1, int64_t stride2,
                  int64_t width, int64_t height, int intype, int precision, int nthreads, double* score,
                  double* measure108) {
    if (width <= 0 || height <= 0 || !score) return 1;
    if (precision == 16 || precision == 17) {
        // FP64 arithmetic over an FP16-stored XYB pyramid: 16 = both pyramids as half(v - offset),
        // 17 = reference in full precision, distorted as half(distorted - reference)
        *score = ssimu2<double>(src1, src2, stride1, stride2, width, height, intype, nthreads, nullptr,
                                precision == 16 ? 1 : 2);
        return 0;
    }
    if (precision == 64) {
        double m[108];
        *score = ssimu2<double>(src1, src2, stride1, stride2, width, height, intype, nthreads, m);
        if (measure108) std::memcpy(measure108, m, sizeof(m));
    } else {
        float m[108];
        *score = ssimu2<float>(src1, src2, stride1, stride2, width, height, intype, nthreads, m);
        if (measure108)
            for (int i = 0; i < 108; i++) measure108[i] = m[i];
    }
    return 0;
}

int oracle_butteraugli(const uint8_t* const* src1, const uint8_t* const* src2, int64_t stride1, int64_t stride2,
                       int64_t width, int64_t height, int intype, int qnorm, float intensity, int precision,
                       int nthreads, double* norms3, float* distmap) {
    if (width <= 0 || height <= 0 || !norms3) return 1;
    // precision 16: FP32 with every band stored as half; 17: FP32 with the distorted image's
    // bands stored as half deltas against the reference's; 18: 17 with the LF bands exact;
    // 19: FP32 with the UHF bands stored as half
    if (precision == 64)
        butteraugli<double>(src1, src2, stride1, stride2, width, height, intype, qnorm, intensity, nthreads, norms3,
                            distmap);
    else
        butteraugli<float>(src1, src2, stride1, stride2, width, height, intype, qnorm, intensity, nthreads, norms3,
                           distmap, precision == 16 ? 1 : precision == 17 ? 2 : precision == 18 ? 3 : precision == 19 ? 4 : 0);
    return 0;
}

// Constant tables, exported so that tests can compare them with the reference source text.
int oracle_malta_pattern(int hf_unit, int index, int* dxdy18) {
    if (index < 0 || index >= 16) return -1;
    const Pattern& p = hf_unit ? kMaltaHF[index] : kMaltaLF[index];
    for (int t = 0; t < p.n; t++) {
        dxdy18[2 * t] = p.t[t].dx;
        dxdy18[2 * t + 1] = p.t[t].dy;
    }
    return p.n;
}

const double* oracle_ssimu2_weights() { return kSsimu2Weights; }

}  // extern "C"
