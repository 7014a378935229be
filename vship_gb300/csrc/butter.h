// butter.h -- Butteraugli engine (host interface of butter.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace vship {

struct FrameDesc;

// Per-scale plane set of the Butteraugli pipeline (all planes dense FP32, pitch == width).
struct ButterScale {
    int w, h;
    int64_t n;  // w*h
};

// Device workspace and launch sequence for up to `max_pairs` frame pairs of one resolution.
class ButterEngine {
public:
    int64_t w = 0, h = 0;
    int qnorm = 2;
    float intensity = 203.f;
    int max_pairs = 0;
    ButterScale sc[2]{};
    float* work = nullptr;       // all intermediate planes
    size_t work_floats = 0;      // per pair
    float* partials = nullptr;   // norm partial sums
    int norm_blocks = 0;
    float* distmap = nullptr;    // [pair][h][w]
    double* norms = nullptr;     // [pair][3]

    int init(int64_t width, int64_t height, int qnorm, float intensity, int max_pairs);
    void destroy();
    // frames_dev: 2*npairs FrameDesc in device memory (pair-major: reference, distorted).
    // Writes the final distortion maps to this->distmap and {Qnorm, 3-norm, inf-norm} to
    // norms_out (device, 3 doubles per pair) or to this->norms when norms_out is null.
    int launch(const FrameDesc* frames_dev, int intype, int npairs, double* norms_out, cudaStream_t st);
    static size_t device_bytes(int64_t w, int64_t h, int pairs);
};

}  // namespace vship
