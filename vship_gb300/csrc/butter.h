// butter.h -- Butteraugli engine (host interface of butter.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "common.cuh"

namespace vship {

// Per-scale plane set of the Butteraugli pipeline (all planes dense FP32, pitch == width).
struct ButterScale {
    int w, h;
    int64_t n;  // w*h
};

// Device workspace and launch sequence of one resolution. The workspace holds up to max_images
// images (each its planes at both scales); a launch runs every image's own stage once, then
// every pair's stage on (reference image, distorted image) index pairs, so an image can serve
// as the reference of several pairs.
class ButterEngine {
public:
    int64_t w = 0, h = 0;
    int qnorm = 2;
    float intensity = 203.f;
    int max_pairs = 0, max_images = 0;
    // Keep the UHF bands as FP16 (set before init): 15 instead of 16 planes per image and scale;
    // the norms move by those bands' FP16 rounding (up to ~5e-5 relative, the inf-norm)
    bool half_bands = false;
    ButterScale sc[2]{};
    float* work = nullptr;          // all intermediate planes, [image][scale][plane]
    size_t img_floats = 0;          // per image
    float* partials = nullptr;      // norm partial sums
    int norm_blocks = 0;
    float* distmap = nullptr;       // [pair][h][w] (paired form)
    double* norms = nullptr;        // [pair][3]
    int2* pimg_identity = nullptr;  // (2p, 2p + 1): the paired form's pair table
    float** ibase = nullptr;        // device: base of image i = work + i * img_floats
    // the half scale's chain runs on `side` beside the full scale's (butter_enqueue)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

    // Paired form: images 2p and 2p + 1 are pair p's reference and distorted frames.
    int init(int64_t width, int64_t height, int qnorm, float intensity, int max_pairs);
    // Image/pair form; keep_distmap allocates this->distmap for max_pairs maps.
    int init_images(int64_t width, int64_t height, int qnorm, float intensity, int max_images, int max_pairs,
                    bool keep_distmap);
    void destroy();
    // frames_dev: 2*npairs FrameDesc in device memory (pair-major: reference, distorted).
    // Writes the final distortion maps to this->distmap and {Qnorm, 3-norm, inf-norm} to
    // norms_out (device, 3 doubles per pair) or to this->norms when norms_out is null.
    int launch(const FrameDesc* frames_dev, int intype, int npairs, double* norms_out, cudaStream_t st,
               const YuvParams* yuv = nullptr);
    // frames_dev: nimages FrameDesc (device); pimg: npairs (reference, distorted) image indices
    // (device); distmap_out: null or npairs maps.
    int launch_images(const FrameDesc* frames_dev, int nimages, const int2* pimg, int npairs, int intype,
                      double* norms_out, float* distmap_out, cudaStream_t st, const YuvParams* yuv = nullptr);
    static size_t device_bytes(int64_t w, int64_t h, int pairs, bool half_bands = false);
    static size_t image_bytes(int64_t w, int64_t h, bool half_bands = false);
};

// Engine-free form (the serving runtime places images anywhere): upload this device's tables and
// kernel attributes; floats of one image's workspace; norm partials per pair (x3 floats).
int butter_prepare_device();
size_t butter_image_floats(int64_t w, int64_t h, bool half_bands = false);
int butter_norm_tiles(int64_t w, int64_t h);
// ib: device table of image workspaces; images [0, nstage) run their own stage (frames_dev[i]
// is image i's frame), then every pair of pimg (indices into ib) runs the pair stage. partials:
// npairs x 3 x norm_tiles floats; norms_out: npairs x 3 doubles; distmap_out: null or npairs maps;
// yuv: format of IN_YUV frames (null: 10-bit 4:2:0 BT.709 limited, left siting); half_bands:
// the images' layout (butter_image_floats). side, ev_fork, ev_join (optional): a second stream
// and two events of the caller's; the half scale's chain then runs on side beside the full
// scale's (the two share nothing until the full-scale diffmap adds the half-scale map), unless
// per-kernel profiling is on.
int butter_enqueue(int64_t w, int64_t h, int qnorm, float intensity, float* const* ib, const FrameDesc* frames_dev,
                   int nstage, const int2* pimg, int npairs, int intype, float* partials, double* norms_out,
                   float* distmap_out, cudaStream_t st, const YuvParams* yuv = nullptr, bool half_bands = false,
                   cudaStream_t side = nullptr, cudaEvent_t ev_fork = nullptr, cudaEvent_t ev_join = nullptr);

}  // namespace vship
