// ssimu2.h -- SSIMULACRA2 engine (host interface of ssimu2.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "common.cuh"

namespace vship {

// Side of the level-0 tile one pyramid CTA builds (all six levels of it).
constexpr int kPyrTile = 32;

// One pyramid level in device memory: planar FP32, rows padded to `pitch` floats.
struct Ssimu2Level {
    int w, h, pitch;
    int tiles_x, tiles_y;
    int seg;      // rows per stats-kernel segment at this level (576 or 192)
    int64_t off;  // element offset of the level inside one channel plane
};

// Geometry of the 6-scale pyramid and of the stats-kernel tiling (segments of 32 columns x
// `seg` rows, one CTA each).
struct Ssimu2Geom {
    Ssimu2Level lv[6];
    int tile_begin[7];
    int tiles_total;
    int64_t plane_elems;  // elements of one channel's whole pyramid
};

// tall: stats segments of 576 rows on the levels that keep enough of them (ssimu2.cu); otherwise
// 192 rows throughout. The pyramid layout is the same either way.
Ssimu2Geom make_ssimu2_geom(int64_t w, int64_t h, bool tall = false);

// Device workspace and launch sequence for up to `max_pairs` frame pairs of one resolution.
// Launches of at least this many pairs use the tall stats segments (geom_tall): 2 % more pairs/s
// at 1080p. Smaller launches keep 192-row segments, which spread one pair over more CTAs (a lone
// 1080p pair takes 12 % longer with the tall ones). The two tile the pooled sums differently, so
// scores of the two kinds of launch agree to FP32 rounding of the partial sums, not bit for bit.
constexpr int kSsimu2TallPairs = 16;

// Layout: pyr[pair][image][channel][plane_elems], partials[pair][tile][18], scores[pair]. With
// fp16 deltas the distorted images' pyramids are stored as half(distorted - reference) in d16
// [pair][channel][plane_elems], after the references' FP32 pyramids pyr[pair][channel][...].
class Ssimu2Engine {
public:
    int64_t w = 0, h = 0;
    int max_pairs = 0;
    bool fp16 = false;
    Ssimu2Geom geom{};       // 192-row stats segments: launches of fewer than kSsimu2TallPairs pairs
    Ssimu2Geom geom_tall{};  // 576-row segments where a level keeps enough of them: larger launches
    float* pyr = nullptr;
    __half* d16 = nullptr;
    float* partials = nullptr;
    double* scores = nullptr;

    int init(int64_t width, int64_t height, int max_pairs, bool fp16_deltas = false);
    void destroy();
    // frames_dev: 2*npairs FrameDesc in device memory (pair-major: reference, distorted).
    // Scores land in out_scores (device) or in this->scores when out_scores is null.
    // yuv: the Y'CbCr format of IN_YUV frames (null: 10-bit 4:2:0 BT.709 limited, left siting).
    int launch(const FrameDesc* frames_dev, int intype, int npairs, double* out_scores, cudaStream_t st,
               const YuvParams* yuv = nullptr);
    static size_t device_bytes(int64_t w, int64_t h, int pairs, bool fp16_deltas = false);
    static size_t pyramid_bytes(const Ssimu2Geom& g, int pairs, bool fp16_deltas);

private:
    int launch_fp16(const FrameDesc* frames_dev, int intype, int npairs, double* out_scores, cudaStream_t st,
                    const YuvParams& yp);
};

// For callers that supply the scratch themselves (noalloc.cu): upload this device's constant
// tables, the number of floats of scratch one pair needs, and the launch sequence for one pair
// with every intermediate placed in `scratch` and the two frame descriptors in frames_scratch.
int ssimu2_prepare_device();
size_t ssimu2_scratch_floats(const Ssimu2Geom& g);
int ssimu2_launch_scratch(const FrameDesc& ref, const FrameDesc& dist, int intype, const Ssimu2Geom& geom,
                          FrameDesc* frames_scratch, float* scratch, double* out_score, cudaStream_t st);

// ------------------------------------------------------------------------------------------
// Work-list form over many images of several resolutions (multi.cu builds the tables).
// One entry per image whose pyramid is built: sources write FP32 planes to f32; candidates
// write FP32 planes to f32, or (d16 != null) FP16 deltas against their source's planes `ref`.
struct Ssimu2MultiImage {
    int geom;
    FrameDesc fd;
    YuvParams yp;  // IN_YUV frames
    float* f32;
    void* d16;
    const float* ref;
};
// One scored pair: its geometry, the source pyramid, the candidate pyramid (FP32 or FP16
// deltas), the pair's [18][tiles_total] partial sums and where the score goes.
struct Ssimu2MultiPair {
    int geom;
    const float* src;
    const void* cand;
    float* partials;
    double* score;
};

int ssimu2_multi_prepare();
// shape: the stats kernel's tile shape, 0 = 48-row chunks through a ring of horizontal-pass
// rows, 1 = 64-row chunks through a carried buffer (same segments, same sums)
int ssimu2_multi_stats_blocks_per_sm(bool delta, int shape, int* blocks);
// items: {image, level-0 tile x, tile y, 0} in kPyrTile tiles, one CTA each. delta selects the FP16-delta store.
int ssimu2_multi_pyramid(const Ssimu2MultiImage* imgs, const int4* items, int nitems, const Ssimu2Geom* geoms,
                         int intype, bool delta, cudaStream_t st);
// Persistent: `grid` CTAs walk items {pair, tile} with stride grid.
int ssimu2_multi_stats(const Ssimu2MultiPair* pairs, const int2* items, int nitems, const Ssimu2Geom* geoms,
                       bool delta, int grid, int shape, cudaStream_t st);
int ssimu2_default_stats_shape();  // the shape the per-pair entry points use
int ssimu2_multi_finalize(const Ssimu2MultiPair* pairs, int npairs, const Ssimu2Geom* geoms, cudaStream_t st);

}  // namespace vship
