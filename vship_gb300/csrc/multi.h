// multi.h -- batched multi-resolution scoring with source reuse (host interface of multi.cu).
//
// One call scores many (source, candidate) pairs whose sources come in up to kMaxRes
// resolutions; every source is shared by any number of candidates (an encoder's rate/quality
// search scores one source frame against several encodes of it). Per call:
//   SSIMULACRA2  -- one work-list pyramid launch for the sources (FP32 XYB pyramids, built once
//                   per source), one for the candidates (FP32, or FP16 deltas against their
//                   source's pyramid), one persistent stats launch over (pair, tile) items of all
//                   resolutions, one finalize launch;
//   Butteraugli  -- per resolution, chunks of (source, its candidates) groups: every image's own
//                   stage (decode, opsin, frequency bands) once per chunk, then every pair's
//                   stage against its source's planes.
// The launch sequence of a given batch layout is captured once in a CUDA graph and replayed
// while the layout (resolution of each source, source of each candidate, sample type) repeats.
// Launch knobs (persistent grid, work order) come from a small autotuner whose choices are
// cached in a JSON file.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "butter.h"
#include "common.cuh"
#include "ssimu2.h"

namespace vship {

enum : int {
    MULTI_SSIMU2 = 1,
    MULTI_BUTTERAUGLI = 2,
    MULTI_FP16 = 4,      // candidate SSIMU2 pyramids stored as FP16 deltas
    MULTI_NO_GRAPH = 8,  // launch directly instead of replaying a CUDA graph
    MULTI_AUTOTUNE = 16,     // time the launch-knob candidates on the first call of a new layout
    MULTI_BUTTER_HALF = 32   // Butteraugli UHF bands stored as FP16 (ButterEngine::half_bands)
};
constexpr int kMaxRes = 8;

// SSIMU2 launch knobs chosen by the autotuner.
struct MultiKnobs {
    int grid_per_sm = 2;  // persistent stats grid = grid_per_sm x SMs (0 = one CTA per item)
    int order = 0;        // 0 = source-tile-major (a source tile's candidates back to back), 1 = pair-major
    int shape = 0;        // stats tile shape: 0 = 48-row chunks through a ring, 1 = 64-row chunks, carried halo
};

class MultiEngine {
public:
    int flags = 0;
    int nres = 0;
    int64_t rw[kMaxRes]{}, rh[kMaxRes]{};
    int max_src[kMaxRes]{}, max_pairs[kMaxRes]{};
    int src_cap = 0, pair_cap = 0;
    int device = 0, sms = 0;
    int qnorm = 2;
    float intensity = 203.f;
    std::string tune_path;
    std::string device_name;

    int init(int nres, const int* widths, const int* heights, const int* max_sources, const int* max_pairs,
             int flags, int qnorm, float intensity, const char* tune_cache_path);
    void destroy();
    // src/cand: HOST arrays of frame descriptors pointing at device planes.
    int compute(int nsrc, const FrameDesc* src, const int* src_res, int npairs, const FrameDesc* cand,
                const int* cand_src, int intype, double* ssimu2_dev, double* butter_dev, cudaStream_t st);
    // Format of IN_YUV frames for every resolution (make_yuv_params; matrix 2 resolves per height).
    int set_yuv_format(int bits, int ssw, int ssh, int matrix, int range, int loc, int transfer = 1,
                       int primaries = 1);
    // The knobs in use as JSON ({"grid_per_sm": g, "order": o, "source": "default|cache|tuned"}).
    std::string knobs_json() const;
    static size_t device_bytes(int nres, const int* widths, const int* heights, const int* max_sources,
                               const int* max_pairs, int flags);

private:
    // SSIMU2 state
    Ssimu2Geom geoms_h[kMaxRes]{};
    Ssimu2Geom* geoms_d = nullptr;
    float* s_src[kMaxRes]{};
    void* s_cand[kMaxRes]{};
    float* s_part[kMaxRes]{};
    double* s_scores = nullptr;
    Ssimu2MultiImage* s_imgs_d = nullptr;
    Ssimu2MultiImage* s_imgs_h = nullptr;  // pinned staging
    Ssimu2MultiPair* s_pairs_d = nullptr;
    int4* s_pitems_d = nullptr;
    int2* s_sitems_d = nullptr;
    int n_pitems_src = 0, n_pitems_cand = 0, n_sitems = 0;
    size_t cap_pitems = 0, cap_sitems = 0;
    int stats_blocks_per_sm = 1;  // resident stats CTAs per SM for the current knobs' shape
    int stats_bps[2] = {1, 1};    // ... for each tile shape
    // Butteraugli state: one image/pair engine per resolution, run over chunks
    struct BChunk {
        int res, img_off, nimg, pair_off, npairs;
    };
    ButterEngine b_eng[kMaxRes];
    int b_cap_img[kMaxRes]{}, b_cap_pair[kMaxRes]{};
    std::vector<BChunk> b_chunks;
    std::vector<int> b_img_of;        // chunk image -> caller frame (source i >= 0, candidate j as -1 - j)
    FrameDesc* b_frames_d = nullptr;  // chunk images' descriptors, all chunks back to back
    FrameDesc* b_frames_h = nullptr;  // pinned staging
    int2* b_pimg_d = nullptr;         // per grouped pair: (source, candidate) image inside its chunk
    double* b_norms_d = nullptr;      // grouped norms, then the caller-ordered copy
    int* b_perm_d = nullptr;          // grouped pair -> caller's pair index

    YuvParams yuv_r[kMaxRes];

    // current layout
    bool plan_valid = false;
    int plan_intype = -1;
    std::vector<int> plan_src_res, plan_cand_src;
    std::vector<int> src_slot, cand_slot;  // slot of each image inside its resolution's arena
    MultiKnobs knobs;
    const char* knobs_source = "default";

    cudaStream_t cap_stream = nullptr;
    cudaStream_t side[kMaxRes + 1]{};  // per-resolution Butteraugli streams, then SSIMULACRA2's
    cudaEvent_t ev_fork = nullptr, ev_join[kMaxRes + 1]{};
    cudaGraphExec_t gexec = nullptr;
    cudaEvent_t staging_free = nullptr;

    int build_plan(int nsrc, const int* src_res, int npairs, const int* cand_src, int intype, cudaStream_t st);
    int upload_items(cudaStream_t st);
    void fill_images(int nsrc, const FrameDesc* src, int npairs, const FrameDesc* cand);
    int enqueue(int npairs, cudaStream_t st);
    int autotune(int npairs, cudaStream_t st);
    std::string tune_key() const;
    bool tune_lookup(const std::string& key, MultiKnobs* k);
    void tune_store(const std::string& key, const MultiKnobs& k, double ms);
};

}  // namespace vship
