// multi.cu -- batched multi-resolution scoring with source reuse (MultiEngine, multi.h).
//
// Device memory, per resolution r (all sized at init from the declared capacities):
//   SSIMU2     source pyramids   max_src[r]   x 3 x plane_elems FP32
//              candidate pyramids max_pairs[r] x 3 x plane_elems FP32, or FP16 deltas
//              partial sums      max_pairs[r] x 18 x tiles_total FP32
//   Butteraugli one ButterEngine holding b_cap_img[r] image workspaces; a batch of that resolution
//              runs as chunks of whole (source, candidates) groups that fit, a source's image
//              stage running once per chunk it appears in
// plus the small tables the kernels walk: image descriptors (re-uploaded every call from pinned
// staging, since the frame pointers change), pair table and work items (uploaded when the batch
// layout changes).
#include "multi.h"
#include "profile.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>

#include <unistd.h>

namespace vship {

// grouped Butteraugli norms -> caller's pair order
__global__ void multi_scatter_norms_kernel(const double* __restrict__ grouped, const int* __restrict__ perm,
                                           double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * n) {
        const int g = i / 3, k = i - 3 * (i / 3);
        out[3 * perm[g] + k] = grouped[i];
    }
}

// Bytes of Butteraugli image workspace per resolution: 6 GiB, or $VSHIP_BUTTER_CHUNK_BYTES.
static size_t butter_chunk_budget() {
    if (const char* e = getenv("VSHIP_BUTTER_CHUNK_BYTES")) {
        const long long v = atoll(e);
        if (v > 0) return (size_t)v;
    }
    return (size_t)6 << 30;
}

static void butter_caps(int64_t w, int64_t h, int max_src, int max_pairs, bool half_bands, int* cap_img,
                        int* cap_pair) {
    const size_t one = ButterEngine::image_bytes(w, h, half_bands);
    const int fit = (int)std::min<size_t>(1 << 20, std::max<size_t>(2, butter_chunk_budget() / one));
    *cap_img = std::min(fit, std::max(2, max_src + max_pairs));
    *cap_pair = std::max(1, std::min(max_pairs, *cap_img - 1));
}

size_t MultiEngine::device_bytes(int nres, const int* widths, const int* heights, const int* max_sources,
                                 const int* max_pairs, int flags) {
    size_t total = 0;
    for (int r = 0; r < nres; r++) {
        if (flags & MULTI_SSIMU2) {
            const Ssimu2Geom g = make_ssimu2_geom(widths[r], heights[r]);
            const size_t pe = (size_t)g.plane_elems;
            total += (size_t)max_sources[r] * 3 * pe * 4;
            total += (size_t)max_pairs[r] * 3 * pe * ((flags & MULTI_FP16) ? 2 : 4);
            total += (size_t)max_pairs[r] * 18 * g.tiles_total * 4;
            total += ((size_t)max_sources[r] + max_pairs[r]) * (size_t)ceil_div(widths[r], kPyrTile) *
                     (size_t)ceil_div(heights[r], kPyrTile) * sizeof(int4);
            total += (size_t)max_pairs[r] * g.tiles_total * sizeof(int2);
        }
        if ((flags & MULTI_BUTTERAUGLI) && max_pairs[r] > 0) {
            int ci = 0, cp = 0;
            const bool hb = (flags & MULTI_BUTTER_HALF) != 0;
            butter_caps(widths[r], heights[r], max_sources[r], max_pairs[r], hb, &ci, &cp);
            total += ButterEngine::image_bytes(widths[r], heights[r], hb) * ci +
                     (size_t)cp * (3 * 4 * (size_t)butter_norm_tiles(widths[r], heights[r]) + 24);
        }
    }
    return total;
}

int MultiEngine::init(int nres_, const int* widths, const int* heights, const int* max_sources, const int* maxp,
                      int flags_, int qnorm_, float intensity_, const char* tune_cache_path) {
    if (nres_ <= 0 || nres_ > kMaxRes) return E_BAD_POINTER;
    if (!widths || !heights || !max_sources || !maxp) return E_BAD_POINTER;
    if (!(flags_ & (MULTI_SSIMU2 | MULTI_BUTTERAUGLI))) return E_BAD_POINTER;
    nres = nres_;
    flags = flags_;
    qnorm = qnorm_;
    intensity = intensity_;
    for (int r = 0; r < nres; r++) {
        if (widths[r] <= 0 || heights[r] <= 0 || max_sources[r] < 0 || maxp[r] < 0) return E_BAD_POINTER;
        rw[r] = widths[r];
        rh[r] = heights[r];
        max_src[r] = max_sources[r];
        max_pairs[r] = maxp[r];
        src_cap += max_src[r];
        pair_cap += max_pairs[r];
    }
    if (src_cap <= 0 || pair_cap <= 0) return E_BAD_POINTER;
    for (int r = 0; r < nres; r++) yuv_r[r] = yuv420p10_params();
    if (tune_cache_path && *tune_cache_path)
        tune_path = tune_cache_path;
    else if (const char* e = getenv("VSHIP_TUNE_CACHE"))
        tune_path = e;
    VSHIP_CUDA_TRY(cudaGetDevice(&device));
    cudaDeviceProp prop;
    VSHIP_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    sms = prop.multiProcessorCount;
    device_name = prop.name;
    VSHIP_CUDA_TRY(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&staging_free, cudaEventDisableTiming));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    for (int i = 0; i <= kMaxRes; i++) {
        VSHIP_CUDA_TRY(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
        VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_join[i], cudaEventDisableTiming));
    }

    if (flags & MULTI_SSIMU2) {
        int rc = ssimu2_multi_prepare();
        if (rc) return rc;
        for (int sh = 0; sh < 2; sh++) {
            rc = ssimu2_multi_stats_blocks_per_sm((flags & MULTI_FP16) != 0, sh, &stats_bps[sh]);
            if (rc) return rc;
            stats_bps[sh] = std::max(1, stats_bps[sh]);
        }
        knobs.shape = ssimu2_default_stats_shape();
        stats_blocks_per_sm = stats_bps[knobs.shape];
        knobs.grid_per_sm = stats_blocks_per_sm;
        const size_t cand_elem = (flags & MULTI_FP16) ? 2 : 4;
        for (int r = 0; r < nres; r++) {
            geoms_h[r] = make_ssimu2_geom(rw[r], rh[r]);
            const size_t pe = (size_t)geoms_h[r].plane_elems;
            if (max_src[r]) VSHIP_CUDA_TRY(vship_malloc((void**)&s_src[r], (size_t)max_src[r] * 3 * pe * 4));
            if (max_pairs[r]) {
                VSHIP_CUDA_TRY(vship_malloc((void**)&s_cand[r], (size_t)max_pairs[r] * 3 * pe * cand_elem));
                VSHIP_CUDA_TRY(vship_malloc((void**)&s_part[r], (size_t)max_pairs[r] * 18 * geoms_h[r].tiles_total * 4));
            }
            cap_pitems += ((size_t)max_src[r] + max_pairs[r]) * (size_t)ceil_div(rw[r], kPyrTile) * (size_t)ceil_div(rh[r], kPyrTile);
            cap_sitems += (size_t)max_pairs[r] * geoms_h[r].tiles_total;
        }
        VSHIP_CUDA_TRY(vship_malloc((void**)&geoms_d, sizeof(Ssimu2Geom) * nres));
        VSHIP_CUDA_TRY(cudaMemcpy(geoms_d, geoms_h, sizeof(Ssimu2Geom) * nres, cudaMemcpyHostToDevice));
        VSHIP_CUDA_TRY(vship_malloc((void**)&s_scores, sizeof(double) * pair_cap));
        VSHIP_CUDA_TRY(vship_malloc((void**)&s_imgs_d, sizeof(Ssimu2MultiImage) * (src_cap + pair_cap)));
        if (vship_malloc_host((void**)&s_imgs_h, sizeof(Ssimu2MultiImage) * (src_cap + pair_cap)) != cudaSuccess)
            return E_OUT_OF_RAM;
        VSHIP_CUDA_TRY(vship_malloc((void**)&s_pairs_d, sizeof(Ssimu2MultiPair) * pair_cap));
        VSHIP_CUDA_TRY(vship_malloc((void**)&s_pitems_d, sizeof(int4) * std::max<size_t>(cap_pitems, 1)));
        VSHIP_CUDA_TRY(vship_malloc((void**)&s_sitems_d, sizeof(int2) * std::max<size_t>(cap_sitems, 1)));
    }
    if (flags & MULTI_BUTTERAUGLI) {
        for (int r = 0; r < nres; r++) {
            if (!max_pairs[r]) continue;
            butter_caps(rw[r], rh[r], max_src[r], max_pairs[r], (flags & MULTI_BUTTER_HALF) != 0, &b_cap_img[r],
                        &b_cap_pair[r]);
            b_eng[r].half_bands = (flags & MULTI_BUTTER_HALF) != 0;
            int rc = b_eng[r].init_images(rw[r], rh[r], qnorm, intensity, b_cap_img[r], b_cap_pair[r], false);
            if (rc) return rc;
        }
        // a chunk image per pair plus its source at worst
        VSHIP_CUDA_TRY(vship_malloc((void**)&b_frames_d, sizeof(FrameDesc) * 2 * pair_cap));
        if (vship_malloc_host((void**)&b_frames_h, sizeof(FrameDesc) * 2 * pair_cap) != cudaSuccess)
            return E_OUT_OF_RAM;
        VSHIP_CUDA_TRY(vship_malloc((void**)&b_pimg_d, sizeof(int2) * pair_cap));
        VSHIP_CUDA_TRY(vship_malloc((void**)&b_norms_d, sizeof(double) * 3 * pair_cap * 2));
        VSHIP_CUDA_TRY(vship_malloc((void**)&b_perm_d, sizeof(int) * pair_cap));
    }
    return E_OK;
}

void MultiEngine::destroy() {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    for (int r = 0; r < kMaxRes; r++) {
        if (s_src[r]) cudaFree(s_src[r]);
        if (s_cand[r]) cudaFree(s_cand[r]);
        if (s_part[r]) cudaFree(s_part[r]);
        s_src[r] = nullptr;
        s_cand[r] = nullptr;
        s_part[r] = nullptr;
        b_eng[r].destroy();
    }
    if (geoms_d) cudaFree(geoms_d);
    if (s_scores) cudaFree(s_scores);
    if (s_imgs_d) cudaFree(s_imgs_d);
    if (s_imgs_h) cudaFreeHost(s_imgs_h);
    if (s_pairs_d) cudaFree(s_pairs_d);
    if (s_pitems_d) cudaFree(s_pitems_d);
    if (s_sitems_d) cudaFree(s_sitems_d);
    if (b_frames_d) cudaFree(b_frames_d);
    if (b_frames_h) cudaFreeHost(b_frames_h);
    if (b_pimg_d) cudaFree(b_pimg_d);
    if (b_norms_d) cudaFree(b_norms_d);
    if (b_perm_d) cudaFree(b_perm_d);
    geoms_d = nullptr;
    s_scores = nullptr;
    s_imgs_d = nullptr;
    s_imgs_h = nullptr;
    s_pairs_d = nullptr;
    s_pitems_d = nullptr;
    s_sitems_d = nullptr;
    b_frames_d = nullptr;
    b_frames_h = nullptr;
    b_pimg_d = nullptr;
    b_norms_d = nullptr;
    b_perm_d = nullptr;
    if (staging_free) cudaEventDestroy(staging_free);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (ev_fork) cudaEventDestroy(ev_fork);
    ev_fork = nullptr;
    for (int i = 0; i <= kMaxRes; i++) {
        if (side[i]) {
            cudaStreamSynchronize(side[i]);
            cudaStreamDestroy(side[i]);
        }
        if (ev_join[i]) cudaEventDestroy(ev_join[i]);
        side[i] = nullptr;
        ev_join[i] = nullptr;
    }
    staging_free = nullptr;
    cap_stream = nullptr;
}

// ------------------------------------------------------------------------------------------
// Layout: slots, pair table, pyramid items, Butteraugli grouping. Stats items follow the knobs.

int MultiEngine::build_plan(int nsrc, const int* src_res, int npairs, const int* cand_src, int intype,
                            cudaStream_t st) {
    int nsrc_r[kMaxRes] = {}, npair_r[kMaxRes] = {};
    src_slot.assign(nsrc, 0);
    cand_slot.assign(npairs, 0);
    for (int i = 0; i < nsrc; i++) {
        if (src_res[i] < 0 || src_res[i] >= nres) return E_BAD_POINTER;
        src_slot[i] = nsrc_r[src_res[i]]++;
    }
    for (int j = 0; j < npairs; j++) {
        if (cand_src[j] < 0 || cand_src[j] >= nsrc) return E_BAD_POINTER;
        const int r = src_res[cand_src[j]];
        cand_slot[j] = npair_r[r]++;
    }
    for (int r = 0; r < nres; r++) {
        if (flags & MULTI_SSIMU2) {
            if (nsrc_r[r] > max_src[r] || npair_r[r] > max_pairs[r]) return E_BAD_POINTER;
        } else if (npair_r[r] > max_pairs[r]) {
            return E_BAD_POINTER;
        }
    }
    plan_src_res.assign(src_res, src_res + nsrc);
    plan_cand_src.assign(cand_src, cand_src + npairs);
    plan_intype = intype;

    if (flags & MULTI_SSIMU2) {
        const bool fp16 = (flags & MULTI_FP16) != 0;
        std::vector<Ssimu2MultiPair> pairs(npairs);
        for (int j = 0; j < npairs; j++) {
            const int s = cand_src[j], r = src_res[s];
            const Ssimu2Geom& g = geoms_h[r];
            const size_t plane3 = (size_t)3 * g.plane_elems;
            Ssimu2MultiPair& P = pairs[j];
            P.geom = r;
            P.src = s_src[r] + src_slot[s] * plane3;
            P.cand = fp16 ? static_cast<const void*>(static_cast<__half*>(s_cand[r]) + cand_slot[j] * plane3)
                          : static_cast<const void*>(static_cast<float*>(s_cand[r]) + cand_slot[j] * plane3);
            P.partials = s_part[r] + (size_t)cand_slot[j] * 18 * g.tiles_total;
            P.score = s_scores + j;
        }
        std::vector<int4> pit;
        for (int i = 0; i < nsrc; i++) {
            const int r = src_res[i];
            const int tx = (int)ceil_div(rw[r], kPyrTile), ty = (int)ceil_div(rh[r], kPyrTile);
            for (int y = 0; y < ty; y++)
                for (int x = 0; x < tx; x++) pit.push_back(make_int4(i, x, y, 0));
        }
        n_pitems_src = (int)pit.size();
        for (int j = 0; j < npairs; j++) {
            const int r = src_res[cand_src[j]];
            const int tx = (int)ceil_div(rw[r], kPyrTile), ty = (int)ceil_div(rh[r], kPyrTile);
            for (int y = 0; y < ty; y++)
                for (int x = 0; x < tx; x++) pit.push_back(make_int4(nsrc + j, x, y, 0));
        }
        n_pitems_cand = (int)pit.size() - n_pitems_src;
        VSHIP_CUDA_TRY(cudaMemcpyAsync(s_pairs_d, pairs.data(), sizeof(Ssimu2MultiPair) * npairs,
                                       cudaMemcpyHostToDevice, st));
        VSHIP_CUDA_TRY(cudaMemcpyAsync(s_pitems_d, pit.data(), sizeof(int4) * pit.size(), cudaMemcpyHostToDevice, st));
    }
    if (flags & MULTI_BUTTERAUGLI) {
        // chunks of whole (source, candidates) groups, split only where one group alone exceeds
        // the resolution's workspace
        std::vector<std::vector<int>> by_src(nsrc);
        for (int j = 0; j < npairs; j++) by_src[cand_src[j]].push_back(j);
        std::vector<int> perm;
        std::vector<int2> pimg;
        b_chunks.clear();
        b_img_of.clear();
        for (int r = 0; r < nres; r++) {
            BChunk cur{r, (int)b_img_of.size(), 0, (int)perm.size(), 0};
            auto flush = [&]() {
                if (cur.npairs) b_chunks.push_back(cur);
                cur = BChunk{r, (int)b_img_of.size(), 0, (int)perm.size(), 0};
            };
            for (int s = 0; s < nsrc; s++) {
                if (src_res[s] != r) continue;
                int src_local = -1;
                for (size_t k = 0; k < by_src[s].size();) {
                    const int need = (src_local < 0 ? 1 : 0) + 1;
                    if (cur.nimg + need > b_cap_img[r] || cur.npairs + 1 > b_cap_pair[r]) {
                        flush();
                        src_local = -1;
                        continue;
                    }
                    if (src_local < 0) {
                        src_local = cur.nimg++;
                        b_img_of.push_back(s);
                    }
                    const int j = by_src[s][k++];
                    const int cand_local = cur.nimg++;
                    b_img_of.push_back(-1 - j);
                    pimg.push_back(make_int2(src_local, cand_local));
                    perm.push_back(j);
                    cur.npairs++;
                }
            }
            flush();
        }
        if ((int)b_img_of.size() > 2 * pair_cap) return E_BAD_POINTER;
        VSHIP_CUDA_TRY(cudaMemcpyAsync(b_pimg_d, pimg.data(), sizeof(int2) * pimg.size(), cudaMemcpyHostToDevice, st));
        VSHIP_CUDA_TRY(cudaMemcpyAsync(b_perm_d, perm.data(), sizeof(int) * npairs, cudaMemcpyHostToDevice, st));
    }
    plan_valid = true;
    return E_OK;
}

int MultiEngine::upload_items(cudaStream_t st) {
    if (!(flags & MULTI_SSIMU2)) return E_OK;
    const int nsrc = (int)plan_src_res.size(), npairs = (int)plan_cand_src.size();
    std::vector<int2> it;
    if (knobs.order == 0) {
        std::vector<std::vector<int>> by_src(nsrc);
        for (int j = 0; j < npairs; j++) by_src[plan_cand_src[j]].push_back(j);
        for (int s = 0; s < nsrc; s++) {
            const int tiles = geoms_h[plan_src_res[s]].tiles_total;
            for (int t = 0; t < tiles; t++)
                for (int j : by_src[s]) it.push_back(make_int2(j, t));
        }
    } else {
        for (int j = 0; j < npairs; j++) {
            const int tiles = geoms_h[plan_src_res[plan_cand_src[j]]].tiles_total;
            for (int t = 0; t < tiles; t++) it.push_back(make_int2(j, t));
        }
    }
    n_sitems = (int)it.size();
    VSHIP_CUDA_TRY(cudaMemcpyAsync(s_sitems_d, it.data(), sizeof(int2) * it.size(), cudaMemcpyHostToDevice, st));
    return E_OK;
}

void MultiEngine::fill_images(int nsrc, const FrameDesc* src, int npairs, const FrameDesc* cand) {
    if (flags & MULTI_SSIMU2) {
        const bool fp16 = (flags & MULTI_FP16) != 0;
        for (int i = 0; i < nsrc; i++) {
            const int r = plan_src_res[i];
            const size_t plane3 = (size_t)3 * geoms_h[r].plane_elems;
            Ssimu2MultiImage& I = s_imgs_h[i];
            I.geom = r;
            I.fd = src[i];
            I.yp = yuv_r[r];
            I.f32 = s_src[r] + src_slot[i] * plane3;
            I.d16 = nullptr;
            I.ref = nullptr;
        }
        for (int j = 0; j < npairs; j++) {
            const int s = plan_cand_src[j], r = plan_src_res[s];
            const size_t plane3 = (size_t)3 * geoms_h[r].plane_elems;
            Ssimu2MultiImage& I = s_imgs_h[nsrc + j];
            I.geom = r;
            I.fd = cand[j];
            I.yp = yuv_r[r];
            if (fp16) {
                I.f32 = nullptr;
                I.d16 = static_cast<__half*>(s_cand[r]) + cand_slot[j] * plane3;
                I.ref = s_src[r] + src_slot[s] * plane3;
            } else {
                I.f32 = static_cast<float*>(s_cand[r]) + cand_slot[j] * plane3;
                I.d16 = nullptr;
                I.ref = nullptr;
            }
        }
    }
    if (flags & MULTI_BUTTERAUGLI) {
        for (size_t k = 0; k < b_img_of.size(); k++) {
            const int f = b_img_of[k];
            b_frames_h[k] = f >= 0 ? src[f] : cand[-1 - f];
        }
    }
}

// The whole launch sequence of one batch (captured into the graph, or run directly).
int MultiEngine::enqueue(int npairs, cudaStream_t st) {
    // Fork: SSIMULACRA2 on one side stream, the Butteraugli chunks of each resolution on that
    // resolution's side stream (chunks of one resolution share its workspace, so they stay in
    // order), joined back into st. Kernels with different limits (the FMA-bound stats and diff
    // kernels, the memory-heavy vertical blurs) then fill each other's gaps.
    // With per-kernel timing on (Vship_ProfileSetEnabled), everything runs in order on st: CUDA
    // events bracketing a kernel then time that kernel alone, not whatever overlaps it on the
    // side streams. The timed (graph) runs keep the fork.
    const bool serial = prof_enabled();
    VSHIP_CUDA_TRY(cudaEventRecord(ev_fork, st));
    int rc = E_OK;
    int joins = 0;
    if (flags & MULTI_SSIMU2) {
        cudaStream_t s2 = serial ? st : side[kMaxRes];
        VSHIP_CUDA_TRY(cudaStreamWaitEvent(s2, ev_fork, 0));
        const bool fp16 = (flags & MULTI_FP16) != 0;
        rc = ssimu2_multi_pyramid(s_imgs_d, s_pitems_d, n_pitems_src, geoms_d, plan_intype, false, s2);
        if (!rc) rc = ssimu2_multi_pyramid(s_imgs_d, s_pitems_d + n_pitems_src, n_pitems_cand, geoms_d, plan_intype,
                                           fp16, s2);
        const int grid = knobs.grid_per_sm > 0 ? knobs.grid_per_sm * sms : n_sitems;
        if (!rc) rc = ssimu2_multi_stats(s_pairs_d, s_sitems_d, n_sitems, geoms_d, fp16, grid, knobs.shape, s2);
        if (!rc) rc = ssimu2_multi_finalize(s_pairs_d, npairs, geoms_d, s2);
        VSHIP_CUDA_TRY(cudaEventRecord(ev_join[kMaxRes], s2));
        VSHIP_CUDA_TRY(cudaStreamWaitEvent(st, ev_join[kMaxRes], 0));
        joins++;
        if (rc) return rc;
    }
    if (flags & MULTI_BUTTERAUGLI) {
        bool used[kMaxRes] = {};
        for (const BChunk& c : b_chunks) {
            cudaStream_t sr = serial ? st : side[c.res];
            if (!used[c.res]) {
                VSHIP_CUDA_TRY(cudaStreamWaitEvent(sr, ev_fork, 0));
                used[c.res] = true;
            }
            rc = b_eng[c.res].launch_images(b_frames_d + c.img_off, c.nimg, b_pimg_d + c.pair_off, c.npairs,
                                            plan_intype, b_norms_d + 3 * c.pair_off, nullptr, sr, &yuv_r[c.res]);
            if (rc) return rc;
        }
        for (int r = 0; r < nres; r++)
            if (used[r] && !serial) {
                VSHIP_CUDA_TRY(cudaEventRecord(ev_join[r], side[r]));
                VSHIP_CUDA_TRY(cudaStreamWaitEvent(st, ev_join[r], 0));
                joins++;
            }
        multi_scatter_norms_kernel<<<(unsigned)ceil_div(3 * npairs, 256), 256, 0, st>>>(
            b_norms_d, b_perm_d, b_norms_d + 3 * pair_cap, npairs);
        VSHIP_CUDA_TRY(cudaGetLastError());
    }
    (void)joins;
    return E_OK;
}

// ------------------------------------------------------------------------------------------
// Autotuner: time the SSIMU2 stats launch under every knob candidate on the batch at hand.

std::string MultiEngine::tune_key() const {
    std::ostringstream k;
    k << "ssimu2_multi_stats|" << device_name << "|sm" << sms << "|in" << plan_intype << "|"
      << ((flags & MULTI_FP16) ? "fp16" : "fp32");
    int nsrc_r[kMaxRes] = {}, npair_r[kMaxRes] = {};
    for (int r : plan_src_res) nsrc_r[r]++;
    for (int s : plan_cand_src) npair_r[plan_src_res[s]]++;
    for (int r = 0; r < nres; r++)
        if (npair_r[r]) k << "|" << rw[r] << "x" << rh[r] << ":" << nsrc_r[r] << ":" << npair_r[r];
    return k.str();
}

static std::map<std::string, std::string> read_tune_file(const std::string& path) {
    std::map<std::string, std::string> m;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t q0 = line.find('"');
        if (q0 == std::string::npos) continue;
        const size_t q1 = line.find('"', q0 + 1);
        const size_t b0 = line.find('{', q1 == std::string::npos ? 0 : q1);
        const size_t b1 = line.rfind('}');
        if (q1 == std::string::npos || b0 == std::string::npos || b1 == std::string::npos || b1 < b0) continue;
        m[line.substr(q0 + 1, q1 - q0 - 1)] = line.substr(b0, b1 - b0 + 1);
    }
    return m;
}

static int json_int(const std::string& obj, const char* name, int dflt) {
    const std::string pat = std::string("\"") + name + "\":";
    const size_t p = obj.find(pat);
    if (p == std::string::npos) return dflt;
    return atoi(obj.c_str() + p + pat.size());
}

bool MultiEngine::tune_lookup(const std::string& key, MultiKnobs* k) {
    if (tune_path.empty()) return false;
    const auto m = read_tune_file(tune_path);
    const auto it = m.find(key);
    if (it == m.end()) return false;
    // 0 means one CTA per work item; a corrupt or hand-edited entry is clamped to [0, occupancy]
    k->shape = json_int(it->second, "shape", k->shape) ? 1 : 0;
    k->grid_per_sm = std::max(0, std::min(json_int(it->second, "grid_per_sm", k->grid_per_sm), stats_bps[k->shape]));
    k->order = json_int(it->second, "order", k->order) ? 1 : 0;
    return true;
}

void MultiEngine::tune_store(const std::string& key, const MultiKnobs& k, double ms) {
    if (tune_path.empty()) return;
    auto m = read_tune_file(tune_path);
    char buf[160];
    snprintf(buf, sizeof(buf), "{\"grid_per_sm\":%d, \"order\":%d, \"shape\":%d, \"ms\":%.4f}", k.grid_per_sm,
             k.order, k.shape, ms);
    m[key] = buf;
    // a temporary file of this process's own, renamed over the cache: concurrent writers (ranks of
    // one job, other jobs sharing the file) never interleave their writes in one file
    const std::string tmp = tune_path + ".tmp." + std::to_string((long long)getpid()) + "." +
                            std::to_string((unsigned long long)std::hash<std::thread::id>{}(std::this_thread::get_id()));
    {
        std::ofstream f(tmp, std::ios::trunc);
        if (!f) return;
        f << "{\n";
        size_t i = 0;
        for (const auto& kv : m) f << "  \"" << kv.first << "\": " << kv.second << (++i < m.size() ? ",\n" : "\n");
        f << "}\n";
    }
    std::rename(tmp.c_str(), tune_path.c_str());
}

int MultiEngine::autotune(int npairs, cudaStream_t st) {
    const bool fp16 = (flags & MULTI_FP16) != 0;
    int rc = ssimu2_multi_pyramid(s_imgs_d, s_pitems_d, n_pitems_src, geoms_d, plan_intype, false, st);
    if (!rc) rc = ssimu2_multi_pyramid(s_imgs_d, s_pitems_d + n_pitems_src, n_pitems_cand, geoms_d, plan_intype,
                                       fp16, st);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    VSHIP_CUDA_TRY(cudaEventCreate(&e0));
    VSHIP_CUDA_TRY(cudaEventCreate(&e1));
    MultiKnobs best = knobs;
    double best_ms = 1e30;
    // every tile shape x work order x persistent grid (0 = one CTA per item)
    for (int order = 0; order < 2 && !rc; order++) {
        knobs.order = order;
        rc = upload_items(st);
        for (int shape = 0; shape < 2 && !rc; shape++)
        for (int gps = 0; gps <= stats_bps[shape] && !rc; gps++) {
            const int grid = gps > 0 ? gps * sms : n_sitems;
            double ms_min = 1e30;
            for (int rep = 0; rep < 4 && !rc; rep++) {
                cudaEventRecord(e0, st);
                rc = ssimu2_multi_stats(s_pairs_d, s_sitems_d, n_sitems, geoms_d, fp16, grid, shape, st);
                cudaEventRecord(e1, st);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = E_BAD_DEVICE_CODE;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) ms_min = std::min(ms_min, (double)ms);  // first run is a warm-up
            }
            if (!rc && ms_min < best_ms) {
                best_ms = ms_min;
                best.grid_per_sm = gps;
                best.order = order;
                best.shape = shape;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    (void)npairs;
    if (rc) return rc;
    knobs = best;
    stats_blocks_per_sm = stats_bps[knobs.shape];
    knobs_source = "tuned";
    tune_store(tune_key(), knobs, best_ms);
    return upload_items(st);
}

int MultiEngine::set_yuv_format(int bits, int ssw, int ssh, int matrix, int range, int loc, int transfer, int primaries) {
    YuvParams p[kMaxRes];
    for (int r = 0; r < nres; r++)
        if (!make_yuv_params(bits, ssw, ssh, matrix, range, loc, rh[r], &p[r], transfer, primaries))
            return E_BAD_POINTER;
    for (int r = 0; r < nres; r++) yuv_r[r] = p[r];
    if (gexec) {  // the Butteraugli launches carry the format as a kernel argument
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    return E_OK;
}

std::string MultiEngine::knobs_json() const {
    char buf[160];
    snprintf(buf, sizeof(buf), "{\"grid_per_sm\": %d, \"order\": %d, \"shape\": %d, \"source\": \"%s\"}",
             knobs.grid_per_sm, knobs.order, knobs.shape, knobs_source);
    return buf;
}

// ------------------------------------------------------------------------------------------

int MultiEngine::compute(int nsrc, const FrameDesc* src, const int* src_res, int npairs, const FrameDesc* cand,
                         const int* cand_src, int intype, double* ssimu2_dev, double* butter_dev, cudaStream_t st) {
    if (nsrc <= 0 || npairs <= 0 || !src || !src_res || !cand || !cand_src) return E_BAD_POINTER;
    if (nsrc > src_cap || npairs > pair_cap) return E_BAD_POINTER;
    if (intype < 0 || intype > IN_YUV) return E_BAD_POINTER;
    if ((flags & MULTI_SSIMU2) && !ssimu2_dev) return E_BAD_POINTER;
    if ((flags & MULTI_BUTTERAUGLI) && !butter_dev) return E_BAD_POINTER;

    const bool same = plan_valid && intype == plan_intype && (int)plan_src_res.size() == nsrc &&
                      (int)plan_cand_src.size() == npairs &&
                      std::equal(plan_src_res.begin(), plan_src_res.end(), src_res) &&
                      std::equal(plan_cand_src.begin(), plan_cand_src.end(), cand_src);
    // the previous call's table upload must have left the pinned staging before it is rewritten
    VSHIP_CUDA_TRY(cudaEventSynchronize(staging_free));
    bool tune_now = false;
    if (!same) {
        plan_valid = false;
        if (gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        int rc = build_plan(nsrc, src_res, npairs, cand_src, intype, st);
        if (rc) return rc;
        if (flags & MULTI_SSIMU2) {
            knobs = MultiKnobs{};
            knobs.shape = ssimu2_default_stats_shape();
            knobs.grid_per_sm = stats_bps[knobs.shape];
            knobs_source = "default";
            if (tune_lookup(tune_key(), &knobs))
                knobs_source = "cache";
            else if (flags & MULTI_AUTOTUNE)
                tune_now = true;
            stats_blocks_per_sm = stats_bps[knobs.shape];
            rc = upload_items(st);
            if (rc) return rc;
        }
    }
    fill_images(nsrc, src, npairs, cand);
    if (flags & MULTI_SSIMU2)
        VSHIP_CUDA_TRY(cudaMemcpyAsync(s_imgs_d, s_imgs_h, sizeof(Ssimu2MultiImage) * (nsrc + npairs),
                                       cudaMemcpyHostToDevice, st));
    if (flags & MULTI_BUTTERAUGLI)
        VSHIP_CUDA_TRY(cudaMemcpyAsync(b_frames_d, b_frames_h, sizeof(FrameDesc) * b_img_of.size(),
                                       cudaMemcpyHostToDevice, st));
    VSHIP_CUDA_TRY(cudaEventRecord(staging_free, st));
    if (tune_now) {
        int rc = autotune(npairs, st);
        if (rc) return rc;
    }

    const bool use_graph = !(flags & MULTI_NO_GRAPH) && !prof_enabled();
    if (use_graph) {
        if (!gexec) {
            VSHIP_CUDA_TRY(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue(npairs, cap_stream);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(cap_stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            VSHIP_CUDA_TRY(ce);
            const cudaError_t ie = cudaGraphInstantiate(&gexec, graph, 0);
            cudaGraphDestroy(graph);
            VSHIP_CUDA_TRY(ie);
        }
        VSHIP_CUDA_TRY(cudaGraphLaunch(gexec, st));
    } else {
        const int rc = enqueue(npairs, st);
        if (rc) return rc;
    }
    if (flags & MULTI_SSIMU2)
        VSHIP_CUDA_TRY(cudaMemcpyAsync(ssimu2_dev, s_scores, sizeof(double) * npairs, cudaMemcpyDeviceToDevice, st));
    if (flags & MULTI_BUTTERAUGLI)
        VSHIP_CUDA_TRY(cudaMemcpyAsync(butter_dev, b_norms_d + 3 * pair_cap, sizeof(double) * 3 * npairs,
                                       cudaMemcpyDeviceToDevice, st));
    return E_OK;
}

}  // namespace vship
