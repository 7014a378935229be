// serve.h -- serving runtime: a request queue feeding continuous batches of SSIMULACRA2 and
// Butteraugli pairs onto one GPU stream, with memory admission and an LRU cache of per-source
// device state (SSIMULACRA2 XYB pyramids, Butteraugli opsin / frequency-band planes).
//
// Threads: the caller submits and polls; a scheduler thread forms a batch whenever fewer than
// kMaxInflight batches are on the GPU (requests join the next batch as soon as admission
// budget frees up) and enqueues it; a completion thread waits for each batch in order, copies
// the results to the requests' host buffers and reports completions with their latency.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "butter.h"
#include "common.cuh"
#include "serve_policy.h"
#include "ssimu2.h"

namespace vship {

enum : int {
    SERVE_FP32_CANDIDATES = 1,   // keep SSIMULACRA2 candidate pyramids in FP32
    SERVE_BUTTER_HALF_BANDS = 2  // Butteraugli UHF bands as FP16 (ButterEngine::half_bands)
};

struct ServeReq {
    uint64_t id = 0;
    int metric = SERVE_SSIMU2;
    int res = 0;
    uint64_t key = 0;  // source identity for the cache; 0 = never cached
    FrameDesc src{};
    std::vector<FrameDesc> cands;
    double* out = nullptr;  // host: npairs scores, or 3 x npairs norms
    uint64_t charge = 0;
    double t_submit = 0.0;
};

struct ServeDone {
    uint64_t id;
    int status;
    double latency;  // seconds from submit to results in the host buffer
};

class Server {
public:
    static constexpr int kMaxRes = 8;
    static constexpr int kMaxInflight = 2;
    int device = 0;

    int create(int nres, const int* widths, const int* heights, int intype, uint64_t admission_bytes,
               uint64_t cache_bytes, int max_batch_pairs, int flags, int qnorm, float intensity);
    int submit(ServeReq* r);  // takes ownership (deleted after completion)
    // Withdraws a request that is still queued (not yet in a batch): it completes at once with
    // status kCancelled. E_BAD_POINTER when no queued request has this id.
    int cancel(uint64_t id);
    static constexpr int kCancelled = -1;
    int poll(ServeDone* out, int max, double timeout_s);
    // Format of IN_YUV frames for every resolution (make_yuv_params; matrix 2 resolves per height).
    int set_yuv_format(int bits, int ssw, int ssh, int matrix, int range, int loc, int transfer = 1,
                       int primaries = 1);
    int drain();
    std::string stats_json();
    void destroy();

private:
    struct Batch {
        std::vector<ServeReq*> reqs;
        std::vector<SourceKey> pinned;
        std::vector<size_t> out_off;  // per request: first result (doubles) in the result block
        uint8_t* host = nullptr;      // pinned: tables (in), results (out)
        size_t host_cap = 0, res_off = 0, nres_doubles = 0;
        cudaEvent_t done = nullptr;
        uint64_t charge = 0;
        int status = E_OK;
    };

    int nres = 0, intype = IN_YUV, flags = 0, qnorm = 2, max_batch_pairs = 256, sms = 0, stats_grid = 0;
    float intensity = 203.f;
    int64_t rw[kMaxRes]{}, rh[kMaxRes]{};
    Ssimu2Geom sgeom[kMaxRes]{};
    Ssimu2Geom* sgeom_d = nullptr;
    size_t bimg_floats[kMaxRes]{};
    YuvParams yuv_r[kMaxRes];
    int bnorm_tiles[kMaxRes]{};

    cudaStream_t st = nullptr;
    // Butteraugli's half-scale chain runs on `side` beside the full scale's (butter_enqueue)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaMemPool_t pool = nullptr;
    Admission adm;
    SourceCache<void*> cache;

    std::mutex mu;
    std::condition_variable cv;  // any state change: queue, in-flight, done, stop
    std::deque<ServeReq*> queue;
    std::deque<Batch*> inflight;
    std::deque<ServeDone> done;
    std::vector<std::pair<uint8_t*, size_t>> host_pool;  // free pinned staging buffers
    bool stop = false;
    std::thread sched_thr, done_thr;

    // counters
    uint64_t n_submitted = 0, n_completed = 0, n_batches = 0, n_pairs = 0, n_admission_waits = 0;
    uint64_t n_uncached_sources = 0, n_cancelled = 0, n_failed = 0;
    int max_batch_seen = 0;

    void scheduler();
    void completer();
    int launch(Batch* b);
    void release_sources(Batch* b, const std::vector<SourceKey>& inserted);
    void* dev_alloc(size_t bytes);
};

}  // namespace vship
