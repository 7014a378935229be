// serve.cu -- serving runtime (Server, serve.h).
//
// Device memory comes from a private stream-ordered pool on the server's stream: each batch
// takes one block for its candidates' planes, per-tile partial sums, tables and results and
// returns it (stream-ordered) right after its last kernel; cached source state is allocated per
// source and returned when the LRU cache drops it. Every batch's work runs on the one stream, so
// a batch that hits a source computed by an earlier batch still in flight reads it after it is
// written.
#include "serve.h"
#include "profile.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <sstream>

namespace vship {

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

int Server::create(int nres_, const int* widths, const int* heights, int intype_, uint64_t admission_bytes,
                   uint64_t cache_bytes, int max_batch_pairs_, int flags_, int qnorm_, float intensity_) {
    if (nres_ <= 0 || nres_ > kMaxRes || !widths || !heights) return E_BAD_POINTER;
    if (intype_ < 0 || intype_ > IN_YUV || max_batch_pairs_ <= 0 || admission_bytes == 0) return E_BAD_POINTER;
    nres = nres_;
    intype = intype_;
    flags = flags_;
    qnorm = qnorm_;
    intensity = intensity_;
    max_batch_pairs = max_batch_pairs_;
    adm = Admission(admission_bytes);
    cache = SourceCache<void*>(cache_bytes);
    for (int r = 0; r < nres; r++) {
        if (widths[r] <= 0 || heights[r] <= 0) return E_BAD_POINTER;
        rw[r] = widths[r];
        rh[r] = heights[r];
        sgeom[r] = make_ssimu2_geom(rw[r], rh[r]);
        bimg_floats[r] = butter_image_floats(rw[r], rh[r], (flags & SERVE_BUTTER_HALF_BANDS) != 0);
        bnorm_tiles[r] = butter_norm_tiles(rw[r], rh[r]);
        yuv_r[r] = yuv420p10_params();
    }
    VSHIP_CUDA_TRY(cudaGetDevice(&device));
    cudaDeviceProp prop;
    VSHIP_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    sms = prop.multiProcessorCount;
    int rc = ssimu2_multi_prepare();
    if (!rc) rc = butter_prepare_device();
    if (rc) return rc;
    int bps = 1;
    rc = ssimu2_multi_stats_blocks_per_sm(!(flags & SERVE_FP32_CANDIDATES), ssimu2_default_stats_shape(), &bps);
    if (rc) return rc;
    stats_grid = std::max(1, bps) * sms;
    VSHIP_CUDA_TRY(vship_malloc((void**)&sgeom_d, sizeof(Ssimu2Geom) * nres));
    VSHIP_CUDA_TRY(cudaMemcpy(sgeom_d, sgeom, sizeof(Ssimu2Geom) * nres, cudaMemcpyHostToDevice));
    VSHIP_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    VSHIP_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    VSHIP_CUDA_TRY(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;  // keep freed blocks for reuse instead of returning them to the driver
    VSHIP_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    sched_thr = std::thread(&Server::scheduler, this);
    done_thr = std::thread(&Server::completer, this);
    return E_OK;
}

void* Server::dev_alloc(size_t bytes) {
    void* p = nullptr;
    if (vship_alloc_injected_failure()) return nullptr;
    if (cudaMallocFromPoolAsync(&p, bytes, pool, st) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

int Server::submit(ServeReq* r) {
    if (!r || r->metric < SERVE_SSIMU2 || r->metric > SERVE_BUTTERAUGLI || r->res < 0 || r->res >= nres ||
        r->cands.empty() || (int)r->cands.size() > max_batch_pairs || !r->out) {
        delete r;
        return E_BAD_POINTER;
    }
    r->charge = serve_charge_per_pair(r->metric, rw[r->res], rh[r->res]) * r->cands.size();
    if (!adm.fits_alone(r->charge)) {
        delete r;
        return E_OUT_OF_VRAM;
    }
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> g(mu);
        if (stop) {
            delete r;
            return E_BAD_HANDLER;
        }
        queue.push_back(r);
        n_submitted++;
    }
    cv.notify_all();
    return E_OK;
}

int Server::set_yuv_format(int bits, int ssw, int ssh, int matrix, int range, int loc, int transfer, int primaries) {
    YuvParams p[kMaxRes];
    for (int r = 0; r < nres; r++)
        if (!make_yuv_params(bits, ssw, ssh, matrix, range, loc, rh[r], &p[r], transfer, primaries))
            return E_BAD_POINTER;
    std::lock_guard<std::mutex> g(mu);
    // The source cache is keyed by (metric, resolution, source key), not by format: state decoded
    // under one format must never be scored against candidates of another, so the format is
    // fixed once the first request has been submitted.
    if (n_submitted > 0) return E_BAD_POINTER;
    for (int r = 0; r < nres; r++) yuv_r[r] = p[r];
    return E_OK;
}

int Server::cancel(uint64_t id) {
    ServeReq* r = nullptr;
    {
        std::lock_guard<std::mutex> g(mu);
        for (auto it = queue.begin(); it != queue.end(); ++it)
            if ((*it)->id == id) {
                r = *it;
                queue.erase(it);
                break;
            }
        if (!r) return E_BAD_POINTER;
        done.push_back(ServeDone{r->id, kCancelled, now_s() - r->t_submit});
        n_completed++;
        n_cancelled++;
    }
    delete r;
    cv.notify_all();
    return E_OK;
}

int Server::poll(ServeDone* out, int max, double timeout_s) {
    std::unique_lock<std::mutex> lk(mu);
    if (done.empty() && timeout_s > 0)
        cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !done.empty() || stop; });
    int n = 0;
    while (n < max && !done.empty()) {
        out[n++] = done.front();
        done.pop_front();
    }
    return n;
}

int Server::drain() {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return (queue.empty() && inflight.empty() && n_completed == n_submitted) || stop; });
    return E_OK;
}

void Server::scheduler() {
    cudaSetDevice(device);
    for (;;) {
        Batch* b = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return stop || (!queue.empty() && (int)inflight.size() < kMaxInflight); });
            if (stop) return;
            std::vector<ServeReq*> reqs = form_batch(
                queue, adm, max_batch_pairs, [](ServeReq* r) { return r->charge; },
                [](ServeReq* r) { return (int)r->cands.size(); });
            if (reqs.empty()) {
                // the oldest request waits for budget held by batches in flight
                n_admission_waits++;
                cv.wait(lk, [&] { return stop || inflight.empty() || adm.used() + queue.front()->charge <= adm.budget(); });
                continue;
            }
            b = new Batch();
            b->reqs = std::move(reqs);
            for (ServeReq* r : b->reqs) b->charge += r->charge;
        }
        b->status = launch(b);
        {
            std::lock_guard<std::mutex> g(mu);
            inflight.push_back(b);
            n_batches++;
            int np = 0;
            for (ServeReq* r : b->reqs) np += (int)r->cands.size();
            n_pairs += np;
            max_batch_seen = std::max(max_batch_seen, np);
        }
        cv.notify_all();
    }
}

void Server::completer() {
    cudaSetDevice(device);
    for (;;) {
        Batch* b = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return !inflight.empty() || stop; });
            if (inflight.empty()) return;
            b = inflight.front();
        }
        int status = b->status;
        if (!b->done || cudaEventSynchronize(b->done) != cudaSuccess)
            if (status == E_OK) status = E_BAD_DEVICE_CODE;
        const double t = now_s();
        const double* res = reinterpret_cast<const double*>(b->host + b->res_off);
        std::vector<ServeDone> fin;
        for (size_t i = 0; i < b->reqs.size(); i++) {
            ServeReq* r = b->reqs[i];
            const size_t n = r->cands.size() * (r->metric == SERVE_SSIMU2 ? 1 : 3);
            if (status == E_OK) std::memcpy(r->out, res + b->out_off[i], n * sizeof(double));
            fin.push_back(ServeDone{r->id, status, t - r->t_submit});
        }
        if (status != E_OK) n_failed += b->reqs.size();
        if (b->done) cudaEventDestroy(b->done);
        {
            std::lock_guard<std::mutex> g(mu);
            adm.release(b->charge);
            for (const SourceKey& k : b->pinned) cache.unpin(k);
            for (const ServeDone& d : fin) done.push_back(d);
            n_completed += fin.size();
            if (b->host) host_pool.emplace_back(b->host, b->host_cap);
            inflight.pop_front();
        }
        for (ServeReq* r : b->reqs) delete r;
        delete b;
        cv.notify_all();
    }
}

// ------------------------------------------------------------------------------------------
// One batch: resolve sources through the cache, lay out one device block, fill the tables in
// pinned staging, enqueue the SSIMULACRA2 work-list launches and the Butteraugli launches (one
// sequence per resolution), copy the results back, return the block, record the event.

// A batch that failed: the state of sources it inserted never became valid (drop them), the
// ones it found in the cache are released.
void Server::release_sources(Batch* b, const std::vector<SourceKey>& inserted) {
    std::lock_guard<std::mutex> g(mu);
    for (const SourceKey& k : b->pinned) {
        if (std::find(inserted.begin(), inserted.end(), k) != inserted.end()) {
            void* p = nullptr;
            if (cache.erase(k, &p)) cudaFreeAsync(p, st);
        } else {
            cache.unpin(k);
        }
    }
    b->pinned.clear();
}

int Server::launch(Batch* b) {
    VSHIP_CUDA_TRY(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    const bool fp16 = !(flags & SERVE_FP32_CANDIDATES);
    const int nreq = (int)b->reqs.size();
    std::vector<float*> src(nreq, nullptr);
    std::vector<char> stage(nreq, 0);
    std::vector<void*> temp, evicted;
    std::vector<SourceKey> inserted;
    YuvParams yuv[kMaxRes];
    int rc = E_OK;
    {
        std::lock_guard<std::mutex> g(mu);
        for (int r = 0; r < nres; r++) yuv[r] = yuv_r[r];
        for (int i = 0; i < nreq && !rc; i++) {
            ServeReq* r = b->reqs[i];
            const size_t bytes = r->metric == SERVE_SSIMU2 ? sizeof(float) * 3 * (size_t)sgeom[r->res].plane_elems
                                                          : sizeof(float) * bimg_floats[r->res];
            const SourceKey k{r->metric, r->res, r->key};
            void* p = nullptr;
            if (r->key && cache.acquire(k, &p)) {
                b->pinned.push_back(k);
            } else {
                p = dev_alloc(bytes);
                if (!p) {
                    rc = E_OUT_OF_VRAM;
                    break;
                }
                stage[i] = 1;
                if (r->key && cache.insert(k, p, bytes, &evicted)) {
                    b->pinned.push_back(k);
                    inserted.push_back(k);
                } else {
                    temp.push_back(p);
                    n_uncached_sources++;
                }
            }
            src[i] = static_cast<float*>(p);
        }
    }
    for (void* e : evicted) cudaFreeAsync(e, st);

    // --- layout: data block (candidates, partials), tables, results
    size_t dcur = 0, tcur = 0;
    auto dtake = [&](size_t n) { const size_t o = align256(dcur); dcur = o + n; return o; };
    auto ttake = [&](size_t n) { const size_t o = align256(tcur); tcur = o + n; return o; };
    const size_t celem = fp16 ? 2 : 4;
    int np_s2 = 0, np_b = 0, nstage_s2 = 0;
    std::vector<size_t> cand_off(nreq), part_off(nreq);
    for (int i = 0; i < nreq; i++) {
        ServeReq* r = b->reqs[i];
        const size_t n = r->cands.size();
        if (r->metric == SERVE_SSIMU2) {
            const Ssimu2Geom& G = sgeom[r->res];
            cand_off[i] = dtake(n * 3 * (size_t)G.plane_elems * celem);
            part_off[i] = dtake(n * 18 * (size_t)G.tiles_total * 4);
            np_s2 += (int)n;
            nstage_s2 += stage[i];
        } else {
            cand_off[i] = dtake(n * bimg_floats[r->res] * 4);
            np_b += (int)n;
        }
    }
    // SSIMU2 tables
    size_t n_pitems_src = 0, n_pitems_cand = 0, n_sitems = 0;
    for (int i = 0; i < nreq; i++) {
        ServeReq* r = b->reqs[i];
        if (r->metric != SERVE_SSIMU2) continue;
        const size_t t0 = (size_t)ceil_div(rw[r->res], kPyrTile) * (size_t)ceil_div(rh[r->res], kPyrTile);
        if (stage[i]) n_pitems_src += t0;
        n_pitems_cand += t0 * r->cands.size();
        n_sitems += (size_t)sgeom[r->res].tiles_total * r->cands.size();
    }
    const size_t t_imgs = ttake(sizeof(Ssimu2MultiImage) * (nstage_s2 + np_s2));
    const size_t t_pit = ttake(sizeof(int4) * (n_pitems_src + n_pitems_cand));
    const size_t t_pairs = ttake(sizeof(Ssimu2MultiPair) * np_s2);
    const size_t t_sit = ttake(sizeof(int2) * n_sitems);
    // Butteraugli tables, one group per resolution
    struct BGroup {
        int res = 0, nstage = 0, ncached = 0, npairs = 0;
        size_t t_ib = 0, t_fr = 0, t_pi = 0, part = 0;
        std::vector<int> reqs;
    };
    std::vector<BGroup> bg;
    for (int r = 0; r < nres; r++) {
        BGroup G;
        G.res = r;
        for (int i = 0; i < nreq; i++) {
            ServeReq* q = b->reqs[i];
            if (q->metric != SERVE_BUTTERAUGLI || q->res != r) continue;
            G.reqs.push_back(i);
            G.npairs += (int)q->cands.size();
            if (stage[i])
                G.nstage++;
            else
                G.ncached++;
        }
        if (!G.npairs) continue;
        G.nstage += G.npairs;  // every candidate runs its own stage
        G.part = dtake((size_t)G.npairs * 3 * bnorm_tiles[r] * 4);
        G.t_ib = ttake(sizeof(float*) * (G.nstage + G.ncached));
        G.t_fr = ttake(sizeof(FrameDesc) * G.nstage);
        G.t_pi = ttake(sizeof(int2) * G.npairs);
        bg.push_back(std::move(G));
    }
    const size_t tab_bytes = align256(tcur);
    const size_t res_doubles = (size_t)np_s2 + 3 * (size_t)np_b;
    const size_t data_bytes = align256(dcur);
    const size_t block_bytes = data_bytes + tab_bytes + res_doubles * sizeof(double);

    // pinned staging: tables, then results
    const size_t host_need = tab_bytes + res_doubles * sizeof(double);
    {
        std::lock_guard<std::mutex> g(mu);
        for (size_t k = 0; k < host_pool.size(); k++)
            if (host_pool[k].second >= host_need) {
                b->host = host_pool[k].first;
                b->host_cap = host_pool[k].second;
                host_pool.erase(host_pool.begin() + k);
                break;
            }
    }
    if (!b->host) {
        b->host_cap = std::max<size_t>(host_need, 1 << 20);
        if (vship_malloc_host((void**)&b->host, b->host_cap) != cudaSuccess) {
            cudaGetLastError();
            b->host = nullptr;
            b->host_cap = 0;
            rc = rc ? rc : E_OUT_OF_RAM;
        }
    }
    b->res_off = tab_bytes;
    b->nres_doubles = res_doubles;
    uint8_t* block = nullptr;
    if (!rc) {
        block = static_cast<uint8_t*>(dev_alloc(block_bytes));
        if (!block) rc = E_OUT_OF_VRAM;
    }
    if (rc) {
        release_sources(b, inserted);
        for (void* p : temp) cudaFreeAsync(p, st);
        cudaEventRecord(b->done, st);
        return rc;
    }
    uint8_t* dtab = block + data_bytes;
    double* dres = reinterpret_cast<double*>(dtab + tab_bytes);
    uint8_t* h = b->host;

    // --- fill tables
    b->out_off.assign(nreq, 0);
    {
        auto* imgs = reinterpret_cast<Ssimu2MultiImage*>(h + t_imgs);
        auto* pit = reinterpret_cast<int4*>(h + t_pit);
        auto* pairs = reinterpret_cast<Ssimu2MultiPair*>(h + t_pairs);
        auto* sit = reinterpret_cast<int2*>(h + t_sit);
        int ni = 0, npair = 0;
        size_t ps = 0, pc = n_pitems_src, si = 0, ro = 0;
        auto add_tiles = [&](int img, int res, size_t& cursor) {
            const int tx = (int)ceil_div(rw[res], kPyrTile), ty = (int)ceil_div(rh[res], kPyrTile);
            for (int y = 0; y < ty; y++)
                for (int x = 0; x < tx; x++) pit[cursor++] = make_int4(img, x, y, 0);
        };
        for (int i = 0; i < nreq; i++) {  // sources whose pyramid this batch builds
            ServeReq* r = b->reqs[i];
            if (r->metric != SERVE_SSIMU2 || !stage[i]) continue;
            imgs[ni] = Ssimu2MultiImage{r->res, r->src, yuv[r->res], src[i], nullptr, nullptr};
            add_tiles(ni, r->res, ps);
            ni++;
        }
        for (int i = 0; i < nreq; i++) {
            ServeReq* r = b->reqs[i];
            if (r->metric != SERVE_SSIMU2) continue;
            const Ssimu2Geom& G = sgeom[r->res];
            const size_t plane3 = (size_t)3 * G.plane_elems;
            b->out_off[i] = ro;
            for (size_t c = 0; c < r->cands.size(); c++) {
                uint8_t* cp = block + cand_off[i] + c * plane3 * celem;
                float* part = reinterpret_cast<float*>(block + part_off[i]) + c * 18 * (size_t)G.tiles_total;
                imgs[ni] = fp16 ? Ssimu2MultiImage{r->res, r->cands[c], yuv[r->res], nullptr, cp, src[i]}
                                : Ssimu2MultiImage{r->res, r->cands[c], yuv[r->res], reinterpret_cast<float*>(cp),
                                                   nullptr, nullptr};
                add_tiles(ni, r->res, pc);
                ni++;
                pairs[npair] = Ssimu2MultiPair{r->res, src[i], cp, part, dres + ro};
                for (int t = 0; t < G.tiles_total; t++) sit[si++] = make_int2(npair, t);
                npair++;
                ro++;
            }
        }
        for (BGroup& G : bg) {
            auto* ib = reinterpret_cast<float**>(h + G.t_ib);
            auto* fr = reinterpret_cast<FrameDesc*>(h + G.t_fr);
            auto* pi = reinterpret_cast<int2*>(h + G.t_pi);
            int k = 0;
            std::vector<int> src_idx(nreq, -1);
            for (int i : G.reqs)  // new sources first: they run their own stage
                if (stage[i]) {
                    src_idx[i] = k;
                    fr[k] = b->reqs[i]->src;
                    ib[k++] = src[i];
                }
            const size_t img_bytes = bimg_floats[G.res] * 4;
            const size_t cand_first = k;
            for (int i : G.reqs) {
                ServeReq* r = b->reqs[i];
                for (size_t c = 0; c < r->cands.size(); c++) {
                    fr[k] = r->cands[c];
                    ib[k++] = reinterpret_cast<float*>(block + cand_off[i] + c * img_bytes);
                }
            }
            for (int i : G.reqs)  // cached sources: pair stage only
                if (!stage[i]) {
                    src_idx[i] = k;
                    ib[k++] = src[i];
                }
            size_t ci = cand_first;
            int p = 0;
            for (int i : G.reqs) {
                ServeReq* r = b->reqs[i];
                b->out_off[i] = ro;
                for (size_t c = 0; c < r->cands.size(); c++) {
                    pi[p++] = make_int2(src_idx[i], (int)ci++);
                    ro += 3;
                }
            }
        }
    }

    // --- enqueue
    rc = E_OK;
    if (cudaMemcpyAsync(dtab, h, tab_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = E_BAD_DEVICE_CODE;
    if (!rc && np_s2) {
        auto* imgs = reinterpret_cast<const Ssimu2MultiImage*>(dtab + t_imgs);
        auto* pit = reinterpret_cast<const int4*>(dtab + t_pit);
        auto* pairs = reinterpret_cast<const Ssimu2MultiPair*>(dtab + t_pairs);
        auto* sit = reinterpret_cast<const int2*>(dtab + t_sit);
        rc = ssimu2_multi_pyramid(imgs, pit, (int)n_pitems_src, sgeom_d, intype, false, st);
        if (!rc) rc = ssimu2_multi_pyramid(imgs, pit + n_pitems_src, (int)n_pitems_cand, sgeom_d, intype, fp16, st);
        if (!rc) rc = ssimu2_multi_stats(pairs, sit, (int)n_sitems, sgeom_d, fp16, stats_grid, ssimu2_default_stats_shape(), st);
        if (!rc) rc = ssimu2_multi_finalize(pairs, np_s2, sgeom_d, st);
    }
    for (const BGroup& G : bg) {
        if (rc) break;
        rc = butter_enqueue(rw[G.res], rh[G.res], qnorm, intensity, reinterpret_cast<float* const*>(dtab + G.t_ib),
                            reinterpret_cast<const FrameDesc*>(dtab + G.t_fr), G.nstage,
                            reinterpret_cast<const int2*>(dtab + G.t_pi), G.npairs, intype,
                            reinterpret_cast<float*>(block + G.part), dres + b->out_off[G.reqs[0]], nullptr, st,
                            &yuv[G.res], (flags & SERVE_BUTTER_HALF_BANDS) != 0, side, ev_fork, ev_join);
    }
    if (!rc && cudaMemcpyAsync(h + b->res_off, dres, res_doubles * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                   cudaSuccess)
        rc = E_BAD_DEVICE_CODE;
    cudaFreeAsync(block, st);
    for (void* p : temp) cudaFreeAsync(p, st);
    if (rc) release_sources(b, inserted);
    if (cudaEventRecord(b->done, st) != cudaSuccess && !rc) rc = E_BAD_DEVICE_CODE;
    return rc;
}

std::string Server::stats_json() {
    std::lock_guard<std::mutex> g(mu);
    std::ostringstream o;
    o << "{\"submitted\": " << n_submitted << ", \"completed\": " << n_completed << ", \"batches\": " << n_batches
      << ", \"pairs\": " << n_pairs << ", \"max_batch_pairs\": " << max_batch_seen
      << ", \"admission_waits\": " << n_admission_waits << ", \"admission_peak_bytes\": " << adm.peak()
      << ", \"admission_budget_bytes\": " << adm.budget() << ", \"cache_hits\": " << cache.hits()
      << ", \"cache_misses\": " << cache.misses() << ", \"cache_evictions\": " << cache.evictions()
      << ", \"cache_entries\": " << cache.size() << ", \"cache_bytes\": " << cache.bytes()
      << ", \"uncached_sources\": " << n_uncached_sources << ", \"cancelled\": " << n_cancelled
      << ", \"failed\": " << n_failed << ", \"queued\": " << queue.size()
      << ", \"inflight\": " << inflight.size() << "}";
    return o.str();
}

void Server::destroy() {
    if (sched_thr.joinable()) {
        drain();
        {
            std::lock_guard<std::mutex> g(mu);
            stop = true;
        }
        cv.notify_all();
        sched_thr.join();
        done_thr.join();
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(device);
    if (st) {
        std::vector<void*> left;
        cache.clear(&left);
        for (void* p : left) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
    }
    for (ServeReq* r : queue) delete r;
    queue.clear();
    for (auto& hp : host_pool) cudaFreeHost(hp.first);
    host_pool.clear();
    if (pool) cudaMemPoolDestroy(pool);
    if (sgeom_d) cudaFree(sgeom_d);
    if (st) cudaStreamDestroy(st);
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    pool = nullptr;
    sgeom_d = nullptr;
    st = side = nullptr;
    ev_fork = ev_join = nullptr;
    cudaSetDevice(dev);
}

}  // namespace vship
