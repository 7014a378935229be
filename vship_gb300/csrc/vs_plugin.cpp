// vs_plugin.cpp -- VapourSynth plugin entry of libvship.so: vship.SSIMULACRA2, vship.BUTTERAUGLI,
// vship.GpuInfo with the reference plugin's id, namespace, argument lists, defaults, errors and
// frame properties (src/VshipLib.cpp:8-64, src/ssimu2/vapoursynth.hpp, src/butter/vapoursynth.hpp).
//
// Compiled only when the VapourSynth SDK headers (VapourSynth4.h, VSHelper4.h) are available;
// the filters call the library's own C ABI, so scores are those of the C-ABI tests.
#include <VSHelper4.h>
#include <VapourSynth4.h>

#include "../../include/VshipAPI.h"

#include <algorithm>
#include <condition_variable>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace {

std::string vship_error(Vship_Exception e) {
    // same layout as the reference's VshipError::getErrorMessage (src/util/VshipExceptions.hpp:97-104)
    const int n = Vship_GetErrorMessage(e, nullptr, 0);
    std::string m(n, '\0');
    Vship_GetErrorMessage(e, &m[0], n);
    m.resize(n - 1);
    return "VshipException\n" + m + "\n";
}

// The reference converts any non-RGBS clip with resize.Bicubic (src/util/torgbs.hpp): BT.709
// transfer and primaries, limited range in, full range out, matrix BT.709 above 650 rows and
// BT.601 (170M) otherwise.
VSNode* to_rgbs(VSNode* node, VSCore* core, const VSAPI* api) {
    const VSVideoInfo* vi = api->getVideoInfo(node);
    if (vi->format.colorFamily == cfRGB && vi->format.sampleType == stFloat && vi->format.bitsPerSample == 32)
        return node;
    VSMap* args = api->createMap();
    api->mapConsumeNode(args, "clip", node, maReplace);
    api->mapSetInt(args, "matrix_in", vi->height > 650 ? 1 : 6, maReplace);
    api->mapSetInt(args, "transfer_in", 1, maReplace);
    api->mapSetInt(args, "primaries_in", 1, maReplace);
    api->mapSetInt(args, "range_in", 0, maReplace);
    api->mapSetInt(args, "matrix", 0, maReplace);
    api->mapSetInt(args, "transfer", 1, maReplace);
    api->mapSetInt(args, "primaries", 1, maReplace);
    api->mapSetInt(args, "range", 1, maReplace);
    api->mapSetInt(args, "format", pfRGBS, maReplace);
    VSMap* ret = api->invoke(api->getPluginByID(VSH_RESIZE_PLUGIN_ID, core), "Bicubic", args);
    VSNode* out = api->mapGetNode(ret, "clip", 0, nullptr);
    api->freeMap(ret);
    api->freeMap(args);
    return out;
}

enum class Metric { SSIMU2, Butteraugli };

struct Filter {
    Metric metric;
    VSNode* ref = nullptr;
    VSNode* dist = nullptr;
    bool distmap = false;
    std::vector<int> handlers;  // handler ids, one per stream
    std::vector<int> idle;      // indices into handlers
    std::mutex mu;
    std::condition_variable cv;

    int acquire() {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return !idle.empty(); });
        const int k = idle.back();
        idle.pop_back();
        return k;
    }
    void release(int k) {
        {
            std::lock_guard<std::mutex> lk(mu);
            idle.push_back(k);
        }
        cv.notify_one();
    }
};

const VSFrame* VS_CC get_frame(int n, int reason, void* inst, void**, VSFrameContext* ctx, VSCore* core,
                               const VSAPI* api) {
    Filter* d = static_cast<Filter*>(inst);
    if (reason == arInitial) {
        api->requestFrameFilter(n, d->ref, ctx);
        api->requestFrameFilter(n, d->dist, ctx);
        return nullptr;
    }
    if (reason != arAllFramesReady) return nullptr;
    const VSFrame* a = api->getFrameFilter(n, d->ref, ctx);
    const VSFrame* b = api->getFrameFilter(n, d->dist, ctx);
    const int w = api->getFrameWidth(a, 0), h = api->getFrameHeight(a, 0);
    const uint8_t* pa[3] = {api->getReadPtr(a, 0), api->getReadPtr(a, 1), api->getReadPtr(a, 2)};
    const uint8_t* pb[3] = {api->getReadPtr(b, 0), api->getReadPtr(b, 1), api->getReadPtr(b, 2)};
    VSFrame* dst;
    if (d->distmap) {
        VSVideoFormat gray;
        api->queryVideoFormat(&gray, cfGray, stFloat, 32, 0, 0, core);
        dst = api->newVideoFrame(&gray, w, h, nullptr, core);
    } else {
        dst = api->copyFrame(b, core);
    }
    const int k = d->acquire();
    Vship_Exception e;
    VSMap* props = api->getFramePropertiesRW(dst);
    if (d->metric == Metric::SSIMU2) {
        double s = 0;
        e = Vship_ComputeSSIMU2Floatv2(Vship_SSIMU2Handler{d->handlers[k]}, &s, pa, pb, api->getStride(a, 0),
                                       api->getStride(b, 0));
        if (e == Vship_NoError) api->mapSetFloat(props, "_SSIMULACRA2", s, maReplace);
    } else {
        double v[3] = {0, 0, 0};
        e = Vship_ComputeButteraugliFloatv3(Vship_ButteraugliHandler{d->handlers[k]}, v,
                                            d->distmap ? api->getWritePtr(dst, 0) : nullptr,
                                            d->distmap ? api->getStride(dst, 0) : 0, pa, pb, api->getStride(a, 0),
                                            api->getStride(b, 0));
        if (e == Vship_NoError) {
            api->mapSetFloat(props, "_BUTTERAUGLI_QNorm", v[0], maReplace);
            api->mapSetFloat(props, "_BUTTERAUGLI_3Norm", v[1], maReplace);
            api->mapSetFloat(props, "_BUTTERAUGLI_INFNorm", v[2], maReplace);
            // documented (doc/BUTTERAUGLI.md) but never set by the reference: the Q-norm, i.e. the
            // 2-norm for the default qnorm = 2
            api->mapSetFloat(props, "_BUTTERAUGLI_2Norm", v[0], maReplace);
        }
    }
    d->release(k);
    api->freeFrame(a);
    api->freeFrame(b);
    if (e != Vship_NoError) {
        api->setFilterError(vship_error(e).c_str(), ctx);
        api->freeFrame(dst);
        return nullptr;
    }
    return dst;
}

void VS_CC free_filter(void* inst, VSCore*, const VSAPI* api) {
    Filter* d = static_cast<Filter*>(inst);
    api->freeNode(d->ref);
    api->freeNode(d->dist);
    for (int id : d->handlers) {
        if (d->metric == Metric::SSIMU2) Vship_SSIMU2Free(Vship_SSIMU2Handler{id});
        else Vship_ButteraugliFree(Vship_ButteraugliHandler{id});
    }
    delete d;
}

void create(const VSMap* in, VSMap* out, VSCore* core, const VSAPI* api, Metric metric) {
    Filter* d = new Filter();
    d->metric = metric;
    d->ref = to_rgbs(api->mapGetNode(in, "reference", 0, nullptr), core, api);
    d->dist = to_rgbs(api->mapGetNode(in, "distorted", 0, nullptr), core, api);
    auto fail = [&](Vship_Exception e) {
        api->mapSetError(out, vship_error(e).c_str());
        free_filter(d, core, api);
    };
    const VSVideoInfo* vr = api->getVideoInfo(d->ref);
    const VSVideoInfo* vd = api->getVideoInfo(d->dist);
    if (!vsh::isSameVideoInfo(vr, vd)) return fail(Vship_DifferingInputType);
    if (vr->format.colorFamily != cfRGB || vr->format.sampleType != stFloat || vr->format.bitsPerSample != 32)
        return fail(Vship_NonRGBSInput);
    int err = 0;
    int gpu = (int)api->mapGetInt(in, "gpu_id", 0, &err);
    if (err) gpu = 0;
    if (Vship_Exception e = Vship_GPUFullCheck(gpu); e != Vship_NoError) return fail(e);
    VSCoreInfo info;
    api->getCoreInfo(core, &info);
    int streams = (int)api->mapGetInt(in, "numStream", 0, &err);
    if (err) streams = metric == Metric::SSIMU2 ? info.numThreads : 4;
    streams = std::max(1, std::min(streams, info.numThreads));
    int qnorm = 2;
    float intensity = 203.f;
    if (metric == Metric::Butteraugli) {
        qnorm = (int)api->mapGetInt(in, "qnorm", 0, &err);
        if (err) qnorm = 2;
        intensity = (float)api->mapGetFloat(in, "intensity_multiplier", 0, &err);
        if (err) intensity = 203.f;
        const int64_t dm = api->mapGetInt(in, "distmap", 0, &err);
        d->distmap = !err && dm != 0;
    }
    for (int s = 0; s < streams; s++) {
        Vship_Exception e;
        if (metric == Metric::SSIMU2) {
            Vship_SSIMU2Handler h;
            e = Vship_SSIMU2Init(&h, vr->width, vr->height);
            if (e == Vship_NoError) d->handlers.push_back(h.id);
        } else {
            Vship_ButteraugliHandler h;
            e = Vship_ButteraugliInitv2(&h, vr->width, vr->height, qnorm, intensity);
            if (e == Vship_NoError) d->handlers.push_back(h.id);
        }
        if (e != Vship_NoError) return fail(e);
        d->idle.push_back(s);
    }
    VSVideoInfo vo = *vd;
    if (d->distmap) api->queryVideoFormat(&vo.format, cfGray, stFloat, 32, 0, 0, core);
    VSFilterDependency deps[] = {{d->ref, rpStrictSpatial}, {d->dist, rpStrictSpatial}};
    api->createVideoFilter(out, "vship", &vo, get_frame, free_filter, fmParallel, deps, 2, d, core);
}

void VS_CC ssimulacra2_create(const VSMap* in, VSMap* out, void*, VSCore* core, const VSAPI* api) {
    create(in, out, core, api, Metric::SSIMU2);
}
void VS_CC butteraugli_create(const VSMap* in, VSMap* out, void*, VSCore* core, const VSAPI* api) {
    create(in, out, core, api, Metric::Butteraugli);
}

// src/VshipLib.cpp:8-56
void VS_CC gpu_info(const VSMap* in, VSMap* out, void*, VSCore*, const VSAPI* api) {
    int count = 0;
    if (Vship_Exception e = Vship_GetDeviceCount(&count); e != Vship_NoError) {
        api->mapSetError(out, vship_error(e).c_str());
        return;
    }
    int err = 0;
    const int gpu = (int)api->mapGetInt(in, "gpu_id", 0, &err);
    std::ostringstream ss;
    if (err) {
        for (int i = 0; i < count; i++) {
            Vship_DeviceInfo di;
            Vship_GetDeviceInfo(&di, i);
            ss << "GPU " << i << ": " << di.name << "\n";
        }
    } else {
        if (gpu < 0 || gpu >= count) {
            api->mapSetError(out, vship_error(Vship_BadDeviceArgument).c_str());
            return;
        }
        Vship_DeviceInfo di;
        Vship_GetDeviceInfo(&di, gpu);
        ss << "Name: " << di.name << "\n"
           << "MultiProcessorCount: " << di.MultiProcessorCount << "\n"
           << "WarpSize: " << di.WarpSize << "\n"
           << "VRAMCapacity: " << (double)di.VRAMSize / 1e9 << " GB\n"
           << "Integrated: " << di.integrated << "\n"
           << "PassKernelCheck : " << (Vship_GPUFullCheck(gpu) == Vship_NoError ? 1 : 0) << "\n";
    }
    const std::string s = ss.str();
    api->mapSetData(out, "gpu_human_data", s.data(), (int)s.size(), dtUtf8, maReplace);
}

}  // namespace

VS_EXTERNAL_API(void) VapourSynthPluginInit2(VSPlugin* plugin, const VSPLUGINAPI* vspapi) {
    vspapi->configPlugin("com.lumen.vship", "vship", "VapourSynth GPU Perceptual Metrics", VS_MAKE_VERSION(3, 3),
                         VAPOURSYNTH_API_VERSION, 0, plugin);
    vspapi->registerFunction("SSIMULACRA2", "reference:vnode;distorted:vnode;numStream:int:opt;gpu_id:int:opt;",
                             "clip:vnode;", ssimulacra2_create, nullptr, plugin);
    vspapi->registerFunction("BUTTERAUGLI",
                             "reference:vnode;distorted:vnode;qnorm:int:opt;intensity_multiplier:float:opt;"
                             "distmap:int:opt;numStream:int:opt;gpu_id:int:opt;",
                             "clip:vnode;", butteraugli_create, nullptr, plugin);
    vspapi->registerFunction("GpuInfo", "gpu_id:int:opt;", "gpu_human_data:data;", gpu_info, nullptr, plugin);
}
