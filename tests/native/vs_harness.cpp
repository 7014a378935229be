// vs_harness.cpp -- a minimal stand-in for the VapourSynth core, enough to run a plugin's filters
// end to end without VapourSynth installed (test infrastructure only).
//
// It dlopens a plugin library, calls its VapourSynthPluginInit2 with a VSPLUGINAPI that records
// the registered functions, builds two RGBS source clips from a raw file, calls one registered
// function (SSIMULACRA2, BUTTERAUGLI or GpuInfo) with the arguments given on the command line,
// and pulls every output frame through the filter's getFrame (arInitial, then
// arAllFramesReady with the requested frames) from several host threads at once, as
// VapourSynth does for an fmParallel filter. It prints one JSON object per frame with the
// frame's float properties, and writes GrayS output frames to a file.
//
// Usage: vs_harness <plugin.so> <frames.raw> <function> <threads> <out_frames.raw|-> [key=value ...]
//   frames.raw: int32 width, height, nframes, then per frame 3 float32 planes of the reference
//   and 3 of the distorted clip, rows packed. key=value: int arguments (numStream=3) or, with a
//   dot in the value, float arguments (intensity_multiplier=80.0).
#include <VSHelper4.h>
#include <VapourSynth4.h>

#include <dlfcn.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

struct VSMap {
    struct Entry {
        int type = ptUnset;
        std::vector<int64_t> i;
        std::vector<double> f;
        std::vector<std::string> d;
        std::vector<VSNode*> n;
    };
    std::map<std::string, Entry> kv;
    std::string error;
};

struct VSFrame {
    VSVideoFormat fmt{};
    int w = 0, h = 0;
    ptrdiff_t stride = 0;
    std::vector<std::vector<uint8_t>> planes;
    VSMap props;
    std::atomic<int> refs{1};
};

struct VSNode {
    VSVideoInfo vi{};
    std::atomic<int> refs{1};
    std::vector<VSFrame*> source;  // a source clip's frames
    VSFilterGetFrame get = nullptr;
    VSFilterFree free_fn = nullptr;
    void* inst = nullptr;
    int mode = 0;
};

struct VSCore {
    int threads = 8;
};

struct VSFrameContext {
    std::map<std::pair<VSNode*, int>, const VSFrame*> ready;
    std::vector<std::pair<VSNode*, int>> requested;
    std::string error;
};

struct VSPlugin {
    std::map<std::string, std::pair<std::string, VSPublicFunction>> fns;
};

static const VSAPI* g_api = nullptr;

static void fmt_of(VSVideoFormat* f, int cf, int st, int bits, int ssw, int ssh) {
    f->colorFamily = cf;
    f->sampleType = st;
    f->bitsPerSample = bits;
    f->bytesPerSample = bits <= 8 ? 1 : bits <= 16 ? 2 : 4;
    f->subSamplingW = ssw;
    f->subSamplingH = ssh;
    f->numPlanes = cf == cfGray ? 1 : 3;
}

static VSFrame* new_frame(const VSVideoFormat* fmt, int w, int h) {
    VSFrame* f = new VSFrame();
    f->fmt = *fmt;
    f->w = w;
    f->h = h;
    f->stride = ((ptrdiff_t)w * fmt->bytesPerSample + 63) / 64 * 64;  // padded rows, as VapourSynth's
    f->planes.assign(fmt->numPlanes, std::vector<uint8_t>((size_t)f->stride * h, 0));
    return f;
}

// ------------------------------------------------------------------------------------------
// the VSAPI functions the plugin uses

static void VS_CC freeFrame(const VSFrame* f) noexcept {
    if (f && --const_cast<VSFrame*>(f)->refs == 0) delete f;
}
static const VSFrame* VS_CC addFrameRef(const VSFrame* f) noexcept {
    ++const_cast<VSFrame*>(f)->refs;
    return f;
}
static void VS_CC freeNode(VSNode* n) noexcept {
    if (!n || --n->refs > 0) return;
    if (n->free_fn) n->free_fn(n->inst, nullptr, g_api);
    for (VSFrame* f : n->source) freeFrame(f);
    delete n;
}
static VSNode* VS_CC addNodeRef(VSNode* n) noexcept {
    ++n->refs;
    return n;
}
static const VSVideoInfo* VS_CC getVideoInfo(VSNode* n) noexcept { return &n->vi; }
static VSMap* VS_CC createMap() noexcept { return new VSMap(); }
static void VS_CC freeMap(VSMap* m) noexcept {
    if (!m) return;
    for (auto& kv : m->kv)
        for (VSNode* n : kv.second.n) freeNode(n);
    delete m;
}
static void VS_CC mapSetError(VSMap* m, const char* e) noexcept { m->error = e ? e : "(null)"; }
static const char* VS_CC mapGetError(const VSMap* m) noexcept { return m->error.empty() ? nullptr : m->error.c_str(); }

static const VSMap::Entry* find(const VSMap* m, const char* key, int type, int index, int* err) {
    auto it = m->kv.find(key);
    int e = peSuccess;
    const VSMap::Entry* r = nullptr;
    if (it == m->kv.end()) e = peUnset;
    else if (it->second.type != type) e = peType;
    else {
        r = &it->second;
        size_t n = type == ptInt ? r->i.size() : type == ptFloat ? r->f.size() : type == ptData ? r->d.size() : r->n.size();
        if (index < 0 || (size_t)index >= n) e = peIndex, r = nullptr;
    }
    if (err) *err = e;
    else if (e != peSuccess) {
        fprintf(stderr, "harness: missing property %s\n", key);
        abort();
    }
    return r;
}
static int64_t VS_CC mapGetInt(const VSMap* m, const char* key, int index, int* err) noexcept {
    const VSMap::Entry* e = find(m, key, ptInt, index, err);
    return e ? e->i[index] : 0;
}
static double VS_CC mapGetFloat(const VSMap* m, const char* key, int index, int* err) noexcept {
    const VSMap::Entry* e = find(m, key, ptFloat, index, err);
    return e ? e->f[index] : 0.0;
}
static VSNode* VS_CC mapGetNode(const VSMap* m, const char* key, int index, int* err) noexcept {
    const VSMap::Entry* e = find(m, key, ptVideoNode, index, err);
    return e ? addNodeRef(e->n[index]) : nullptr;
}
static VSMap::Entry& slot(VSMap* m, const char* key, int type, int append) {
    VSMap::Entry& e = m->kv[key];
    if (append == maReplace || e.type != type) {
        for (VSNode* n : e.n) freeNode(n);
        e = VSMap::Entry();
        e.type = type;
    }
    return e;
}
static int VS_CC mapSetInt(VSMap* m, const char* key, int64_t v, int append) noexcept {
    slot(m, key, ptInt, append).i.push_back(v);
    return 0;
}
static int VS_CC mapSetFloat(VSMap* m, const char* key, double v, int append) noexcept {
    slot(m, key, ptFloat, append).f.push_back(v);
    return 0;
}
static int VS_CC mapSetData(VSMap* m, const char* key, const char* data, int size, int, int append) noexcept {
    slot(m, key, ptData, append).d.push_back(size < 0 ? std::string(data) : std::string(data, size));
    return 0;
}
static int VS_CC mapConsumeNode(VSMap* m, const char* key, VSNode* n, int append) noexcept {
    slot(m, key, ptVideoNode, append).n.push_back(n);
    return 0;
}
static int VS_CC mapSetNode(VSMap* m, const char* key, VSNode* n, int append) noexcept {
    return mapConsumeNode(m, key, addNodeRef(n), append);
}

static VSFrame* VS_CC newVideoFrame(const VSVideoFormat* fmt, int w, int h, const VSFrame* prop_src, VSCore*) noexcept {
    VSFrame* f = new_frame(fmt, w, h);
    if (prop_src) f->props.kv = prop_src->props.kv;
    return f;
}
static VSFrame* VS_CC copyFrame(const VSFrame* src, VSCore*) noexcept {
    VSFrame* f = new VSFrame();
    f->fmt = src->fmt;
    f->w = src->w;
    f->h = src->h;
    f->stride = src->stride;
    f->planes = src->planes;
    f->props.kv = src->props.kv;
    return f;
}
static VSMap* VS_CC getFramePropertiesRW(VSFrame* f) noexcept { return &f->props; }
static const VSMap* VS_CC getFramePropertiesRO(const VSFrame* f) noexcept { return &f->props; }
static ptrdiff_t VS_CC getStride(const VSFrame* f, int) noexcept { return f->stride; }
static const uint8_t* VS_CC getReadPtr(const VSFrame* f, int p) noexcept { return f->planes[p].data(); }
static uint8_t* VS_CC getWritePtr(VSFrame* f, int p) noexcept { return f->planes[p].data(); }
static int VS_CC getFrameWidth(const VSFrame* f, int) noexcept { return f->w; }
static int VS_CC getFrameHeight(const VSFrame* f, int) noexcept { return f->h; }
static int VS_CC queryVideoFormat(VSVideoFormat* f, int cf, int st, int bits, int ssw, int ssh, VSCore*) noexcept {
    fmt_of(f, cf, st, bits, ssw, ssh);
    return 1;
}

static void VS_CC requestFrameFilter(int n, VSNode* node, VSFrameContext* ctx) noexcept { ctx->requested.push_back({node, n}); }
static const VSFrame* VS_CC getFrameFilter(int n, VSNode* node, VSFrameContext* ctx) noexcept {
    auto it = ctx->ready.find({node, n});
    return it == ctx->ready.end() ? nullptr : addFrameRef(it->second);
}
static void VS_CC setFilterError(const char* msg, VSFrameContext* ctx) noexcept { ctx->error = msg ? msg : "(null)"; }

static void VS_CC createVideoFilter(VSMap* out, const char*, const VSVideoInfo* vi, VSFilterGetFrame get,
                                    VSFilterFree free_fn, int mode, const VSFilterDependency*, int, void* inst,
                                    VSCore*) noexcept {
    VSNode* n = new VSNode();
    n->vi = *vi;
    n->get = get;
    n->free_fn = free_fn;
    n->inst = inst;
    n->mode = mode;
    mapConsumeNode(out, "clip", n, maAppend);
}

static VSPlugin* VS_CC getPluginByID(const char*, VSCore*) noexcept { return nullptr; }  // no resize plugin here
static VSMap* VS_CC invoke(VSPlugin*, const char* name, const VSMap*) noexcept {
    VSMap* m = createMap();
    mapSetError(m, (std::string("harness: no plugin provides ") + name).c_str());
    return m;
}
static void VS_CC getCoreInfo(VSCore* core, VSCoreInfo* info) noexcept {
    memset(info, 0, sizeof(*info));
    info->versionString = "vs_harness";
    info->core = 70;
    info->api = VAPOURSYNTH_API_VERSION;
    info->numThreads = core->threads;
}

// VSPLUGINAPI
static int VS_CC configPlugin(const char* id, const char* ns, const char* name, int, int, int, VSPlugin*) noexcept {
    printf("{\"plugin\": \"%s\", \"namespace\": \"%s\", \"name\": \"%s\"}\n", id, ns, name);
    return 1;
}
static int VS_CC registerFunction(const char* name, const char* args, const char*, VSPublicFunction fn, void*,
                                  VSPlugin* plugin) noexcept {
    plugin->fns[name] = {args, fn};
    return 1;
}

// ------------------------------------------------------------------------------------------

static const VSFrame* produce(VSNode* node, int n, VSCore* core, std::string* err) {
    if (!node->source.empty()) return addFrameRef(node->source[n]);
    VSFrameContext ctx;
    void* frame_data = nullptr;
    node->get(n, arInitial, node->inst, &frame_data, &ctx, core, g_api);
    if (!ctx.error.empty()) {
        *err = ctx.error;
        return nullptr;
    }
    for (auto& rq : ctx.requested) {
        const VSFrame* f = produce(rq.first, rq.second, core, err);
        if (!f) return nullptr;
        ctx.ready[rq] = f;
    }
    const VSFrame* out = node->get(n, arAllFramesReady, node->inst, &frame_data, &ctx, core, g_api);
    for (auto& kv : ctx.ready) freeFrame(kv.second);
    if (!out) *err = ctx.error.empty() ? "getFrame returned no frame" : ctx.error;
    return out;
}

static std::string json_escape(const std::string& s) {
    std::string o;
    for (char c : s) {
        if (c == '"' || c == '\\') o += '\\', o += c;
        else if (c == '\n') o += "\\n";
        else o += c;
    }
    return o;
}

int main(int argc, char** argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s plugin.so frames.raw function threads out.raw|- [key=value ...]\n", argv[0]);
        return 2;
    }
    static VSAPI api;
    memset(&api, 0, sizeof(api));
    api.createVideoFilter = createVideoFilter;
    api.freeNode = freeNode;
    api.addNodeRef = addNodeRef;
    api.getVideoInfo = getVideoInfo;
    api.newVideoFrame = newVideoFrame;
    api.freeFrame = freeFrame;
    api.addFrameRef = addFrameRef;
    api.copyFrame = copyFrame;
    api.getFramePropertiesRO = getFramePropertiesRO;
    api.getFramePropertiesRW = getFramePropertiesRW;
    api.getStride = getStride;
    api.getReadPtr = getReadPtr;
    api.getWritePtr = getWritePtr;
    api.getFrameWidth = getFrameWidth;
    api.getFrameHeight = getFrameHeight;
    api.queryVideoFormat = queryVideoFormat;
    api.getFrameFilter = getFrameFilter;
    api.requestFrameFilter = requestFrameFilter;
    api.setFilterError = setFilterError;
    api.createMap = createMap;
    api.freeMap = freeMap;
    api.mapSetError = mapSetError;
    api.mapGetError = mapGetError;
    api.mapGetInt = mapGetInt;
    api.mapSetInt = mapSetInt;
    api.mapGetFloat = mapGetFloat;
    api.mapSetFloat = mapSetFloat;
    api.mapSetData = mapSetData;
    api.mapGetNode = mapGetNode;
    api.mapSetNode = mapSetNode;
    api.mapConsumeNode = mapConsumeNode;
    api.getPluginByID = getPluginByID;
    api.invoke = invoke;
    api.getCoreInfo = getCoreInfo;
    g_api = &api;
    static VSPLUGINAPI papi;
    memset(&papi, 0, sizeof(papi));
    papi.configPlugin = configPlugin;
    papi.registerFunction = registerFunction;

    void* so = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);
    if (!so) {
        fprintf(stderr, "harness: %s\n", dlerror());
        return 2;
    }
    auto init = (VSInitPlugin)dlsym(so, "VapourSynthPluginInit2");
    if (!init) {
        fprintf(stderr, "harness: no VapourSynthPluginInit2 in %s\n", argv[1]);
        return 2;
    }
    VSPlugin plugin;
    init(&plugin, &papi);
    for (auto& kv : plugin.fns) printf("{\"function\": \"%s\", \"args\": \"%s\"}\n", kv.first.c_str(), kv.second.first.c_str());

    const std::string fname = argv[3];
    const int threads = atoi(argv[4]);
    const std::string outpath = argv[5];
    auto it = plugin.fns.find(fname);
    if (it == plugin.fns.end()) {
        fprintf(stderr, "harness: %s not registered\n", fname.c_str());
        return 2;
    }
    VSCore core;
    core.threads = threads;
    VSMap* in = createMap();
    std::vector<VSNode*> sources;
    if (fname != "GpuInfo") {
        FILE* fp = fopen(argv[2], "rb");
        int hdr[3];
        if (!fp || fread(hdr, sizeof(int), 3, fp) != 3) {
            fprintf(stderr, "harness: cannot read %s\n", argv[2]);
            return 2;
        }
        const int w = hdr[0], h = hdr[1], nf = hdr[2];
        for (int clip = 0; clip < 2; clip++) {
            VSNode* n = new VSNode();
            fmt_of(&n->vi.format, cfRGB, stFloat, 32, 0, 0);
            n->vi.width = w;
            n->vi.height = h;
            n->vi.numFrames = nf;
            n->vi.fpsNum = 24;
            n->vi.fpsDen = 1;
            sources.push_back(n);
        }
        for (int t = 0; t < nf; t++)
            for (int clip = 0; clip < 2; clip++) {
                VSFrame* f = new_frame(&sources[clip]->vi.format, w, h);
                for (int p = 0; p < 3; p++)
                    for (int y = 0; y < h; y++)
                        if (fread(f->planes[p].data() + (size_t)y * f->stride, 4, w, fp) != (size_t)w) {
                            fprintf(stderr, "harness: short read\n");
                            return 2;
                        }
                sources[clip]->source.push_back(f);
            }
        fclose(fp);
        mapConsumeNode(in, "reference", sources[0], maReplace);
        mapConsumeNode(in, "distorted", sources[1], maReplace);
    }
    for (int a = 6; a < argc; a++) {
        std::string kv = argv[a];
        const size_t eq = kv.find('=');
        const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
        if (v.find('.') != std::string::npos) mapSetFloat(in, k.c_str(), atof(v.c_str()), maReplace);
        else mapSetInt(in, k.c_str(), atoll(v.c_str()), maReplace);
    }
    VSMap* out = createMap();
    it->second.second(in, out, nullptr, &core, &api);
    freeMap(in);
    if (const char* e = mapGetError(out)) {
        printf("{\"error\": \"%s\"}\n", json_escape(e).c_str());
        freeMap(out);
        return 0;
    }
    if (fname == "GpuInfo") {
        int err = 0;
        const VSMap::Entry* e = find(out, "gpu_human_data", ptData, 0, &err);
        printf("{\"gpu_human_data\": \"%s\"}\n", err ? "" : json_escape(e->d[0]).c_str());
        freeMap(out);
        return 0;
    }
    VSNode* node = mapGetNode(out, "clip", 0, nullptr);
    freeMap(out);
    const int nf = node->vi.numFrames;
    printf("{\"output\": {\"width\": %d, \"height\": %d, \"frames\": %d, \"color_family\": %d, \"bits\": %d}}\n",
           node->vi.width, node->vi.height, nf, node->vi.format.colorFamily, node->vi.format.bitsPerSample);
    std::vector<const VSFrame*> frames(nf, nullptr);
    std::vector<std::string> errors(nf);
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int k = 0; k < threads; k++)
        pool.emplace_back([&] {
            for (int t; (t = next++) < nf;) frames[t] = produce(node, t, &core, &errors[t]);
        });
    for (auto& th : pool) th.join();
    FILE* fo = outpath == "-" ? nullptr : fopen(outpath.c_str(), "wb");
    for (int t = 0; t < nf; t++) {
        if (!frames[t]) {
            printf("{\"frame\": %d, \"error\": \"%s\"}\n", t, json_escape(errors[t]).c_str());
            continue;
        }
        printf("{\"frame\": %d", t);
        for (auto& kv : frames[t]->props.kv)
            if (kv.second.type == ptFloat) printf(", \"%s\": %.17g", kv.first.c_str(), kv.second.f[0]);
        printf("}\n");
        if (fo && frames[t]->fmt.colorFamily == cfGray)
            for (int y = 0; y < frames[t]->h; y++)
                fwrite(frames[t]->planes[0].data() + (size_t)y * frames[t]->stride, 4, frames[t]->w, fo);
        freeFrame(frames[t]);
    }
    if (fo) fclose(fo);
    freeNode(node);
    return 0;
}
