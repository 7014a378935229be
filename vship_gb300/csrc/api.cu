// api.cpp -- the C ABI of libvship.so (include/VshipAPI.h).
//
// Reference-facing entry points follow src/VshipLib.cpp:66-368 and src/util/gpuhelper.hpp:
// handler ids are small integers reused through a free list (src/util/concurrency.hpp:176-200),
// errors are returned as Vship_Exception, compute calls are synchronous.
//
// GB300-specific differences behind the same interface:
//   * all device memory of a handler (staging planes, pyramid / band planes, partial sums) is
//     allocated once at Init and reused, instead of a stream-ordered malloc per frame pair;
//   * only the width*bytes of each row travel host->device (2-D copies skip stride padding);
//   * the final reductions run on the GPU in FP64, so one 8- or 24-byte result comes back.
#include "../../include/VshipAPI.h"

#include "butter.h"
#include "common.cuh"
#include "ssimu2.h"
#include "multi.h"
#include "serve.h"
#include "profile.h"

#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

using namespace vship;

namespace {

// ------------------------------------------------------------------------------------------
// handler tables

template <typename H>
struct HandleTable {
    std::mutex mu;
    std::vector<std::unique_ptr<H>> items;
    std::vector<int> free_ids;

    int put(std::unique_ptr<H> h) {
        std::lock_guard<std::mutex> g(mu);
        if (!free_ids.empty()) {
            int id = free_ids.back();
            free_ids.pop_back();
            items[id] = std::move(h);
            return id;
        }
        items.push_back(std::move(h));
        return (int)items.size() - 1;
    }
    H* get(int id) {
        std::lock_guard<std::mutex> g(mu);
        if (id < 0 || id >= (int)items.size() || !items[id]) return nullptr;
        return items[id].get();
    }
    std::unique_ptr<H> take(int id) {
        std::lock_guard<std::mutex> g(mu);
        if (id < 0 || id >= (int)items.size() || !items[id]) return nullptr;
        std::unique_ptr<H> h = std::move(items[id]);
        free_ids.push_back(id);
        return h;
    }
};

bool yuv_from_format(const Vship_YuvFormat& f, int64_t height, YuvParams* out) {
    return make_yuv_params(f.bits, f.subsampling_w, f.subsampling_h, f.matrix, f.range, f.chroma_location, height, out,
                           f.transfer, f.primaries);
}

Vship_Exception to_exc(int e) {
    return (e >= 0 && e <= E_BAD_ERROR_TYPE) ? (Vship_Exception)e : Vship_BadErrorType;
}

int map_cuda(cudaError_t e) {
    if (e == cudaSuccess) return E_OK;
    if (getenv("VSHIP_DEBUG")) fprintf(stderr, "vship: %s\n", cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return E_OUT_OF_VRAM;
    if (e == cudaErrorNoDevice) return E_NO_DEVICE;
    if (e == cudaErrorInvalidDevice) return E_BAD_DEVICE_ARG;
    return E_BAD_DEVICE_CODE;
}

#define TRY_CUDA(expr)                              \
    do {                                            \
        int _rc = map_cuda(expr);                   \
        if (_rc != E_OK) return _rc;                \
    } while (0)

// Copy the three planes of one frame into dense device rows of `row_bytes`. Rows without
// padding travel as one linear copy per plane, or as a single copy when the three planes are
// also adjacent in host memory; padded rows use a 2-D copy that skips the padding.
int upload_frame(uint8_t* dst, const uint8_t* const* src, int64_t stride, int64_t row_bytes, int64_t h,
                 cudaStream_t st) {
    for (int c = 0; c < 3; c++)
        if (!src[c]) return E_BAD_POINTER;
    const size_t plane = (size_t)row_bytes * h;
    if (stride == row_bytes) {
        if (src[1] == src[0] + plane && src[2] == src[1] + plane) {
            TRY_CUDA(cudaMemcpyAsync(dst, src[0], 3 * plane, cudaMemcpyHostToDevice, st));
            return E_OK;
        }
        for (int c = 0; c < 3; c++)
            TRY_CUDA(cudaMemcpyAsync(dst + (size_t)c * plane, src[c], plane, cudaMemcpyHostToDevice, st));
        return E_OK;
    }
    for (int c = 0; c < 3; c++)
        TRY_CUDA(cudaMemcpy2DAsync(dst + (size_t)c * plane, row_bytes, src[c], stride, row_bytes, h,
                                   cudaMemcpyHostToDevice, st));
    return E_OK;
}

// Host-buffer handler state shared by both metrics: stream, staging planes, pinned result.
struct HostPath {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint8_t* staging = nullptr;      // 2 frames x 3 planes x h x (w*4) bytes
    FrameDesc* frames_d = nullptr;   // [0..1]: 2-byte samples, [2..3]: 4-byte, [4..5]: Y'CbCr
    int64_t yuv_stride = 0, yuv_stride_c = 0;  // row pitches the Y'CbCr descriptors hold
    void* result_h = nullptr;        // pinned
    std::mutex mu;                   // one compute at a time per handler

    int init(int64_t w, int64_t h, size_t result_bytes) {
        TRY_CUDA(cudaGetDevice(&device));
        TRY_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        const size_t plane4 = (size_t)w * 4 * h;
        TRY_CUDA(vship_malloc((void**)&staging, plane4 * 6));
        TRY_CUDA(vship_malloc((void**)&frames_d, sizeof(FrameDesc) * 6));
        FrameDesc fd[6];
        for (int bps = 2, k = 0; bps <= 4; bps += 2, k++)
            for (int m = 0; m < 2; m++) {
                const size_t plane = (size_t)w * bps * h;
                for (int c = 0; c < 3; c++) fd[k * 2 + m].plane[c] = staging + (size_t)(m * 3 + c) * plane;
                fd[k * 2 + m].stride = w * bps;
                fd[k * 2 + m].stride_c = w * bps;
            }
        for (int m = 0; m < 2; m++) {  // Y'CbCr: planes at the float-plane slots of each frame
            for (int c = 0; c < 3; c++) fd[4 + m].plane[c] = staging + (size_t)(m * 3 + c) * plane4;
            fd[4 + m].stride = w * 2;
            fd[4 + m].stride_c = ((w + 1) / 2) * 2;
        }
        yuv_stride = w * 2;
        yuv_stride_c = ((w + 1) / 2) * 2;
        TRY_CUDA(cudaMemcpy(frames_d, fd, sizeof(fd), cudaMemcpyHostToDevice));
        if (vship_malloc_host((void**)&result_h, result_bytes) != cudaSuccess) return E_OUT_OF_RAM;
        return E_OK;
    }
    void destroy() {
        if (stream) cudaStreamSynchronize(stream);
        if (staging) cudaFree(staging);
        if (frames_d) cudaFree(frames_d);
        if (result_h) cudaFreeHost(result_h);
        if (stream) cudaStreamDestroy(stream);
        staging = nullptr;
        frames_d = nullptr;
        result_h = nullptr;
        stream = nullptr;
    }
    // Uploads both frames; returns the device descriptor pair to pass to an engine.
    int upload(const uint8_t* const* s1, const uint8_t* const* s2, int64_t stride1, int64_t stride2, int64_t w,
               int64_t h, int bps, const FrameDesc** fd_out) {
        if (!s1 || !s2) return E_BAD_POINTER;
        const int64_t row = w * bps;
        if (stride1 < row || stride2 < row) return E_BAD_POINTER;
        const size_t plane = (size_t)row * h;
        int rc = upload_frame(staging, s1, stride1, row, h, stream);
        if (rc) return rc;
        rc = upload_frame(staging + 3 * plane, s2, stride2, row, h, stream);
        if (rc) return rc;
        *fd_out = frames_d + (bps == 4 ? 2 : 0);
        return E_OK;
    }
    // Uploads two Y'CbCr frames (Y, Cb, Cr with their own strides) of format yp into the YUV
    // slots (dense rows) and points their descriptors at them.
    int upload_yuv(const uint8_t* const* s1, const int64_t* st1, const uint8_t* const* s2, const int64_t* st2,
                   int64_t w, int64_t h, const YuvParams& yp, const FrameDesc** fd_out) {
        if (!s1 || !s2 || !st1 || !st2) return E_BAD_POINTER;
        const int64_t cw = yp.ssw ? (w + 1) / 2 : w, ch = yp.ssh ? (h + 1) / 2 : h;
        const size_t plane4 = (size_t)w * 4 * h;
        if (yuv_stride != w * yp.bytes || yuv_stride_c != cw * yp.bytes) {
            FrameDesc fd[2];
            TRY_CUDA(cudaMemcpy(fd, frames_d + 4, sizeof(fd), cudaMemcpyDeviceToHost));
            for (int m = 0; m < 2; m++) {
                fd[m].stride = w * yp.bytes;
                fd[m].stride_c = cw * yp.bytes;
            }
            TRY_CUDA(cudaMemcpy(frames_d + 4, fd, sizeof(fd), cudaMemcpyHostToDevice));
            yuv_stride = w * yp.bytes;
            yuv_stride_c = cw * yp.bytes;
        }
        for (int m = 0; m < 2; m++) {
            const uint8_t* const* src = m == 0 ? s1 : s2;
            const int64_t* st = m == 0 ? st1 : st2;
            for (int c = 0; c < 3; c++) {
                if (!src[c]) return E_BAD_POINTER;
                const int64_t row = (c == 0 ? w : cw) * yp.bytes, rows = c == 0 ? h : ch;
                if (st[c] < row) return E_BAD_POINTER;
                uint8_t* dst = staging + (size_t)(m * 3 + c) * plane4;
                if (st[c] == row)
                    TRY_CUDA(cudaMemcpyAsync(dst, src[c], (size_t)row * rows, cudaMemcpyHostToDevice, stream));
                else
                    TRY_CUDA(cudaMemcpy2DAsync(dst, row, src[c], st[c], row, rows, cudaMemcpyHostToDevice, stream));
            }
        }
        *fd_out = frames_d + 4;
        return E_OK;
    }
};

struct Ssimu2Handle {
    Ssimu2Engine eng;
    HostPath io;
    bool host_io = true;
    YuvParams yuv = yuv420p10_params();  // format of Vship_InYuv frames
    ~Ssimu2Handle() {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaSetDevice(io.device);
        if (host_io) io.destroy();
        eng.destroy();
        cudaSetDevice(dev);
    }
};

struct ButterHandle {
    ButterEngine eng;
    HostPath io;
    bool host_io = true;
    YuvParams yuv = yuv420p10_params();  // format of Vship_InYuv frames
    ~ButterHandle() {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaSetDevice(io.device);
        if (host_io) io.destroy();
        eng.destroy();
        cudaSetDevice(dev);
    }
};

HandleTable<Ssimu2Handle> g_ssimu2;
HandleTable<ButterHandle> g_butter;

struct MultiHandle {
    MultiEngine eng;
    ~MultiHandle() {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaSetDevice(eng.device);
        eng.destroy();
        cudaSetDevice(dev);
    }
};
HandleTable<MultiHandle> g_multi;

struct ServeHandle {
    Server srv;
    ~ServeHandle() { srv.destroy(); }
};
HandleTable<ServeHandle> g_serve;

// Device guard: make the handler's device current for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int check_gpu_count(int* count) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) return E_DEVICE_COUNT;
    if (c == 0) return E_NO_DEVICE;
    *count = c;
    return E_OK;
}

__global__ void probe_kernel(int* out) { *out = 4320984; }

// ------------------------------------------------------------------------------------------
// compute bodies

// yuv_fixed: the Yuv420p10 entry points, whose format is fixed whatever the handler's setting
int ssimu2_compute(int id, double* score, const uint8_t* s1[3], const uint8_t* s2[3], int64_t stride1,
                   int64_t stride2, int intype, const int64_t* ystr1 = nullptr, const int64_t* ystr2 = nullptr,
                   bool yuv_fixed = false) {
    Ssimu2Handle* h = g_ssimu2.get(id);
    if (!h || !h->host_io) return E_BAD_HANDLER;
    if (!score) return E_BAD_POINTER;
    std::lock_guard<std::mutex> lk(h->io.mu);
    DeviceGuard dg(h->io.device);
    const int bps = intype == IN_FLOAT ? 4 : 2;
    const YuvParams yp = yuv_fixed ? yuv420p10_params() : h->yuv;
    const FrameDesc* fd = nullptr;
    int rc = intype == IN_YUV ? h->io.upload_yuv(s1, ystr1, s2, ystr2, h->eng.w, h->eng.h, yp, &fd)
                              : h->io.upload(s1, s2, stride1, stride2, h->eng.w, h->eng.h, bps, &fd);
    if (rc) return rc;
    rc = h->eng.launch(fd, intype, 1, nullptr, h->io.stream, &yp);
    if (rc) return rc;
    TRY_CUDA(cudaMemcpyAsync(h->io.result_h, h->eng.scores, sizeof(double), cudaMemcpyDeviceToHost, h->io.stream));
    TRY_CUDA(cudaStreamSynchronize(h->io.stream));
    *score = *(double*)h->io.result_h;
    return E_OK;
}

int butter_compute(int id, double norms[3], const uint8_t* dstp, int64_t dststride, const uint8_t* s1[3],
                   const uint8_t* s2[3], int64_t stride1, int64_t stride2, int intype,
                   const int64_t* ystr1 = nullptr, const int64_t* ystr2 = nullptr, bool yuv_fixed = false) {
    ButterHandle* h = g_butter.get(id);
    if (!h || !h->host_io) return E_BAD_HANDLER;
    if (dstp && dststride < h->eng.w * 4) return E_BAD_POINTER;  // checked before any work is queued
    std::lock_guard<std::mutex> lk(h->io.mu);
    DeviceGuard dg(h->io.device);
    const int bps = intype == IN_FLOAT ? 4 : 2;
    const YuvParams yp = yuv_fixed ? yuv420p10_params() : h->yuv;
    const FrameDesc* fd = nullptr;
    int rc = intype == IN_YUV ? h->io.upload_yuv(s1, ystr1, s2, ystr2, h->eng.w, h->eng.h, yp, &fd)
                              : h->io.upload(s1, s2, stride1, stride2, h->eng.w, h->eng.h, bps, &fd);
    if (rc) return rc;
    rc = h->eng.launch(fd, intype, 1, nullptr, h->io.stream, &yp);
    if (rc) return rc;
    if (dstp) {
        const int64_t row = h->eng.w * 4;
        TRY_CUDA(cudaMemcpy2DAsync((void*)dstp, dststride, h->eng.distmap, row, row, h->eng.h, cudaMemcpyDeviceToHost,
                                   h->io.stream));
    }
    TRY_CUDA(cudaMemcpyAsync(h->io.result_h, h->eng.norms, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->io.stream));
    TRY_CUDA(cudaStreamSynchronize(h->io.stream));
    std::memcpy(norms, h->io.result_h, 3 * sizeof(double));
    return E_OK;
}

int butter_compute_int(int id, Vship_ButteraugliScore* score, const uint8_t* dstp, int64_t dststride,
                       const uint8_t* s1[3], const uint8_t* s2[3], int64_t stride1, int64_t stride2, int intype) {
    if (!score) return E_BAD_POINTER;
    double n[3];
    int rc = butter_compute(id, n, dstp, dststride, s1, s2, stride1, stride2, intype);
    if (rc) return rc;
    // src/VshipLib.cpp:306-308 assigns the float norms to the int fields (truncation).
    score->norm2 = (int)(float)n[0];
    score->norm3 = (int)(float)n[1];
    score->norminf = (int)(float)n[2];
    return E_OK;
}

const char* error_name_and_text(int e) {
    switch (e) {
        case E_OK: return "NoError: the call succeeded";
        case E_OUT_OF_VRAM: return "OutOfVRAM: a GPU memory allocation failed. (Advice) use fewer handlers / numStream or a smaller resolution";
        case E_OUT_OF_RAM: return "OutOfRAM: a host (pinned) memory allocation failed. (Advice) check the system's free RAM";
        case E_DIFFERING_INPUT: return "DifferingInputType: the two clips differ in width, height, format or length";
        case E_NON_RGBS: return "NonRGBSInput: the input could not be brought to planar float RGB. (Advice) convert to RGBS before calling";
        case E_DEVICE_COUNT: return "DeviceCountError: the number of GPUs could not be queried. (Advice) check the NVIDIA driver installation";
        case E_NO_DEVICE: return "NoDeviceDetected: no GPU was found. (Advice) check the NVIDIA driver and that the process can see a GPU";
        case E_BAD_DEVICE_ARG: return "BadDeviceArgument: gpu_id is negative or not smaller than the number of GPUs";
        case E_BAD_DEVICE_CODE: return "BadDeviceCode: a GPU kernel or CUDA call failed. (Advice) this library targets sm_103a (GB300); check the GPU model";
        case E_BAD_HANDLER: return "BadHandler: the handler was never initialised or was already freed";
        case E_BAD_POINTER: return "BadPointer: a pointer argument was NULL, a stride was smaller than a row, or the memory was not from Vship_PinnedMalloc";
        default: return "BadErrorType: unknown error";
    }
}

}  // namespace

namespace vship {
int prof_report(char* buf, int len);
void prof_set(bool on);
}  // namespace vship

// ==========================================================================================
extern "C" {

void Vship_ProfileSetEnabled(int enabled) { vship::prof_set(enabled != 0); }

int Vship_ProfileReport(char* out_json, int len) { return vship::prof_report(out_json, len); }


Vship_Version Vship_GetVersion(void) {
    Vship_Version v;
    v.major = 3;
    v.minor = 1;
    v.minorMinor = 0;
    v.backend = Vship_Cuda;
    return v;
}

Vship_Exception Vship_GetDeviceCount(int* number) {
    if (!number) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    *number = c;
    return Vship_NoError;
}

Vship_Exception Vship_SetDevice(int gpu_id) {
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    if (gpu_id < 0 || gpu_id >= c) return Vship_BadDeviceArgument;
    if (cudaSetDevice(gpu_id) != cudaSuccess) return Vship_BadDeviceCode;
    return Vship_NoError;
}

Vship_Exception Vship_GetDeviceInfo(Vship_DeviceInfo* info, int gpu_id) {
    if (!info) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    if (gpu_id < 0 || gpu_id >= c) return Vship_BadDeviceArgument;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, gpu_id) != cudaSuccess) return Vship_BadDeviceCode;
    std::memset(info->name, 0, sizeof(info->name));
    std::strncpy(info->name, p.name, sizeof(info->name) - 1);
    info->VRAMSize = p.totalGlobalMem;
    info->integrated = p.integrated;
    info->MultiProcessorCount = p.multiProcessorCount;
    info->WarpSize = p.warpSize;
    return Vship_NoError;
}

Vship_Exception Vship_GPUFullCheck(int gpu_id) {
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    if (gpu_id < 0 || gpu_id >= c) return Vship_BadDeviceArgument;
    if (cudaSetDevice(gpu_id) != cudaSuccess) return Vship_BadDeviceCode;
    int* d = nullptr;
    int v = 0;
    if (vship_malloc((void**)&d, sizeof(int)) != cudaSuccess) return Vship_BadDeviceCode;
    cudaMemset(d, 0, sizeof(int));
    probe_kernel<<<1, 1>>>(d);
    cudaError_t e = cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess || v != 4320984) return Vship_BadDeviceCode;
    return Vship_NoError;
}

int Vship_GetErrorMessage(Vship_Exception exception, char* out_message, int len) {
    const char* m = error_name_and_text((int)exception);
    const int need = (int)std::strlen(m) + 1;
    if (len <= 0 || !out_message) return need;
    const int ncopy = std::min(len - 1, need - 1);
    std::memcpy(out_message, m, ncopy);
    out_message[ncopy] = '\0';
    return need;
}

Vship_Exception Vship_PinnedMalloc(void** ptr, uint64_t size) {
    if (!ptr) return Vship_BadPointer;
    if (vship_malloc_host(ptr, size) != cudaSuccess) return Vship_OutOfRAM;
    return Vship_NoError;
}

Vship_Exception Vship_PinnedFree(void* ptr) {
    if (cudaFreeHost(ptr) != cudaSuccess) return Vship_BadPointer;
    return Vship_NoError;
}

// ----- SSIMU2 -----------------------------------------------------------------------------

static Vship_Exception ssimu2_init(Vship_SSIMU2Handler* handler, int width, int height, int max_pairs,
                                   bool host_io, int flags = 0) {
    if (!handler) return Vship_BadPointer;
    if (width <= 0 || height <= 0 || max_pairs <= 0) return Vship_BadPointer;
    if (flags & ~(int)Vship_SSIMU2Fp16Deltas) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    std::unique_ptr<Ssimu2Handle> h(new Ssimu2Handle());
    h->host_io = host_io;
    if (cudaGetDevice(&h->io.device) != cudaSuccess) return Vship_BadDeviceCode;
    rc = h->eng.init(width, height, max_pairs, (flags & Vship_SSIMU2Fp16Deltas) != 0);
    if (!rc && host_io) rc = h->io.init(width, height, sizeof(double));
    if (rc) return to_exc(rc);
    handler->id = g_ssimu2.put(std::move(h));
    return Vship_NoError;
}

Vship_Exception Vship_SSIMU2Init(Vship_SSIMU2Handler* handler, int width, int height) {
    return ssimu2_init(handler, width, height, 1, true);
}

Vship_Exception Vship_SSIMU2BatchInit(Vship_SSIMU2Handler* handler, int width, int height, int max_pairs) {
    return ssimu2_init(handler, width, height, max_pairs, false);
}

Vship_Exception Vship_SSIMU2Free(Vship_SSIMU2Handler handler) {
    std::unique_ptr<Ssimu2Handle> h = g_ssimu2.take(handler.id);
    if (!h) return Vship_BadHandler;
    return Vship_NoError;
}

Vship_Exception Vship_ComputeSSIMU2Float(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                         const uint8_t* srcp2[3], int64_t stride) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, stride, stride, IN_FLOAT));
}
Vship_Exception Vship_ComputeSSIMU2Floatv2(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                           const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, stride, stride2, IN_FLOAT));
}
Vship_Exception Vship_ComputeSSIMU2Uint16(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                          const uint8_t* srcp2[3], int64_t stride) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, stride, stride, IN_UINT16));
}
Vship_Exception Vship_ComputeSSIMU2Uint16v2(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                            const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, stride, stride2, IN_UINT16));
}

Vship_Exception Vship_ComputeSSIMU2Yuv420p10(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                             const int64_t stride1[3], const uint8_t* srcp2[3],
                                             const int64_t stride2[3]) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, 0, 0, IN_YUV, stride1, stride2, true));
}

Vship_Exception Vship_ComputeSSIMU2Yuv(Vship_SSIMU2Handler handler, double* score, const uint8_t* srcp1[3],
                                       const int64_t stride1[3], const uint8_t* srcp2[3], const int64_t stride2[3]) {
    return to_exc(ssimu2_compute(handler.id, score, srcp1, srcp2, 0, 0, IN_YUV, stride1, stride2, false));
}

Vship_Exception Vship_SSIMU2SetYuvFormat(Vship_SSIMU2Handler handler, const Vship_YuvFormat* format) {
    Ssimu2Handle* h = g_ssimu2.get(handler.id);
    if (!h) return Vship_BadHandler;
    YuvParams p;
    if (!format || !yuv_from_format(*format, h->eng.h, &p)) return Vship_BadPointer;
    std::lock_guard<std::mutex> lk(h->io.mu);
    h->yuv = p;
    return Vship_NoError;
}

Vship_Exception Vship_SSIMU2ComputeDeviceAsync(Vship_SSIMU2Handler handler, const Vship_DeviceFrame* frames,
                                               int npairs, Vship_InputType input_type, double* scores_dev,
                                               void* stream) {
    Ssimu2Handle* h = g_ssimu2.get(handler.id);
    if (!h) return Vship_BadHandler;
    if (!frames || !scores_dev) return Vship_BadPointer;
    if (npairs <= 0 || npairs > h->eng.max_pairs) return Vship_BadPointer;
    if ((int)input_type < 0 || (int)input_type > 4) return Vship_BadPointer;
    static_assert(sizeof(Vship_DeviceFrame) == sizeof(FrameDesc), "frame descriptor layout");
    DeviceGuard dg(h->io.device);
    return to_exc(h->eng.launch(reinterpret_cast<const FrameDesc*>(frames), (int)input_type, npairs, scores_dev,
                                (cudaStream_t)stream, &h->yuv));
}

uint64_t Vship_SSIMU2DeviceBytes(int width, int height, int max_pairs) {
    return (uint64_t)Ssimu2Engine::device_bytes(width, height, max_pairs);
}

Vship_Exception Vship_SSIMU2InitEx(Vship_SSIMU2Handler* handler, int width, int height, int flags) {
    return ssimu2_init(handler, width, height, 1, true, flags);
}

Vship_Exception Vship_SSIMU2BatchInitEx(Vship_SSIMU2Handler* handler, int width, int height, int max_pairs,
                                        int flags) {
    return ssimu2_init(handler, width, height, max_pairs, false, flags);
}

uint64_t Vship_SSIMU2DeviceBytesEx(int width, int height, int max_pairs, int flags) {
    return (uint64_t)Ssimu2Engine::device_bytes(width, height, max_pairs, (flags & Vship_SSIMU2Fp16Deltas) != 0);
}

// ----- Butteraugli ------------------------------------------------------------------------

static Vship_Exception butter_init(Vship_ButteraugliHandler* handler, int width, int height, int Qnorm,
                                   float intensity_multiplier, int max_pairs, bool host_io, int flags = 0) {
    if (!handler) return Vship_BadPointer;
    if (width <= 0 || height <= 0 || max_pairs <= 0) return Vship_BadPointer;
    if (flags & ~(int)Vship_ButterHalfBands) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    std::unique_ptr<ButterHandle> h(new ButterHandle());
    h->host_io = host_io;
    if (cudaGetDevice(&h->io.device) != cudaSuccess) return Vship_BadDeviceCode;
    h->eng.half_bands = (flags & Vship_ButterHalfBands) != 0;
    rc = h->eng.init(width, height, Qnorm, intensity_multiplier, max_pairs);
    if (!rc && host_io) rc = h->io.init(width, height, 3 * sizeof(double));
    if (rc) return to_exc(rc);
    handler->id = g_butter.put(std::move(h));
    return Vship_NoError;
}

Vship_Exception Vship_ButteraugliInitv2(Vship_ButteraugliHandler* handler, int width, int height, int Qnorm,
                                        float intensity_multiplier) {
    return butter_init(handler, width, height, Qnorm, intensity_multiplier, 1, true);
}

Vship_Exception Vship_ButteraugliBatchInit(Vship_ButteraugliHandler* handler, int width, int height, int Qnorm,
                                           float intensity_multiplier, int max_pairs) {
    return butter_init(handler, width, height, Qnorm, intensity_multiplier, max_pairs, false);
}

Vship_Exception Vship_ButteraugliComputeDeviceAsync(Vship_ButteraugliHandler handler, const Vship_DeviceFrame* frames,
                                                    int npairs, Vship_InputType input_type, double* norms_dev,
                                                    float* distmaps_dev, void* stream) {
    ButterHandle* h = g_butter.get(handler.id);
    if (!h) return Vship_BadHandler;
    if (!frames || !norms_dev) return Vship_BadPointer;
    if (npairs <= 0 || npairs > h->eng.max_pairs) return Vship_BadPointer;
    if ((int)input_type < 0 || (int)input_type > 4) return Vship_BadPointer;
    DeviceGuard dg(h->io.device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = h->eng.launch(reinterpret_cast<const FrameDesc*>(frames), (int)input_type, npairs, norms_dev, st, &h->yuv);
    if (rc) return to_exc(rc);
    if (distmaps_dev) {
        const size_t bytes = sizeof(float) * (size_t)h->eng.w * h->eng.h * npairs;
        if (cudaMemcpyAsync(distmaps_dev, h->eng.distmap, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return Vship_BadPointer;
    }
    return Vship_NoError;
}

uint64_t Vship_ButteraugliDeviceBytes(int width, int height, int max_pairs) {
    return (uint64_t)ButterEngine::device_bytes(width, height, max_pairs);
}

Vship_Exception Vship_ButteraugliInitEx(Vship_ButteraugliHandler* handler, int width, int height, int Qnorm,
                                        float intensity_multiplier, int flags) {
    return butter_init(handler, width, height, Qnorm, intensity_multiplier, 1, true, flags);
}

Vship_Exception Vship_ButteraugliBatchInitEx(Vship_ButteraugliHandler* handler, int width, int height, int Qnorm,
                                             float intensity_multiplier, int max_pairs, int flags) {
    return butter_init(handler, width, height, Qnorm, intensity_multiplier, max_pairs, false, flags);
}

uint64_t Vship_ButteraugliDeviceBytesEx(int width, int height, int max_pairs, int flags) {
    return (uint64_t)ButterEngine::device_bytes(width, height, max_pairs, (flags & Vship_ButterHalfBands) != 0);
}

Vship_Exception Vship_ButteraugliInit(Vship_ButteraugliHandler* handler, int width, int height,
                                      float intensity_multiplier) {
    return Vship_ButteraugliInitv2(handler, width, height, 2, intensity_multiplier);
}

Vship_Exception Vship_ButteraugliFree(Vship_ButteraugliHandler handler) {
    std::unique_ptr<ButterHandle> h = g_butter.take(handler.id);
    if (!h) return Vship_BadHandler;
    return Vship_NoError;
}

Vship_Exception Vship_ComputeButteraugliFloat(Vship_ButteraugliHandler handler, Vship_ButteraugliScore* score,
                                              const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                              const uint8_t* srcp2[3], int64_t stride) {
    return to_exc(butter_compute_int(handler.id, score, dstp, dststride, srcp1, srcp2, stride, stride, IN_FLOAT));
}
Vship_Exception Vship_ComputeButteraugliFloatv2(Vship_ButteraugliHandler handler, Vship_ButteraugliScore* score,
                                                const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                                const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    return to_exc(butter_compute_int(handler.id, score, dstp, dststride, srcp1, srcp2, stride, stride2, IN_FLOAT));
}
Vship_Exception Vship_ComputeButteraugliUint16(Vship_ButteraugliHandler handler, Vship_ButteraugliScore* score,
                                               const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                               const uint8_t* srcp2[3], int64_t stride) {
    return to_exc(butter_compute_int(handler.id, score, dstp, dststride, srcp1, srcp2, stride, stride, IN_UINT16));
}
Vship_Exception Vship_ComputeButteraugliUint16v2(Vship_ButteraugliHandler handler, Vship_ButteraugliScore* score,
                                                 const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                                 const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    return to_exc(butter_compute_int(handler.id, score, dstp, dststride, srcp1, srcp2, stride, stride2, IN_UINT16));
}
Vship_Exception Vship_ComputeButteraugliFloatv3(Vship_ButteraugliHandler handler, double norms[3], const uint8_t* dstp,
                                                int64_t dststride, const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                int64_t stride, int64_t stride2) {
    if (!norms) return Vship_BadPointer;
    return to_exc(butter_compute(handler.id, norms, dstp, dststride, srcp1, srcp2, stride, stride2, IN_FLOAT));
}
Vship_Exception Vship_ComputeButteraugliYuv420p10(Vship_ButteraugliHandler handler, double norms[3],
                                                  const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                                  const int64_t stride1[3], const uint8_t* srcp2[3],
                                                  const int64_t stride2[3]) {
    if (!norms) return Vship_BadPointer;
    return to_exc(butter_compute(handler.id, norms, dstp, dststride, srcp1, srcp2, 0, 0, IN_YUV, stride1,
                                 stride2, true));
}

Vship_Exception Vship_ComputeButteraugliYuv(Vship_ButteraugliHandler handler, double norms[3], const uint8_t* dstp,
                                            int64_t dststride, const uint8_t* srcp1[3], const int64_t stride1[3],
                                            const uint8_t* srcp2[3], const int64_t stride2[3]) {
    if (!norms) return Vship_BadPointer;
    return to_exc(butter_compute(handler.id, norms, dstp, dststride, srcp1, srcp2, 0, 0, IN_YUV, stride1,
                                 stride2, false));
}

Vship_Exception Vship_ButteraugliSetYuvFormat(Vship_ButteraugliHandler handler, const Vship_YuvFormat* format) {
    ButterHandle* h = g_butter.get(handler.id);
    if (!h) return Vship_BadHandler;
    YuvParams p;
    if (!format || !yuv_from_format(*format, h->eng.h, &p)) return Vship_BadPointer;
    std::lock_guard<std::mutex> lk(h->io.mu);
    h->yuv = p;
    return Vship_NoError;
}

Vship_Exception Vship_ComputeButteraugliUint16v3(Vship_ButteraugliHandler handler, double norms[3],
                                                 const uint8_t* dstp, int64_t dststride, const uint8_t* srcp1[3],
                                                 const uint8_t* srcp2[3], int64_t stride, int64_t stride2) {
    if (!norms) return Vship_BadPointer;
    return to_exc(butter_compute(handler.id, norms, dstp, dststride, srcp1, srcp2, stride, stride2, IN_UINT16));
}

// ----- batched multi-resolution ------------------------------------------------------------

Vship_Exception Vship_MultiInit(Vship_MultiHandler* handler, int nres, const int* widths, const int* heights,
                                const int* max_sources, const int* max_pairs, int flags, int Qnorm,
                                float intensity_multiplier, const char* tune_cache_path) {
    if (!handler) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    std::unique_ptr<MultiHandle> h(new MultiHandle());
    rc = h->eng.init(nres, widths, heights, max_sources, max_pairs, flags, Qnorm, intensity_multiplier,
                     tune_cache_path);
    if (rc) return to_exc(rc);
    handler->id = g_multi.put(std::move(h));
    return Vship_NoError;
}

Vship_Exception Vship_MultiFree(Vship_MultiHandler handler) {
    std::unique_ptr<MultiHandle> h = g_multi.take(handler.id);
    if (!h) return Vship_BadHandler;
    return Vship_NoError;
}

Vship_Exception Vship_MultiComputeDeviceAsync(Vship_MultiHandler handler, int nsources, const Vship_DeviceFrame* sources,
                                              const int* source_res, int npairs, const Vship_DeviceFrame* candidates,
                                              const int* candidate_source, Vship_InputType input_type,
                                              double* ssimu2_dev, double* butter_norms_dev, void* stream) {
    MultiHandle* h = g_multi.get(handler.id);
    if (!h) return Vship_BadHandler;
    DeviceGuard dg(h->eng.device);
    return to_exc(h->eng.compute(nsources, reinterpret_cast<const FrameDesc*>(sources), source_res, npairs,
                                 reinterpret_cast<const FrameDesc*>(candidates), candidate_source, (int)input_type,
                                 ssimu2_dev, butter_norms_dev, (cudaStream_t)stream));
}

Vship_Exception Vship_MultiSetYuvFormat(Vship_MultiHandler handler, const Vship_YuvFormat* f) {
    MultiHandle* h = g_multi.get(handler.id);
    if (!h) return Vship_BadHandler;
    if (!f) return Vship_BadPointer;
    DeviceGuard dg(h->eng.device);
    return to_exc(h->eng.set_yuv_format(f->bits, f->subsampling_w, f->subsampling_h, f->matrix, f->range,
                                        f->chroma_location, f->transfer, f->primaries));
}

int Vship_MultiKnobs(Vship_MultiHandler handler, char* out_json, int len) {
    MultiHandle* h = g_multi.get(handler.id);
    const std::string s = h ? h->eng.knobs_json() : std::string("{}");
    const int need = (int)s.size() + 1;
    if (len <= 0 || !out_json) return need;
    const int ncopy = std::min(len - 1, need - 1);
    std::memcpy(out_json, s.data(), ncopy);
    out_json[ncopy] = '\0';
    return need;
}

uint64_t Vship_MultiDeviceBytes(int nres, const int* widths, const int* heights, const int* max_sources,
                                const int* max_pairs, int flags) {
    if (nres <= 0 || nres > kMaxRes || !widths || !heights || !max_sources || !max_pairs) return 0;
    return (uint64_t)MultiEngine::device_bytes(nres, widths, heights, max_sources, max_pairs, flags);
}

// ----- serving runtime ---------------------------------------------------------------------

Vship_Exception Vship_ServeCreate(Vship_ServeHandler* handler, int nres, const int* widths, const int* heights,
                                  Vship_InputType input_type, uint64_t admission_bytes, uint64_t cache_bytes,
                                  int max_batch_pairs, int flags, int Qnorm, float intensity_multiplier) {
    if (!handler) return Vship_BadPointer;
    int c = 0;
    int rc = check_gpu_count(&c);
    if (rc) return to_exc(rc);
    std::unique_ptr<ServeHandle> h(new ServeHandle());
    rc = h->srv.create(nres, widths, heights, (int)input_type, admission_bytes, cache_bytes, max_batch_pairs, flags,
                       Qnorm, intensity_multiplier);
    if (rc) return to_exc(rc);
    handler->id = g_serve.put(std::move(h));
    return Vship_NoError;
}

Vship_Exception Vship_ServeSetYuvFormat(Vship_ServeHandler handler, const Vship_YuvFormat* f) {
    ServeHandle* h = g_serve.get(handler.id);
    if (!h) return Vship_BadHandler;
    if (!f) return Vship_BadPointer;
    return to_exc(h->srv.set_yuv_format(f->bits, f->subsampling_w, f->subsampling_h, f->matrix, f->range,
                                        f->chroma_location, f->transfer, f->primaries));
}

Vship_Exception Vship_ServeSubmit(Vship_ServeHandler handler, const Vship_ServeRequest* q) {
    ServeHandle* h = g_serve.get(handler.id);
    if (!h) return Vship_BadHandler;
    if (!q || !q->candidates || q->npairs <= 0 || !q->results) return Vship_BadPointer;
    ServeReq* r = new ServeReq();
    r->id = q->request_id;
    r->metric = q->metric;
    r->res = q->resolution;
    r->key = q->source_key;
    std::memcpy(&r->src, &q->source, sizeof(FrameDesc));
    r->cands.resize(q->npairs);
    std::memcpy(r->cands.data(), q->candidates, sizeof(FrameDesc) * q->npairs);
    r->out = q->results;
    return to_exc(h->srv.submit(r));
}

Vship_Exception Vship_ServeCancel(Vship_ServeHandler handler, uint64_t request_id) {
    ServeHandle* h = g_serve.get(handler.id);
    if (!h) return Vship_BadHandler;
    return to_exc(h->srv.cancel(request_id));
}

int Vship_ServePoll(Vship_ServeHandler handler, Vship_ServeCompletion* out, int max, double timeout_seconds) {
    ServeHandle* h = g_serve.get(handler.id);
    if (!h || !out || max <= 0) return 0;
    std::vector<ServeDone> d(max);
    const int n = h->srv.poll(d.data(), max, timeout_seconds);
    for (int i = 0; i < n; i++) {
        out[i].request_id = d[i].id;
        out[i].status = d[i].status;
        out[i].latency_seconds = d[i].latency;
    }
    return n;
}

Vship_Exception Vship_ServeDrain(Vship_ServeHandler handler) {
    ServeHandle* h = g_serve.get(handler.id);
    if (!h) return Vship_BadHandler;
    return to_exc(h->srv.drain());
}

int Vship_ServeStats(Vship_ServeHandler handler, char* out_json, int len) {
    ServeHandle* h = g_serve.get(handler.id);
    const std::string s = h ? h->srv.stats_json() : std::string("{}");
    const int need = (int)s.size() + 1;
    if (len <= 0 || !out_json) return need;
    const int ncopy = std::min(len - 1, need - 1);
    std::memcpy(out_json, s.data(), ncopy);
    out_json[ncopy] = '\0';
    return need;
}

Vship_Exception Vship_ServeDestroy(Vship_ServeHandler handler) {
    std::unique_ptr<ServeHandle> h = g_serve.take(handler.id);
    if (!h) return Vship_BadHandler;
    return Vship_NoError;
}

}  // extern "C"
