// noalloc.cu -- SSIMU2 for callers that cannot allocate GPU memory.
//
// Some callers must not allocate device memory once they are running: programs that reserve
// their whole GPU memory budget at start-up (a real-time encoder, a server with a fixed memory
// plan), or plugins hosted by a framework that owns the device memory and forbids allocations
// behind its back. Vship_ComputeSSIMU2DeviceNoAlloc serves them: its scratch -- the two XYB
// pyramids, the per-tile partial sums and the two frame descriptors -- lives in one file-scope
// device array of fixed size, so a call allocates nothing: no cudaMalloc, no cudaFree, no
// allocating library routine.
//
// The array is part of this library's device code: every GPU that loads that code keeps its
// 32 MiB until the process exits. CUDA loads a library's device code lazily by default
// (CUDA_MODULE_LOADING=LAZY), so the 32 MiB is committed on a device by the first call made on
// it: that call looks the array's device address up with cudaGetSymbolAddress (the name of the
// array in host code is only a host-side stand-in), which loads the code and commits the
// array, and uploads the device's constant tables. A caller with a fixed memory plan makes that
// first call at start-up, before it fixes its budget and before any stream capture; if the
// device has no room left for the array, that call returns Vship_OutOfVRAM and a later call
// tries again. All calls on one device share the array and it keeps the last call's contents;
// the kernels write every scratch element they later read, so nothing needs clearing. Calls
// whose GPU work overlaps -- on different streams, or from several host threads -- race on the
// array: order them on one stream or wait between them.
#include "../../include/VshipAPI.h"

#include "common.cuh"
#include "ssimu2.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr size_t kScratchBytes = (size_t)VSHIP_SSIMU2_NOALLOC_SCRATCH_BYTES;
constexpr size_t kFrameBytes = 256;  // two FrameDesc, padded so the pyramid starts 256-byte aligned

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// One-time set-up for the current device (must be current when called).
int scratch_for_current_device(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            // Clear the failed call's error so that no later CUDA call reports it as its own.
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation ? vship::E_OUT_OF_VRAM : vship::E_BAD_DEVICE_CODE;
        }
        int rc = vship::ssimu2_prepare_device();
        if (rc) return rc;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return vship::E_OK;
}

}  // namespace

extern "C" Vship_Exception Vship_ComputeSSIMU2DeviceNoAlloc(const Vship_DeviceFrame* reference,
                                                            const Vship_DeviceFrame* distorted, int width,
                                                            int height, Vship_InputType input_type,
                                                            double* score_dev, void* stream) {
    using namespace vship;
    if (!reference || !distorted || !score_dev) return Vship_BadPointer;
    if (width <= 0 || height <= 0) return Vship_BadPointer;
    if ((int)input_type < 0 || (int)input_type > 4) return Vship_BadPointer;
    const int bps = input_type == Vship_InUint8 ? 1 : input_type == Vship_InFloat ? 4 : 2;
    for (const Vship_DeviceFrame* f : {reference, distorted}) {
        if (!f->plane[0] || !f->plane[1] || !f->plane[2]) return Vship_BadPointer;
        if (f->stride < (int64_t)width * bps) return Vship_BadPointer;
    }
    const Ssimu2Geom geom = make_ssimu2_geom(width, height);
    if (kFrameBytes + ssimu2_scratch_floats(geom) * sizeof(float) > kScratchBytes) return Vship_OutOfVRAM;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return Vship_DeviceCountError;
    if (dev < 0 || dev >= kMaxDevices) return Vship_BadDeviceArgument;
    unsigned char* base = nullptr;
    int rc = scratch_for_current_device(dev, &base);
    if (rc) return (Vship_Exception)rc;
    FrameDesc a, b;
    static_assert(sizeof(Vship_DeviceFrame) == sizeof(FrameDesc), "frame descriptor layout");
    memcpy(&a, reference, sizeof(a));
    memcpy(&b, distorted, sizeof(b));
    rc = ssimu2_launch_scratch(a, b, (int)input_type, geom, reinterpret_cast<FrameDesc*>(base),
                               reinterpret_cast<float*>(base + kFrameBytes), score_dev, (cudaStream_t)stream);
    return (Vship_Exception)rc;
}
