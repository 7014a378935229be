/* VshipAPI.h -- C ABI of vship_gb300, a GB300 (sm_103a) implementation of Vship's per-frame-pair
 * SSIMULACRA2 and Butteraugli scoring.
 *
 * The first block declares exactly the entry points, types and enum values of the reference's
 * src/VshipAPI.h (cited per declaration), so a program or FFI binding written against Vship links
 * against libvship.so unchanged. The second block holds extensions that have no counterpart in
 * the reference; each says why it exists.
 *
 * Threading contract (same as the reference, src/VshipLib.cpp:192-205): handler tables are
 * thread-safe; a compute call is synchronous (it returns after its result is on the host);
 * different handlers may be used concurrently from different threads. Unlike the reference, two
 * threads that share one handler are serialised instead of racing.
 */
#ifndef VSHIP_API_HEADER
#define VSHIP_API_HEADER

#include <stdint.h>

#if defined(_WIN32)
#if defined(EXPORTVSHIPLIB)
#define EXPORTPREPROCESS __declspec(dllexport)
#else
#define EXPORTPREPROCESS __declspec(dllimport)
#endif
#else
#define EXPORTPREPROCESS __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------
 * Reference-compatible surface (src/VshipAPI.h of Vship 3.1.0)
 * ------------------------------------------------------------------------------------------- */

/* src/VshipAPI.h:20-23 */
typedef enum {
    Vship_HIP = 0,
    Vship_Cuda = 1,
} Vship_Backend;

/* src/VshipAPI.h:25-30 */
typedef struct {
    int major;
    int minor;
    int minorMinor;
    Vship_Backend backend;
} Vship_Version;

/* src/VshipAPI.h:32 -- reports 3.1.0, backend Vship_Cuda */
EXPORTPREPROCESS Vship_Version Vship_GetVersion(void);

/* src/VshipAPI.h:35-58 -- values 0..11 are ABI */
typedef enum {
    Vship_NoError = 0,
    Vship_OutOfVRAM,
    Vship_OutOfRAM,
    Vship_DifferingInputType,
    Vship_NonRGBSInput,
    Vship_DeviceCountError,
    Vship_NoDeviceDetected,
    Vship_BadDeviceArgument,
    Vship_BadDeviceCode,
    Vship_BadHandler,
    Vship_BadPointer,
    Vship_BadErrorType,
} Vship_Exception;

/* src/VshipAPI.h:61 */
EXPORTPREPROCESS Vship_Exception Vship_GetDeviceCount(int* number);

/* src/VshipAPI.h:64 */
EXPORTPREPROCESS Vship_Exception Vship_SetDevice(int gpu_id);

/* src/VshipAPI.h:67-73 */
typedef struct {
    char name[256];
    uint64_t VRAMSize;
    int integrated;
    int MultiProcessorCount;
    int WarpSize;
} Vship_DeviceInfo;

/* src/VshipAPI.h:75 */
EXPORTPREPROCESS Vship_Exception Vship_GetDeviceInfo(Vship_DeviceInfo* device_info, int gpu_id);

/* src/VshipAPI.h:78 -- device count, id range, set device, and a one-thread probe kernel */
EXPORTPREPROCESS Vship_Exception Vship_GPUFullCheck(int gpu_id);

/* src/VshipAPI.h:82 -- returns the size needed including the terminating NUL; len == 0 only
 * queries; otherwise copies at most len-1 characters and always NUL-terminates. */
EXPORTPREPROCESS int Vship_GetErrorMessage(Vship_Exception exception, char* out_message, int len);

/* src/VshipAPI.h:87-89 */
typedef struct {
    int id;
} Vship_SSIMU2Handler;

/* src/VshipAPI.h:91-93 -- page-locked host memory; inputs placed there upload at full speed */
EXPORTPREPROCESS Vship_Exception Vship_PinnedMalloc(void** ptr, uint64_t size);
EXPORTPREPROCESS Vship_Exception Vship_PinnedFree(void* ptr);

/* src/VshipAPI.h:96,99 */
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2Init(Vship_SSIMU2Handler* handler, int width, int height);
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2Free(Vship_SSIMU2Handler handler);

/* src/VshipAPI.h:103-111. Inputs: three planar R,G,B planes, BT.709 transfer (gamma-encoded),
 * full range; float32 or uint16 (0..65535) samples; `stride` is the row pitch in bytes of the
 * reference frame (and of the distorted one unless the v2 form gives stride2). Frames are not
 * modified. */
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Float(Vship_SSIMU2Handler handler, double* score,
                                                          const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                          int64_t stride);
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Floatv2(Vship_SSIMU2Handler handler, double* score,
                                                            const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                            int64_t stride, int64_t stride2);
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Uint16(Vship_SSIMU2Handler handler, double* score,
                                                           const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                           int64_t stride);
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Uint16v2(Vship_SSIMU2Handler handler, double* score,
                                                             const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                             int64_t stride, int64_t stride2);

/* src/VshipAPI.h:113-115 */
typedef struct {
    int id;
} Vship_ButteraugliHandler;

/* src/VshipAPI.h:117-121. The reference stores its float norms into these int fields (the
 * value is truncated toward zero); the layout is kept for ABI compatibility. Use the v3 compute
 * functions below for the exact values. */
typedef struct {
    int norm2;
    int norm3;
    int norminf;
} Vship_ButteraugliScore;

/* src/VshipAPI.h:124,127,130 -- Init uses Qnorm = 2 */
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliInit(Vship_ButteraugliHandler* handler, int width, int height,
                                                       float intensity_multiplier);
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliInitv2(Vship_ButteraugliHandler* handler, int width, int height,
                                                         int Qnorm, float intensity_multiplier);
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliFree(Vship_ButteraugliHandler handler);

/* src/VshipAPI.h:137-148. dstp is NULL (no distortion map) or points to dststride*height bytes
 * that receive the float32 distortion map. */
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliFloat(Vship_ButteraugliHandler handler,
                                                               Vship_ButteraugliScore* score, const uint8_t* dstp,
                                                               int64_t dststride, const uint8_t* srcp1[3],
                                                               const uint8_t* srcp2[3], int64_t stride);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliFloatv2(Vship_ButteraugliHandler handler,
                                                                 Vship_ButteraugliScore* score, const uint8_t* dstp,
                                                                 int64_t dststride, const uint8_t* srcp1[3],
                                                                 const uint8_t* srcp2[3], int64_t stride,
                                                                 int64_t stride2);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliUint16(Vship_ButteraugliHandler handler,
                                                                Vship_ButteraugliScore* score, const uint8_t* dstp,
                                                                int64_t dststride, const uint8_t* srcp1[3],
                                                                const uint8_t* srcp2[3], int64_t stride);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliUint16v2(Vship_ButteraugliHandler handler,
                                                                  Vship_ButteraugliScore* score, const uint8_t* dstp,
                                                                  int64_t dststride, const uint8_t* srcp1[3],
                                                                  const uint8_t* srcp2[3], int64_t stride,
                                                                  int64_t stride2);

/* ---------------------------------------------------------------------------------------------
 * Extensions (no counterpart in the reference)
 * ------------------------------------------------------------------------------------------- */

/* Exact Butteraugli norms {Qnorm, 3-norm, inf-norm} as doubles: the reference's score struct
 * truncates them to int. Same arguments as the v2 compute functions otherwise. */
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliFloatv3(Vship_ButteraugliHandler handler, double norms[3],
                                                                 const uint8_t* dstp, int64_t dststride,
                                                                 const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                                 int64_t stride, int64_t stride2);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliUint16v3(Vship_ButteraugliHandler handler, double norms[3],
                                                                  const uint8_t* dstp, int64_t dststride,
                                                                  const uint8_t* srcp1[3], const uint8_t* srcp2[3],
                                                                  int64_t stride, int64_t stride2);

/* Sample formats of the device-resident entry points (0..3 numbered as the reference's
 * InputMemType, src/util/preprocessor.hpp:94). Vship_InYuv is Y'CbCr converted on the GPU to
 * full-range R'G'B' -- the conversion the reference's front-ends do on the CPU before calling
 * the ABI -- in the handler's format (Vship_YuvFormat below), by default 10-bit 4:2:0 in 16-bit
 * little-endian containers, BT.709 limited range, chroma upsampled bilinearly with MPEG-2 (left)
 * siting (Vship_InYuv420p10, the same value): a quarter of the bytes of float RGB. */
typedef enum {
    Vship_InUint8 = 0,
    Vship_InUint16 = 1,
    Vship_InHalf = 2,
    Vship_InFloat = 3,
    Vship_InYuv = 4,
    Vship_InYuv420p10 = 4,
} Vship_InputType;

/* One frame resident in device memory: three planes (R, G, B, or Y, Cb, Cr) and row pitches in
 * bytes (`stride` for RGB planes and luma, `stride_c` for the two chroma planes). */
typedef struct {
    const uint8_t* plane[3];
    int64_t stride;
    int64_t stride_c;
} Vship_DeviceFrame;

/* Host-buffer scoring of 10-bit 4:2:0 Y'CbCr frames (see Vship_InYuv420p10): planes Y, Cb, Cr
 * with their own row strides in bytes (stride1[3], stride2[3]). Synchronous like the reference's
 * compute calls; handlers come from Vship_SSIMU2Init / Vship_ButteraugliInit[v2]. */
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Yuv420p10(Vship_SSIMU2Handler handler, double* score,
                                                              const uint8_t* srcp1[3], const int64_t stride1[3],
                                                              const uint8_t* srcp2[3], const int64_t stride2[3]);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliYuv420p10(Vship_ButteraugliHandler handler, double norms[3],
                                                                   const uint8_t* dstp, int64_t dststride,
                                                                   const uint8_t* srcp1[3], const int64_t stride1[3],
                                                                   const uint8_t* srcp2[3], const int64_t stride2[3]);

/* Y'CbCr input of any common format, converted on the GPU the way the reference's front-ends
 * convert it on the CPU (FFVship's zimg setup, ffmpegToZimgFormat.hpp): chroma upsampled
 * bilinearly at its siting, the matrix and range applied, clamped full-range R'G'B' out.
 * bits: 8 (samples in bytes) to 16 (little-endian 16-bit containers); subsampling_w/_h: log2
 * chroma subsampling (0 or 1: 4:4:4, 4:2:2, 4:2:0); matrix: ITU-T H.273 matrix_coefficients 1
 * (BT.709), 4 (FCC), 5 (BT.470BG), 6 (SMPTE 170M), 7 (SMPTE 240M), 9 (BT.2020 NCL), or 2
 * (unspecified: BT.709 above 650 rows, BT.470BG below, as the reference guesses); range: 0
 * limited, 1 full; chroma_location: 0 left, 1 center, 2 top-left, 3 top, 4 bottom-left,
 * 5 bottom; transfer (H.273 transfer_characteristics): 1 / 6 / 14 / 15 (the BT.709 family,
 * which the reference's metrics linearise as a 2.4 power law) or 2 (unspecified), 13 (sRGB),
 * 4 (gamma 2.2), 5 (gamma 2.8), 8 (linear); primaries (H.273 colour_primaries): 1 (BT.709) or
 * 2 (unspecified), 9 (BT.2020, converted to BT.709 in linear light). */
typedef struct {
    int bits;
    int subsampling_w;
    int subsampling_h;
    int matrix;
    int range;
    int chroma_location;
    int transfer;
    int primaries;
} Vship_YuvFormat;
/* The format a handler uses for Vship_InYuv frames (device entry points) and for the
 * Vship_Compute*Yuv calls; the default is 10-bit 4:2:0 BT.709 limited range, left siting. The
 * Yuv420p10 calls always use that default. Vship_BadPointer: a format outside the list above. */
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2SetYuvFormat(Vship_SSIMU2Handler handler, const Vship_YuvFormat* format);
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliSetYuvFormat(Vship_ButteraugliHandler handler,
                                                               const Vship_YuvFormat* format);
/* Host-buffer scoring of Y'CbCr frames in the handler's format (planes Y, Cb, Cr, strides in bytes). */
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2Yuv(Vship_SSIMU2Handler handler, double* score,
                                                        const uint8_t* srcp1[3], const int64_t stride1[3],
                                                        const uint8_t* srcp2[3], const int64_t stride2[3]);
EXPORTPREPROCESS Vship_Exception Vship_ComputeButteraugliYuv(Vship_ButteraugliHandler handler, double norms[3],
                                                             const uint8_t* dstp, int64_t dststride,
                                                             const uint8_t* srcp1[3], const int64_t stride1[3],
                                                             const uint8_t* srcp2[3], const int64_t stride2[3]);

/* Batched, device-resident SSIMU2 for callers whose frames already live in GPU memory (decoders,
 * encoders' candidate buffers): one launch scores up to max_pairs pairs of one resolution.
 * `frames` is a DEVICE array of 2*npairs frames (pair-major: reference, distorted); scores_dev
 * receives npairs doubles in device memory; `stream` is a cudaStream_t (NULL = legacy default).
 * The call only enqueues work; synchronise the stream before reading scores_dev. */
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2BatchInit(Vship_SSIMU2Handler* handler, int width, int height,
                                                       int max_pairs);
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2ComputeDeviceAsync(Vship_SSIMU2Handler handler,
                                                                const Vship_DeviceFrame* frames, int npairs,
                                                                Vship_InputType input_type, double* scores_dev,
                                                                void* stream);

/* Batched, device-resident Butteraugli (same conventions as the SSIMU2 pair above). norms_dev
 * receives 3 doubles per pair {Qnorm, 3-norm, inf-norm}; distmaps_dev is NULL or a device
 * buffer of npairs * width * height floats (dense rows) that receives the distortion maps. */
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliBatchInit(Vship_ButteraugliHandler* handler, int width,
                                                            int height, int Qnorm, float intensity_multiplier,
                                                            int max_pairs);
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliComputeDeviceAsync(Vship_ButteraugliHandler handler,
                                                                     const Vship_DeviceFrame* frames, int npairs,
                                                                     Vship_InputType input_type, double* norms_dev,
                                                                     float* distmaps_dev, void* stream);
EXPORTPREPROCESS uint64_t Vship_ButteraugliDeviceBytes(int width, int height, int max_pairs);

/* Butteraugli with FP16 band storage -- no counterpart in the reference, whose planes are all
 * FP32 (src/butter/main.hpp:141-195 allocates them per call).
 *
 * With Vship_ButterHalfBands the UHF frequency bands (X, Y) of every image, which only the pair
 * stage reads, are stored as FP16; every other plane and all arithmetic stay FP32. An image then
 * takes 15 instead of 16 FP32-plane equivalents per scale (a 3840x2160 pair: 1.28 instead of
 * 1.36 GB of device memory) at the same throughput. The norms move by the FP16 rounding of those
 * bands: against the FP64 oracle, up to about 5e-6 relative for the 2- and 3-norm and 5e-5 for
 * the inf-norm, which follows one pixel (within 1e-4 on every frame evaluated). FP16 storage of
 * the HF or MF bands as well would move the norms by up to 1e-3 and is not offered.
 * Vship_ButteraugliInitEx is Vship_ButteraugliInitv2 with flags (host-buffer Compute calls);
 * Vship_ButteraugliBatchInitEx is Vship_ButteraugliBatchInit with flags; flags = 0 gives the
 * FP32 planes of the plain functions. Other flag bits are refused (Vship_BadPointer). */
typedef enum { Vship_ButterHalfBands = 1 } Vship_ButterFlags;
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliInitEx(Vship_ButteraugliHandler* handler, int width, int height,
                                                         int Qnorm, float intensity_multiplier, int flags);
EXPORTPREPROCESS Vship_Exception Vship_ButteraugliBatchInitEx(Vship_ButteraugliHandler* handler, int width,
                                                              int height, int Qnorm, float intensity_multiplier,
                                                              int max_pairs, int flags);
EXPORTPREPROCESS uint64_t Vship_ButteraugliDeviceBytesEx(int width, int height, int max_pairs, int flags);

/* SSIMU2 with the distorted image's XYB pyramid stored as FP16 -- no counterpart in the reference,
 * whose pyramids are float3 arrays (src/ssimu2/main.hpp:107-151).
 * With Vship_SSIMU2Fp16Deltas each pair's reference pyramid stays FP32 and the distorted image's
 * is stored as half(distorted - reference), read back as reference + delta: identical samples
 * stay identical and small distortions keep FP16's relative precision, while the pyramid bytes a
 * pair writes and the stats kernel reads fall from 24 to 18 per pyramid element. All arithmetic
 * stays FP32. Against the FP64 oracle the storage moves the score by about 1e-5 at 1920x1080 and
 * up to 2e-4 at 480x270, within the 1e-3 SSIMULACRA2 tolerance; on frames of a few thousand
 * pixels with heavy distortion it can reach 1.5e-3 (the coarsest scales hold a few pixels). Vship_SSIMU2InitEx is Vship_SSIMU2Init with flags (host-buffer
 * Compute calls); Vship_SSIMU2BatchInitEx is Vship_SSIMU2BatchInit with flags; flags = 0 gives
 * the FP32 pyramids of the plain functions. Other flag bits are refused (Vship_BadPointer). */
typedef enum { Vship_SSIMU2Fp16Deltas = 1 } Vship_SSIMU2Flags;
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2InitEx(Vship_SSIMU2Handler* handler, int width, int height, int flags);
EXPORTPREPROCESS Vship_Exception Vship_SSIMU2BatchInitEx(Vship_SSIMU2Handler* handler, int width, int height,
                                                         int max_pairs, int flags);
EXPORTPREPROCESS uint64_t Vship_SSIMU2DeviceBytesEx(int width, int height, int max_pairs, int flags);

/* SSIMU2 for callers that cannot allocate GPU memory -- no counterpart in the reference.
 *
 * Programs that fix their GPU memory budget at start-up (real-time encoders, servers with a
 * static memory plan) and plugins hosted by a framework that owns the device memory cannot let
 * a library call cudaMalloc while they run. This entry point allocates nothing: its scratch is
 * a fixed array of VSHIP_SSIMU2_NOALLOC_SCRATCH_BYTES inside the library's device code, held by
 * every GPU that loads that code until the process exits. The caller passes the two frames
 * (device planes), the resolution, the sample type, a device pointer for the score and a
 * cudaStream_t (NULL = legacy default stream); the call only enqueues work, so synchronise the
 * stream before reading *score_dev.
 *
 * Limit: the two XYB pyramids plus per-tile sums must fit the array; 1280x720 does, larger
 * frames are refused with Vship_OutOfVRAM before anything is launched.
 * CUDA loads device code lazily by default, so the array's 32 MiB is committed on a device by
 * the first call made there, which also uploads that device's constant tables. Make that first
 * call at start-up, before fixing the memory budget and before any stream capture on that
 * device; if the device has no room for the array, it returns Vship_OutOfVRAM.
 * All calls on one device share the array: calls whose GPU work overlaps (different streams or
 * host threads) race, so order them on one stream. */
#define VSHIP_SSIMU2_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
EXPORTPREPROCESS Vship_Exception Vship_ComputeSSIMU2DeviceNoAlloc(const Vship_DeviceFrame* reference,
                                                                  const Vship_DeviceFrame* distorted, int width,
                                                                  int height, Vship_InputType input_type,
                                                                  double* score_dev, void* stream);

/* Batched multi-resolution scoring with source reuse -- no counterpart in the reference, whose
 * API scores one pair of one resolution per call (src/VshipAPI.h:96-148).
 *
 * An encoder's quality search scores each source frame against several encodes of it. One call
 * here scores `npairs` (source, candidate) pairs whose `nsources` sources come in up to 8
 * resolutions: source i has resolution source_res[i] (an index into the widths/heights given
 * at init) and candidate j is scored against source candidate_source[j]. Each source's
 * SSIMULACRA2 XYB pyramid is built once per call and shared by all its candidates; with
 * Vship_MultiFp16 the candidates' pyramids are stored as FP16 differences from their source's.
 * `sources` and `candidates` are HOST arrays of frame descriptors whose planes live in device
 * memory; ssimu2_dev receives npairs doubles, butter_norms_dev 3 doubles per pair {Qnorm,
 * 3-norm, inf-norm} (both device memory, each required when its metric is enabled).
 * max_sources[r] and max_pairs[r] bound the sources and pairs of resolution r in one call.
 * The launch sequence of a batch layout (source_res, candidate_source, input_type) is captured
 * in a CUDA graph on its first call and replayed while the layout repeats (unless
 * Vship_MultiNoGraph). With Vship_MultiAutotune the first call of a new layout times the
 * SSIMULACRA2 stats-launch knobs and keeps the fastest; choices are stored in the JSON file
 * tune_cache_path (NULL: $VSHIP_TUNE_CACHE, unset: kept in memory only) and reused by later
 * handlers. The call only enqueues device work (after waiting for the previous call's table
 * upload); calls on one handler must be ordered on one stream. */
typedef struct {
    int id;
} Vship_MultiHandler;
typedef enum {
    Vship_MultiSSIMU2 = 1,
    Vship_MultiButteraugli = 2,
    Vship_MultiFp16 = 4,
    Vship_MultiNoGraph = 8,
    Vship_MultiAutotune = 16,
    Vship_MultiButterHalfBands = 32, /* Butteraugli UHF bands as FP16 (Vship_ButterHalfBands) */
} Vship_MultiFlags;
EXPORTPREPROCESS Vship_Exception Vship_MultiInit(Vship_MultiHandler* handler, int nres, const int* widths,
                                                 const int* heights, const int* max_sources, const int* max_pairs,
                                                 int flags, int Qnorm, float intensity_multiplier,
                                                 const char* tune_cache_path);
EXPORTPREPROCESS Vship_Exception Vship_MultiFree(Vship_MultiHandler handler);
EXPORTPREPROCESS Vship_Exception Vship_MultiComputeDeviceAsync(Vship_MultiHandler handler, int nsources,
                                                               const Vship_DeviceFrame* sources,
                                                               const int* source_res, int npairs,
                                                               const Vship_DeviceFrame* candidates,
                                                               const int* candidate_source,
                                                               Vship_InputType input_type, double* ssimu2_dev,
                                                               double* butter_norms_dev, void* stream);
/* Format of Vship_InYuv frames (Vship_YuvFormat; matrix 2 resolves per resolution). */
EXPORTPREPROCESS Vship_Exception Vship_MultiSetYuvFormat(Vship_MultiHandler handler, const Vship_YuvFormat* format);
/* The launch knobs in use as JSON (same size/truncation contract as Vship_GetErrorMessage). */
EXPORTPREPROCESS int Vship_MultiKnobs(Vship_MultiHandler handler, char* out_json, int len);
EXPORTPREPROCESS uint64_t Vship_MultiDeviceBytes(int nres, const int* widths, const int* heights,
                                                 const int* max_sources, const int* max_pairs, int flags);

/* Serving runtime -- no counterpart in the reference (whose front-ends score frames in order).
 *
 * A server owns one GPU stream. Requests (one source frame scored against 1..max_batch_pairs
 * candidates, by SSIMULACRA2 or Butteraugli, at one of the resolutions given at creation) are
 * queued by Vship_ServeSubmit and return at once. A scheduler thread gathers queued requests
 * into batches in arrival order whenever fewer than two batches are on the GPU, admitting a
 * request only while the charges of the requests on the GPU stay within admission_bytes
 * (48 x width x height bytes per SSIMULACRA2 pair, 124 x width x height per Butteraugli pair).
 * Per-source device state (the SSIMULACRA2 XYB pyramid, the Butteraugli opsin and frequency
 * planes) is kept in an LRU cache of cache_bytes keyed by (metric, resolution, source_key), so
 * a source that comes back skips its own stage; source_key 0 is never cached. Results go to the
 * request's host buffer `results` (npairs scores, or 3 doubles per pair {Qnorm, 3-norm,
 * inf-norm}) before Vship_ServePoll reports the request with its latency (submit to results).
 * Frames (device planes of input_type) and `results` must stay valid until then; the candidate
 * descriptor array is copied at submit. flags: Vship_ServeFp32Candidates keeps SSIMULACRA2
 * candidate pyramids in FP32 (default: FP16 differences from the source's). */
typedef struct {
    int id;
} Vship_ServeHandler;
typedef enum { Vship_ServeSSIMU2 = 0, Vship_ServeButteraugli = 1 } Vship_ServeMetric;
#define Vship_ServeFp32Candidates 1
#define Vship_ServeButterHalfBands 2 /* Butteraugli UHF bands as FP16 (Vship_ButterHalfBands) */
typedef struct {
    uint64_t request_id;
    int metric;      /* Vship_ServeMetric */
    int resolution;  /* index into the creation's widths / heights */
    uint64_t source_key;
    Vship_DeviceFrame source;
    int npairs;
    const Vship_DeviceFrame* candidates; /* host array of npairs descriptors */
    double* results;                     /* host */
} Vship_ServeRequest;
typedef struct {
    uint64_t request_id;
    int status; /* Vship_Exception, or Vship_ServeCancelled */
    double latency_seconds;
} Vship_ServeCompletion;
EXPORTPREPROCESS Vship_Exception Vship_ServeCreate(Vship_ServeHandler* handler, int nres, const int* widths,
                                                   const int* heights, Vship_InputType input_type,
                                                   uint64_t admission_bytes, uint64_t cache_bytes,
                                                   int max_batch_pairs, int flags, int Qnorm,
                                                   float intensity_multiplier);
/* Format of Vship_InYuv frames (Vship_YuvFormat; matrix 2 resolves per resolution). Set it before
 * the first submit: cached source state is keyed by source, not by format, so once a request has
 * been submitted the call is refused with Vship_BadPointer and the format stays as it was. */
EXPORTPREPROCESS Vship_Exception Vship_ServeSetYuvFormat(Vship_ServeHandler handler, const Vship_YuvFormat* format);
/* Vship_OutOfVRAM: the request's charge alone exceeds admission_bytes. */
EXPORTPREPROCESS Vship_Exception Vship_ServeSubmit(Vship_ServeHandler handler, const Vship_ServeRequest* request);
/* Withdraws a request still waiting in the queue: it is reported at once with status
 * Vship_ServeCancelled. Vship_BadPointer when no queued request has this id (it is already on
 * the GPU, done, or unknown). */
#define Vship_ServeCancelled (-1)
EXPORTPREPROCESS Vship_Exception Vship_ServeCancel(Vship_ServeHandler handler, uint64_t request_id);
/* Up to max completions, waiting up to timeout_seconds for the first; returns how many. */
EXPORTPREPROCESS int Vship_ServePoll(Vship_ServeHandler handler, Vship_ServeCompletion* out, int max,
                                     double timeout_seconds);
/* Blocks until every submitted request has completed. */
EXPORTPREPROCESS Vship_Exception Vship_ServeDrain(Vship_ServeHandler handler);
/* Counters as JSON (same size/truncation contract as Vship_GetErrorMessage). */
EXPORTPREPROCESS int Vship_ServeStats(Vship_ServeHandler handler, char* out_json, int len);
/* Drains, stops the threads and frees everything. */
EXPORTPREPROCESS Vship_Exception Vship_ServeDestroy(Vship_ServeHandler handler);

/* Instrumentation: when enabled, every kernel launch is bracketed by CUDA events on its stream.
 * Vship_ProfileReport synchronises those events and writes a JSON object
 * {"kernel": [launches, total_ms], ...} (same size/truncation contract as
 * Vship_GetErrorMessage); a call with len > 0 also clears the records, a size query (len == 0)
 * does not. Off by default. */
EXPORTPREPROCESS void Vship_ProfileSetEnabled(int enabled);
EXPORTPREPROCESS int Vship_ProfileReport(char* out_json, int len);

/* Bytes of device memory one handler holds for a given resolution and batch size. */
EXPORTPREPROCESS uint64_t Vship_SSIMU2DeviceBytes(int width, int height, int max_pairs);

#ifdef __cplusplus
} /* extern "C" */
#endif
#endif /* VSHIP_API_HEADER */
