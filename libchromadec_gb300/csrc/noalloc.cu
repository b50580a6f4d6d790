// noalloc.cu -- Transform-PAL 3D decode that allocates no device memory.
//
// The regular entry points size their chroma scratch on demand with
// cudaMalloc. This variant runs the same 3D transform and demodulator
// kernels with their scratch in file-scope __device__ arrays instead, for
// callers that cannot allocate device memory on the decode path: hosts whose
// device memory belongs to their own allocator or budget (a framework's
// caching allocator, a media server with a fixed pool), and latency-critical
// playback loops where cudaMalloc's implicit device-wide synchronisation
// would stall other streams.
//
// Static arrays, held by every GPU that loads the library until the process
// exits (sizes at the default 948x576 active picture, 4,440 tile positions):
//   chroma scratch   4 overlap planes x 16 fields x 288 x 948 FP32   69.9 MB
//   decision records 133,200 x 80 B (every kx group of an 8-frame call) 10.7 MB
//   work-item list   2 x 133,200 x 4 B                                  1.1 MB
//   per-bin table    768 x 3 FP32, two counters
// in all 81.6 MB. Calls with more than 8 frames, or with a picture whose
// planes or tile grid do not fit these arrays, are rejected.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/chromadec_gb300.h"
#include "engine.h"
#include "error_state.h"
#include "tpal_kernels.h"

namespace {

constexpr int kStaticMaxFrames = 8;
// 4 overlap planes x 2 fields per frame x 288 active field rows x 948 samples
constexpr size_t kStaticScratchFloats = (size_t)4 * 2 * kStaticMaxFrames * 288 * 948;
// Guard-band decision records: every kx group of every step of an 8-frame
// call over the default picture's 4,440 tile positions (one walk chunk).
constexpr int kStaticTiles = 120 * 37;
constexpr unsigned long long kStaticRecords = tpal::tp3_unc_capacity(kStaticTiles, kStaticMaxFrames, 1);
static_assert(kStaticRecords == 133200ull, "records of an 8-frame call over 4,440 tile positions");
static_assert(sizeof(tpal::UncRecord) == 80, "decision record layout");

// Shared by every call on a device; holds the previous call's chroma planes.
static __device__ __align__(256) float g_static_scratch[kStaticScratchFloats];
static __device__ __align__(256) float g_static_thresholds[3 * 768];
static __device__ __align__(256) tpal::UncRecord g_static_records[kStaticRecords];
static __device__ __align__(256) unsigned g_static_items[2 * kStaticRecords];
static __device__ __align__(256) unsigned g_static_counters[2];

struct DeviceSymbols {
    float *scratch = nullptr;
    float *thresholds = nullptr;
    void *records = nullptr;
    unsigned *items = nullptr, *counters = nullptr;
    cudaError_t status = cudaSuccess;
};
constexpr int kMaxDevices = 64;
static DeviceSymbols g_symbols[kMaxDevices];
static std::once_flag g_symbols_once[kMaxDevices];

// Once per device, with that device current: the device addresses of the
// static arrays (in host code the symbols name host-side stand-ins, not
// device memory). std::call_once makes concurrent first calls on one device
// wait for a single resolution and see all of its results.
int resolve_symbols(int device, DeviceSymbols &out)
{
    if (device < 0 || device >= kMaxDevices) {
        chd::detail::set_last_error("chdg_decode_device_static: device index out of range");
        return CHDG_E_INVALID_ARG;
    }
    std::call_once(g_symbols_once[device], [device]() {
        DeviceSymbols d;
        void *p = nullptr, *q = nullptr, *r = nullptr, *f = nullptr, *c = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_static_thresholds);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&r, g_static_records);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&f, g_static_items);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&c, g_static_counters);
        d.status = e;
        if (e == cudaSuccess) {
            d.scratch = static_cast<float *>(p);
            d.thresholds = static_cast<float *>(q);
            d.records = r;
            d.items = static_cast<unsigned *>(f);
            d.counters = static_cast<unsigned *>(c);
        }
        g_symbols[device] = d;
    });
    const DeviceSymbols &d = g_symbols[device];
    if (d.status != cudaSuccess) {
        chd::detail::set_last_error(std::string("chdg_decode_device_static: cudaGetSymbolAddress: ") +
                                    cudaGetErrorString(d.status));
        return CHDG_E_CUDA;
    }
    out = d;
    return 0;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" int chdg_decode_device_static(const chdg_geometry *g, const chdg_config *c, const uint16_t *d_fields,
                                         int64_t field_stride, int32_t nfields, int32_t frame_begin,
                                         int32_t frame_end, void *d_out, void *stream)
{
    if (g == nullptr || c == nullptr) {
        chd::detail::set_last_error("chdg_decode_device_static: null geometry or config");
        return CHDG_E_INVALID_ARG;
    }
    if (frame_begin < 0 || frame_end < frame_begin) {
        chd::detail::set_last_error("chdg_decode_device_static: frame range must satisfy 0 <= frame_begin <= frame_end");
        return CHDG_E_INVALID_ARG;
    }
    const int64_t nframes = (int64_t)frame_end - (int64_t)frame_begin;
    if (nframes > kStaticMaxFrames) {
        chd::detail::set_last_error("chdg_decode_device_static: at most " + std::to_string(kStaticMaxFrames) +
                                    " frames per call (the static chroma scratch holds " +
                                    std::to_string(kStaticMaxFrames) + " frames)");
        return CHDG_E_INVALID_ARG;
    }
    if (chdg::Engine::scratch_floats_for(*g, (int)nframes) > kStaticScratchFloats) {
        chd::detail::set_last_error("chdg_decode_device_static: active picture too large for the static scratch");
        return CHDG_E_INVALID_ARG;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) {
        chd::detail::set_last_error(std::string("chdg_decode_device_static: cudaGetDevice: ") + cudaGetErrorString(e));
        return CHDG_E_CUDA;
    }
    DeviceSymbols sym;
    if (const int rc = resolve_symbols(device, sym); rc != 0) return rc;
    chdg::Engine eng;
    int rc = eng.init_static(*g, *c, sym.thresholds, (cudaStream_t)stream);
    eng.set_static_decisions(sym.records, sym.items, kStaticRecords, sym.counters);
    // Every chroma sample the demodulator reads is written by the transform
    // in the same call, so the scratch needs no clearing; the decision
    // counters are zeroed on the stream before each transform.
    if (rc == 0)
        rc = eng.decode_scratch(d_fields, field_stride, nfields, frame_begin, frame_end, d_out, sym.scratch,
                                kStaticScratchFloats, (cudaStream_t)stream);
    eng.forget_static();
    return rc;
}
#pragma GCC visibility pop
