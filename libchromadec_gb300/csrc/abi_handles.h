// abi_handles.h -- what the opaque chd_* handles hold in this library.
//
// chd_video owns an opened capture (mmapped .tbc + parsed sidecar) and the
// extra captures of the same disc that multi-source concealment reads.
// chd_decoder stashes options until commit (the reference's two-phase
// lifecycle, src/abi/handles.h:76-200), then owns the GPU frame pipelines:
// one for chd_decode_frame, which decodes ahead in batches while requests
// run sequentially, and a pool that chd_decode_frames_async calls draw from
// so that concurrent or re-entrant calls never share one.
// chd_frame borrows its pixels from a pinned host chunk shared with the
// other frames of its batch; the chunk goes back to its pipeline when the
// last of them is freed.
#pragma once

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <chromadec/chromadec.h>

#include "capture.h"
#include "dropout_plan.h"
#include "frame_pipeline.h"
#include "multi_source.h"

#define CHD_API extern "C" __attribute__((visibility("default")))

namespace chdg {

enum class OptType { F64, I32, Bool, Str };

// registry::optionApplies (src/decoders/registry.cpp:113-171).
bool option_applies(chd_decoder_kind_t kind, const std::string &name, OptType type);

struct OptionMaps {
    std::unordered_map<std::string, double> f64;
    std::unordered_map<std::string, int32_t> i32;
    std::unordered_map<std::string, bool> boolean;
    std::unordered_map<std::string, std::string> str;
};

// A decoded frame waiting in the decode-ahead cache.
struct CachedFrame {
    std::shared_ptr<HostChunk> chunk;
    size_t offset = 0;
    FramePlan stats;
    uint64_t revision = 0;
};

}  // namespace chdg

struct chd_video {
    chdg::Capture cap;
    // chd_video_add_extra_source_*: composite extras (and a Y/C extra's
    // luma), plus the chroma planes of Y/C extras, kept open for their
    // lifetime; frozen by the first decode with concealment on
    // (src/abi/handles.h:68-73).
    std::vector<std::unique_ptr<chdg::Capture>> extras, chromaExtras;
    std::atomic<bool> extrasFrozen{false};
};

struct chd_decoder {
    chd_video_t *video = nullptr;   // not owned
    chd_decoder_kind_t kind = CHD_DEC_AUTO;
    chdg::OptionMaps options;

    bool dropoutOptsSet = false;
    chd_dropout_opts_t dropoutOpts{};
    std::atomic<uint64_t> dropoutRevision{1};
    std::mutex statsMutex;
    chd_dropout_stats_t lastDropoutStats{};

    bool committed = false;
    chd_decoder_kind_t resolvedKind = CHD_DEC_AUTO;
    bool reverseFieldOrder = false;
    chd_pixel_format_t outputPixelFormat = CHD_PIXEL_YUV444P16;
    int32_t threadCount = 0;
    int device = 0;
    chdg_geometry geom{};
    chdg_config cfg{};
    std::vector<double> thresholds;
    chdg::OutputFraming framing{};
    int32_t outWidth = 0, outHeight = 0;
    int64_t numFrames = 0;

    bool firstFieldFirst() const { return video->cap.isFirstFieldFirst() != reverseFieldOrder; }

    // chd_decode_frame: one pipeline plus the frames it decoded ahead.
    std::mutex syncMutex;
    std::unique_ptr<chdg::FramePipeline> syncPipe;
    std::map<int64_t, chdg::CachedFrame> ahead;
    int64_t lastIndex = -2;

    // chd_decode_frames_async: idle pipelines.
    std::mutex poolMutex;
    std::vector<std::unique_ptr<chdg::FramePipeline>> pool;

    // The extras' alignment, built on the first decode with concealment on.
    std::mutex sourcesMutex;
    std::shared_ptr<const chdg::MultiSource> multiSource;
};

struct chd_frame {
    chd_frame_info_t info{};
    chd_pixel_format_t format = CHD_PIXEL_YUV444P16;
    int32_t width = 0, height = 0;
    std::shared_ptr<chdg::HostChunk> chunk;   // decoded frames: borrowed slice
    const void *pixels = nullptr;              // [Y | Cb | Cr] planes, or the mask plane
    std::vector<uint16_t> mask16;              // dropout masks own their plane
    std::vector<float> maskf;
};

struct chd_cancel {
    std::atomic<bool> requested{false};
};

struct chd_nn_model {
    int unused;
};

namespace chdg {

// Builds a pipeline for the committed decoder on its device; returns a
// chd_status_t and sets the last error on failure.
int make_pipeline(chd_decoder_t *d, std::unique_ptr<FramePipeline> &out, int batch_frames);
// A frame handle for `count` frames' chunk slice `index`.
chd_frame_t *make_frame(chd_decoder_t *d, const std::shared_ptr<HostChunk> &chunk, size_t offset, int64_t index);

}  // namespace chdg
