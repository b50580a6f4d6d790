// frame_pipeline.h -- decodes runs of frames of an opened capture on the GPU:
// field windows copied straight from the mmapped .tbc into device memory
// (runs of consecutive fields as one 2D copy; on Grace the GPU reads the
// page-cached mapping over NVLink-C2C at the rate of pinned memory, so no
// host staging copy is made), black padding fields filled on the device,
// dropout-concealed, Transform-PAL decoded and downloaded into pinned host
// chunks that decoded frames borrow. Two slots alternate so the upload of one
// batch and the download of another overlap the kernels of a third.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "capture.h"
#include "dropout_plan.h"
#include "engine.h"
#include "multi_source.h"

namespace chdg {

// Pinned host memory holding `count` decoded frames; frames borrow slices.
struct HostChunk {
    void *data = nullptr;
    size_t bytes = 0;
    ~HostChunk();
};

struct DropoutSettings {
    bool enabled = false, overcorrect = false, intra = false;
    // extra captures to conceal from (null: the primary alone)
    std::shared_ptr<const MultiSource> sources;
};

// Delivery of decoded frames: frame `first + i` lives at chunk->data + i * frame_bytes.
using Deliver = std::function<void(const std::shared_ptr<HostChunk> &chunk, int64_t first, int count)>;

class FramePipeline {
public:
    static constexpr int kEdgeFrames = 16;   // size of the first and last batch of a long run

    FramePipeline() = default;
    ~FramePipeline();
    FramePipeline(const FramePipeline &) = delete;
    FramePipeline &operator=(const FramePipeline &) = delete;

    // Returns a chd_status_t value.
    int init(const Capture *cap, const chdg_geometry &g, const chdg_config &c, bool firstFieldFirst,
             int batch_frames);
    // Changing the overcorrect / intra-field settings or the sources drops
    // the cached plans.
    void set_dropout(const DropoutSettings &d);
    // Concealment statistics of frame `frame`'s own two fields (0-based).
    FramePlan frame_stats(int64_t frame);

    // Decode frames [a, b) in batches; deliver() runs on the calling thread
    // after each batch's frames are in host memory, possibly while the next
    // batch is still on the GPU. `cancelled` is polled before each batch.
    // Stats of the frames decoded (their own dropout statistics) accumulate
    // into *stats when given.
    int decode(int64_t a, int64_t b, const Deliver &deliver, const std::function<bool()> &cancelled,
               FramePlan *stats);

    // Frame `frame`'s two fields (window order) after concealment, as the
    // decode feeds them to the transform, into host_out (2 x field samples).
    int conceal_frame(int64_t frame, uint16_t *host_out);

    size_t frame_bytes() const { return eng_.frame_bytes(); }
    Engine &engine() { return eng_; }
    int num_frames() const { return nframes_; }

private:
    // Enqueue the window fields of frames [w0, w1) into dwin_[slot] on copy_.
    int upload_window(int slot, int64_t w0, int64_t w1);
    // upload_window plus the frames' dropout plans and the extra-source
    // fields they read; nplan = frames with a plan.
    int upload_batch(int slot, int64_t w0, int64_t w1, int &nplan);
    const FramePlan &plan_for(int64_t frame);   // cached, window frame (0-based)
    // the concealment's luma filter: PAL's, or the NTSC taps that NTSC and
    // PAL-M use (dropout_corrector.cpp:498-506)
    bool ntsc_luma_taps() const { return cap_->vp().system == SYS_NTSC || cap_->vp().system == SYS_PAL_M; }
    // A pinned chunk of at least `bytes`, reused once every frame borrowing
    // from it has been freed.
    std::shared_ptr<HostChunk> take_chunk(size_t bytes);

    const Capture *cap_ = nullptr;
    Engine eng_;
    bool ffirst_ = true;
    int nframes_ = 0;
    int batch_ = 32;
    int lb_ = 0, la_ = 0;
    size_t flen_ = 0;
    long long dstride_ = 0;
    DropoutSettings drop_;
    cudaStream_t comp_ = nullptr, copy_ = nullptr, d2h_ = nullptr;   // kernels, uploads, downloads
    uint16_t *dwin_[2] = {nullptr, nullptr};
    void *dout_[2] = {nullptr, nullptr};
    cudaEvent_t ev_h2d_[2] = {}, ev_comp_[2] = {}, ev_d2h_[2] = {};
    // dropout plans uploaded per slot
    DropOp *h_ops_[2] = {nullptr, nullptr}, *d_ops_[2] = {nullptr, nullptr};
    int *h_idx_[2] = {nullptr, nullptr}, *d_idx_[2] = {nullptr, nullptr};   // frames then op_begin
    size_t ops_cap_ = 0, idx_cap_ = 0;
    // extra captures' fields that a batch's plans read replacement lines from
    uint16_t *dext_[2] = {nullptr, nullptr};
    size_t ext_cap_ = 0;   // fields per slot
    std::map<int64_t, FramePlan> plans_;
    std::vector<std::shared_ptr<HostChunk>> chunks_;
};

}  // namespace chdg
