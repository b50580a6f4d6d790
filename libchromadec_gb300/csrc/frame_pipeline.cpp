// frame_pipeline.cpp -- see frame_pipeline.h.
#include "frame_pipeline.h"

#include <algorithm>
#include <cstring>
#include <string>

#include <chromadec/errors.h>

#include "error_state.h"

namespace chdg {

int dropout_apply(uint16_t *fields, long long field_stride, int fw, const int *d_frames, const DropOp *d_ops,
                  const int *d_op_begin, int nframes, const uint16_t *extras, bool ntsc_taps, cudaStream_t s);
int fill_fields(uint16_t *fields, long long field_stride, long long field_len, int nfields, uint16_t value,
                cudaStream_t s);
int fill_samples(uint16_t *p, long long n, uint16_t value, cudaStream_t s);

namespace {

int cuda_status(const char *what, cudaError_t e)
{
    chd::detail::set_last_error(std::string("chromadec_gb300: ") + what + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? CHD_E_OOM : CHD_E_INTERNAL;
}

}  // namespace

HostChunk::~HostChunk()
{
    if (data != nullptr) cudaFreeHost(data);
}

FramePipeline::~FramePipeline()
{
    if (comp_) cudaStreamSynchronize(comp_);
    if (copy_) cudaStreamSynchronize(copy_);
    if (d2h_) cudaStreamSynchronize(d2h_);
    chunks_.clear();
    for (int i = 0; i < 2; i++) {
        if (dwin_[i]) cudaFree(dwin_[i]);
        if (dout_[i]) cudaFree(dout_[i]);
        if (h_ops_[i]) cudaFreeHost(h_ops_[i]);
        if (d_ops_[i]) cudaFree(d_ops_[i]);
        if (h_idx_[i]) cudaFreeHost(h_idx_[i]);
        if (d_idx_[i]) cudaFree(d_idx_[i]);
        if (dext_[i]) cudaFree(dext_[i]);
        if (ev_h2d_[i]) cudaEventDestroy(ev_h2d_[i]);
        if (ev_comp_[i]) cudaEventDestroy(ev_comp_[i]);
        if (ev_d2h_[i]) cudaEventDestroy(ev_d2h_[i]);
    }
    if (comp_) cudaStreamDestroy(comp_);
    if (copy_) cudaStreamDestroy(copy_);
    if (d2h_) cudaStreamDestroy(d2h_);
}

int FramePipeline::init(const Capture *cap, const chdg_geometry &g, const chdg_config &c, bool firstFieldFirst,
                        int batch_frames)
{
    cap_ = cap;
    ffirst_ = firstFieldFirst;
    nframes_ = cap->numFrames(firstFieldFirst);
    batch_ = std::max(1, batch_frames);
    if (const int rc = eng_.init(g, c); rc != 0) return rc == CHDG_E_UNSUPPORTED ? CHD_E_UNSUPPORTED : CHD_E_INVALID_ARG;
    eng_.set_max_batch_frames(batch_);
    lb_ = eng_.look_behind();
    la_ = eng_.look_ahead();
    flen_ = cap->fieldLen();
    dstride_ = (long long)((flen_ + 63) & ~(size_t)63);
    const size_t winFields = (size_t)2 * (batch_ + lb_ + la_) + 1;   // +1: tiles read a few samples past a field
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&comp_, cudaStreamNonBlocking)) != cudaSuccess) return cuda_status("stream", e);
    if ((e = cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking)) != cudaSuccess) return cuda_status("stream", e);
    if ((e = cudaStreamCreateWithFlags(&d2h_, cudaStreamNonBlocking)) != cudaSuccess) return cuda_status("stream", e);
    for (int i = 0; i < 2; i++) {
        if ((e = cudaMalloc(&dwin_[i], winFields * dstride_ * 2)) != cudaSuccess) return cuda_status("window", e);
        cudaMemset(dwin_[i], 0, winFields * dstride_ * 2);
        if ((e = cudaMalloc(&dout_[i], eng_.frame_bytes() * (size_t)batch_)) != cudaSuccess)
            return cuda_status("frames", e);
        cudaEventCreateWithFlags(&ev_h2d_[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_comp_[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ev_d2h_[i], cudaEventDisableTiming);
    }
    return CHD_OK;
}

void FramePipeline::set_dropout(const DropoutSettings &d)
{
    if (d.overcorrect != drop_.overcorrect || d.intra != drop_.intra || d.sources != drop_.sources) plans_.clear();
    drop_ = d;
}

FramePlan FramePipeline::frame_stats(int64_t frame)
{
    FramePlan s;
    if (!drop_.enabled) return s;
    const FramePlan &p = plan_for(frame);
    s.corrected = p.corrected;
    s.failed = p.failed;
    s.totalDistance = p.totalDistance;
    return s;
}

std::shared_ptr<HostChunk> FramePipeline::take_chunk(size_t bytes)
{
    // Every chunk holds a full batch, so any free chunk serves any batch and
    // the pool settles after the first call (a pinned allocation costs
    // milliseconds; one made mid-run would stall the pipeline).
    bytes = std::max(bytes, eng_.frame_bytes() * (size_t)batch_);
    // A chunk only this pool still references is free for reuse.
    for (auto &c : chunks_)
        if (c.use_count() == 1 && c->bytes >= bytes) return c;
    size_t idle = 0;
    for (auto it = chunks_.begin(); it != chunks_.end();) {
        if (it->use_count() == 1 && ++idle > 4) it = chunks_.erase(it);
        else ++it;
    }
    auto c = std::make_shared<HostChunk>();
    if (cudaMallocHost(&c->data, bytes) != cudaSuccess) {
        c->data = nullptr;
        return nullptr;
    }
    c->bytes = bytes;
    chunks_.push_back(c);
    return c;
}

const FramePlan &FramePipeline::plan_for(int64_t frame)
{
    auto it = plans_.find(frame);
    if (it != plans_.end()) return it->second;
    WindowField wf[2];
    cap_->windowFrame((int)frame + 1, ffirst_, wf);
    FramePlan plan;
    // A padding frame carries frame 1's dropouts but none of its picture.
    if (!wf[0].isPadding && !wf[1].isPadding) {
        FieldMeta m0 = cap_->field(wf[0].fieldNumber), m1 = cap_->field(wf[1].fieldNumber);
        if (second_field_shifted(cap_->vp())) m1 = shift_dropouts(m1);
        std::vector<ExtraFrame> extras;
        if (drop_.sources && !(m0.dropouts.empty() && m1.dropouts.empty())) {
            // The extras that hold this window frame, matched by VBI disc frame
            // or positionally, each read by its own pairing
            // (src/abi/c_api_decoder.cpp:245-282)
            const MultiSource &ms = *drop_.sources;
            for (size_t i = 0; i < ms.extras.size(); i++) {
                const AlignedSource &x = ms.extras[i];
                const int exFrame = ms.alignment.frameFor((int)frame + 1, (int)i + 1);
                if (exFrame < 1 || exFrame > x.cap->numFrames(x.firstFieldFirst)) continue;
                const int a = x.cap->fieldNumber(exFrame, 1, x.firstFieldFirst);
                const int b = x.cap->fieldNumber(exFrame, 2, x.firstFieldFirst);
                ExtraFrame ef;
                ef.vp = x.cap->vp();
                ef.first = x.cap->field(a);
                ef.second = x.cap->field(b);
                ef.quality = (ef.first.bPSNR + ef.second.bPSNR) / 2.0;
                const bool sh = second_field_shifted(ef.vp);
                if (sh) ef.second = shift_dropouts(ef.second);
                const uint16_t black = (uint16_t)ef.vp.black16bIre;
                ef.firstField = {x.cap, a, false, black};
                ef.secondField = {x.cap, b, sh, black};
                extras.push_back(std::move(ef));
            }
        }
        plan = plan_frame(cap_->vp(), m0, m1, drop_.overcorrect, drop_.intra, extras);
    }
    return plans_.emplace(frame, std::move(plan)).first->second;
}

int FramePipeline::upload_window(int slot, int64_t w0, int64_t w1)
{
    const int nf = (int)(2 * (w1 - w0));
    const uint16_t black = (uint16_t)cap_->vp().black16bIre;
    const size_t fbytes = flen_ * 2;
    // window field k comes from capture field src[k] (1-based, 0 = black)
    std::vector<int> src((size_t)std::max(nf, 0));
    for (int k = 0; k < nf; k += 2) {
        WindowField wf[2];
        cap_->windowFrame((int)(w0 + k / 2) + 1, ffirst_, wf);
        src[k] = wf[0].source;
        src[k + 1] = wf[1].source;
    }
    cudaError_t e;
    const bool shifted = second_field_shifted(cap_->vp());
    for (int k = 0; k < nf;) {
        int n = 1;
        if (shifted && (k & 1) && src[k] != 0) {
            // shiftSecondField: samples 2.. of the field, then 2 black
            uint16_t *dst = dwin_[slot] + (size_t)k * dstride_;
            if ((e = cudaMemcpyAsync(dst, cap_->fieldData(src[k]) + 2, fbytes - 4, cudaMemcpyHostToDevice, copy_)) !=
                cudaSuccess)
                return cuda_status("H2D", e);
            if (fill_samples(dst + flen_ - 2, 2, black, copy_) != 0) return cuda_status("black tail", cudaGetLastError());
            k += 1;
            continue;
        }
        if (src[k] == 0) {
            while (k + n < nf && src[k + n] == 0) n++;
            if (fill_fields(dwin_[slot] + (size_t)k * dstride_, dstride_, (long long)flen_, n, black, copy_) != 0)
                return cuda_status("black fields", cudaGetLastError());
        } else {
            // a run of consecutive fields (slot-0 fields only when slot 1 is shifted)
            while (k + n < nf && src[k + n] == src[k] + n && !(shifted && ((k + n) & 1))) n++;
            if ((e = cudaMemcpy2DAsync(dwin_[slot] + (size_t)k * dstride_, (size_t)dstride_ * 2,
                                       cap_->fieldData(src[k]), fbytes, fbytes, (size_t)n, cudaMemcpyHostToDevice,
                                       copy_)) != cudaSuccess)
                return cuda_status("H2D", e);
        }
        k += n;
    }
    return CHD_OK;
}

// The window fields of frames [w0, w1) into slot `slot`, with the dropout
// plans of those frames and the extra-source fields they read, all on copy_.
// The slot's plan buffers must be idle (their last upload complete).
int FramePipeline::upload_batch(int slot, int64_t w0, int64_t w1, int &nplan)
{
    cudaError_t e;
    nplan = 0;
    std::vector<ExtraField> extFields;   // the batch's extra-source fields, in buffer order
    size_t nops = 0;
    std::vector<const FramePlan *> plans;
    std::vector<int> planFrames;
    if (drop_.enabled) {
        for (int64_t w = w0; w < w1; w++) {
            const FramePlan &p = plan_for(w);
            if (!p.ops.empty()) {
                plans.push_back(&p);
                planFrames.push_back((int)(2 * (w - w0)));
                nops += p.ops.size();
            }
        }
        nplan = (int)plans.size();
        if (nops > ops_cap_ || (size_t)(2 * nplan + 1) > idx_cap_) {
            cudaStreamSynchronize(comp_);
            cudaStreamSynchronize(copy_);
            cudaStreamSynchronize(d2h_);
            for (int s = 0; s < 2; s++) {
                if (h_ops_[s]) cudaFreeHost(h_ops_[s]);
                if (d_ops_[s]) cudaFree(d_ops_[s]);
                if (h_idx_[s]) cudaFreeHost(h_idx_[s]);
                if (d_idx_[s]) cudaFree(d_idx_[s]);
                h_ops_[s] = d_ops_[s] = nullptr;
                h_idx_[s] = d_idx_[s] = nullptr;
            }
            ops_cap_ = std::max<size_t>(nops * 2, 1024);
            idx_cap_ = std::max<size_t>((size_t)(2 * nplan + 1) * 2, 256);
            for (int s = 0; s < 2; s++) {
                if (cudaMallocHost(&h_ops_[s], ops_cap_ * sizeof(DropOp)) != cudaSuccess ||
                    cudaMalloc(&d_ops_[s], ops_cap_ * sizeof(DropOp)) != cudaSuccess ||
                    cudaMallocHost(&h_idx_[s], idx_cap_ * sizeof(int)) != cudaSuccess ||
                    cudaMalloc(&d_idx_[s], idx_cap_ * sizeof(int)) != cudaSuccess)
                    return cuda_status("dropout plan buffers", cudaErrorMemoryAllocation);
            }
        }
        size_t o = 0;
        extFields.clear();
        std::map<std::pair<const Capture *, int32_t>, int32_t> extIndex;
        auto ext_slot = [&](const FramePlan &pl, int32_t k) -> int32_t {
            if (k < 0) return -1;
            const ExtraField &xf = pl.extras[(size_t)k];
            auto it = extIndex.find({xf.cap, xf.seq});
            if (it != extIndex.end()) return it->second;
            const int32_t idx = (int32_t)extFields.size();
            extFields.push_back(xf);
            extIndex.emplace(std::make_pair(xf.cap, xf.seq), idx);
            return idx;
        };
        for (int p = 0; p < nplan; p++) {
            h_idx_[slot][p] = planFrames[p];
            h_idx_[slot][nplan + p] = (int)o;
            for (const DropOp &op : plans[p]->ops) {
                DropOp d = op;
                d.srcExtra = ext_slot(*plans[p], op.srcExtra);
                d.chrExtra = (op.mode == 2) ? ext_slot(*plans[p], op.chrExtra) : -1;
                h_ops_[slot][o++] = d;
            }
        }
        h_idx_[slot][2 * nplan] = (int)o;
    }
    if (const int rc = upload_window(slot, w0, w1); rc != CHD_OK) return rc;
    if (!extFields.empty()) {
        if (extFields.size() > ext_cap_) {
            cudaStreamSynchronize(comp_);
            cudaStreamSynchronize(copy_);
            for (int s = 0; s < 2; s++) {
                if (dext_[s]) cudaFree(dext_[s]);
                dext_[s] = nullptr;
            }
            ext_cap_ = std::max<size_t>(extFields.size() * 2, 8);
            for (int s = 0; s < 2; s++)
                if ((e = cudaMalloc(&dext_[s], ext_cap_ * (size_t)dstride_ * 2)) != cudaSuccess)
                    return cuda_status("extra source fields", e);
        }
        const size_t fbytes = flen_ * 2;
        for (size_t k = 0; k < extFields.size(); k++) {
            const ExtraField &xf = extFields[k];
            const uint16_t *src = xf.cap->fieldData(xf.seq);
            if (src == nullptr) {
                chd::detail::set_last_error("chromadec_gb300: extra source field " + std::to_string(xf.seq) +
                                            " is outside its .tbc file");
                return CHD_E_INTERNAL;
            }
            uint16_t *dst = dext_[slot] + k * (size_t)dstride_;
            if (xf.shifted) {   // shiftSecondField (src/decoders/source_field.cpp:51-57)
                if ((e = cudaMemcpyAsync(dst, src + 2, fbytes - 4, cudaMemcpyHostToDevice, copy_)) != cudaSuccess)
                    return cuda_status("H2D", e);
                if (fill_samples(dst + flen_ - 2, 2, xf.black, copy_) != 0)
                    return cuda_status("black tail", cudaGetLastError());
            } else if ((e = cudaMemcpyAsync(dst, src, fbytes, cudaMemcpyHostToDevice, copy_)) != cudaSuccess) {
                return cuda_status("H2D", e);
            }
        }
    }
    if (nplan > 0) {
        cudaMemcpyAsync(d_ops_[slot], h_ops_[slot], nops * sizeof(DropOp), cudaMemcpyHostToDevice, copy_);
        cudaMemcpyAsync(d_idx_[slot], h_idx_[slot], (2 * nplan + 1) * sizeof(int), cudaMemcpyHostToDevice, copy_);
    }
    return CHD_OK;
}

// Frame `frame`'s two window fields after concealment, exactly as the
// decode would hand them to the transform: the window of that one frame is
// uploaded into slot 0, its plan applied by the concealment kernel, and the
// two fields copied back (window order: slot 0 first).
int FramePipeline::conceal_frame(int64_t frame, uint16_t *host_out)
{
    if (frame < 0 || frame >= nframes_) return CHD_E_OUT_OF_RANGE;
    cudaError_t e;
    for (cudaStream_t s : {comp_, copy_, d2h_})
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status("sync", e);
    int nplan = 0;
    if (const int rc = upload_batch(0, frame, frame + 1, nplan); rc != CHD_OK) return rc;
    if (nplan > 0 && dropout_apply(dwin_[0], dstride_, cap_->vp().fieldWidth, d_idx_[0], d_ops_[0], d_idx_[0] + nplan,
                                   nplan, dext_[0], ntsc_luma_taps(), copy_) != 0)
        return cuda_status("dropout kernel", cudaGetLastError());
    if ((e = cudaMemcpy2DAsync(host_out, flen_ * 2, dwin_[0], (size_t)dstride_ * 2, flen_ * 2, 2,
                               cudaMemcpyDeviceToHost, copy_)) != cudaSuccess)
        return cuda_status("D2H", e);
    if ((e = cudaStreamSynchronize(copy_)) != cudaSuccess) return cuda_status("sync", e);
    return CHD_OK;
}

int FramePipeline::decode(int64_t a, int64_t b, const Deliver &deliver, const std::function<bool()> &cancelled,
                          FramePlan *stats)
{
    struct Pending {
        std::shared_ptr<HostChunk> out;
        int64_t first = 0;
        int count = 0;
        int slot = 0;
    };
    Pending prev, pendingOut;
    bool havePrev = false;
    const size_t fb = eng_.frame_bytes();
    cudaError_t e;
    // Batch boundaries: full batches in the middle, short ones at both ends.
    const std::vector<std::pair<int64_t, int64_t>> batches = edge_batches(a, b, batch_, kEdgeFrames);
    // Two stages per batch on two window slots: the upload (window fields,
    // dropout plans, extra-source fields) on copy_, and the kernels plus the
    // download on comp_ / d2h_. The next batch's upload is issued before the
    // host waits for the previous batch's frames, so the host's time in the
    // (blocking, pageable) field copies overlaps the GPU's work.
    std::vector<int> nplans(batches.size(), 0);
    auto stage_upload = [&](size_t bi) -> int {
        const int64_t c = batches[bi].first, ce = batches[bi].second;
        const int slot = (int)(bi & 1);
        const int64_t w0 = std::max<int64_t>(0, c - lb_);
        const int64_t w1 = std::min<int64_t>(nframes_, ce + la_);
        // bound the plan cache; plans behind the window are not needed again
        // by this run (references into the map stay valid: only others go)
        if (plans_.size() > 4096) plans_.erase(plans_.begin(), plans_.lower_bound(w0));
        if (bi >= 2) {
            // the window of this slot was last read by batch bi-2's kernels,
            // and its plan buffers were last uploaded for batch bi-2
            cudaStreamWaitEvent(copy_, ev_comp_[slot], 0);
            if ((e = cudaEventSynchronize(ev_h2d_[slot])) != cudaSuccess) return cuda_status("sync", e);
        }
        int nplan = 0;
        if (const int rc = upload_batch(slot, w0, w1, nplan); rc != CHD_OK) return rc;
        cudaEventRecord(ev_h2d_[slot], copy_);
        nplans[bi] = nplan;
        return CHD_OK;
    };
    auto stage_compute = [&](size_t bi) -> int {
        const int64_t c = batches[bi].first, ce = batches[bi].second;
        const int slot = (int)(bi & 1);
        const int64_t w0 = std::max<int64_t>(0, c - lb_);
        const int nplan = nplans[bi];
        cudaStreamWaitEvent(comp_, ev_h2d_[slot], 0);
        if (bi >= 2) cudaStreamWaitEvent(comp_, ev_d2h_[slot], 0);   // output slot drained
        if (nplan > 0 &&
            dropout_apply(dwin_[slot], dstride_, cap_->vp().fieldWidth, d_idx_[slot], d_ops_[slot],
                          d_idx_[slot] + nplan, nplan, dext_[slot], ntsc_luma_taps(), comp_) != 0)
            return cuda_status("dropout kernel", cudaGetLastError());
        if (const int rc = eng_.decode(dwin_[slot], dstride_, (int)(2 * w0), 2 * nframes_, (int)c, (int)ce,
                                       dout_[slot], comp_);
            rc != 0)
            return CHD_E_INTERNAL;
        cudaEventRecord(ev_comp_[slot], comp_);
        auto chunk = take_chunk(fb * (size_t)(ce - c));
        if (!chunk) return cuda_status("pinned frames", cudaErrorMemoryAllocation);
        cudaStreamWaitEvent(d2h_, ev_comp_[slot], 0);
        if ((e = cudaMemcpyAsync(chunk->data, dout_[slot], fb * (size_t)(ce - c), cudaMemcpyDeviceToHost, d2h_)) !=
            cudaSuccess)
            return cuda_status("D2H", e);
        cudaEventRecord(ev_d2h_[slot], d2h_);
        if (stats != nullptr && drop_.enabled) {
            for (int64_t k = c; k < ce; k++) {
                const FramePlan &p = plan_for(k);
                stats->corrected += p.corrected;
                stats->failed += p.failed;
                stats->totalDistance += p.totalDistance;
            }
        }
        pendingOut = {chunk, c, (int)(ce - c), slot};
        return CHD_OK;
    };
    if (!batches.empty() && !(cancelled && cancelled())) {
        if (const int rc = stage_upload(0); rc != CHD_OK) return rc;
    }
    for (size_t bi = 0; bi < batches.size(); bi++) {
        if (cancelled && cancelled()) break;
        if (const int rc = stage_compute(bi); rc != CHD_OK) return rc;
        // the next batch's fields go up while this batch computes
        if (bi + 1 < batches.size() && !(cancelled && cancelled()))
            if (const int rc = stage_upload(bi + 1); rc != CHD_OK) return rc;
        if (havePrev) {
            if ((e = cudaEventSynchronize(ev_d2h_[prev.slot])) != cudaSuccess) return cuda_status("sync", e);
            deliver(prev.out, prev.first, prev.count);
        }
        prev = pendingOut;
        havePrev = true;
    }
    if (havePrev) {
        if ((e = cudaEventSynchronize(ev_d2h_[prev.slot])) != cudaSuccess) return cuda_status("sync", e);
        deliver(prev.out, prev.first, prev.count);
    }
    return CHD_OK;
}

}  // namespace chdg
