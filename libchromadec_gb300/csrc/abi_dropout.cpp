// abi_dropout.cpp -- dropout options, statistics, spans and masks of the
// chd_* ABI (include/chromadec/dropout.h; reference:
// src/abi/c_api_dropout.cpp and src/abi/c_api_dropout_detect.cpp). Spans
// come from the capture's metadata mapped into the committed output framing
// (dropout_plan.cpp); masks are rasterised from them on the GPU.
#include <cstdlib>
#include <cstring>

#include <cuda_runtime.h>

#include "abi_handles.h"
#include "error_state.h"

namespace chdg {
int mask_raster(void *d_plane, bool is_float, int width, int height, const Span *d_spans, int nspans, cudaStream_t s);
}

using namespace chdg;

namespace {

chd_status_t fail(chd_status_t s, const std::string &msg)
{
    chd::detail::set_last_error(msg);
    return s;
}

bool valid_mode(chd_dropout_detect_mode_t m) { return m == CHD_DROPOUT_DETECTED || m == CHD_DROPOUT_OVERCORRECT; }

// collectSpans (c_api_dropout_detect.cpp:134-179): the frame's two fields,
// no look-behind or look-ahead.
chd_status_t collect(const chd_decoder_t *d, int64_t frame, chd_dropout_detect_mode_t mode, std::vector<Span> &spans)
{
    if (frame < 0 || frame >= d->numFrames)
        return fail(CHD_E_OUT_OF_RANGE, "chromadec dropout query: frame_index out of range");
    WindowField wf[2];
    d->video->cap.windowFrame((int)frame + 1, d->firstFieldFirst(), wf);
    const FieldMeta &m0 = d->video->cap.field(wf[0].fieldNumber);
    FieldMeta m1 = d->video->cap.field(wf[1].fieldNumber);
    // the spans of the fields as loaded: a shifted second field's dropouts moved too
    if (second_field_shifted(d->video->cap.vp())) m1 = shift_dropouts(m1);
    spans = frame_spans(d->framing, m0, wf[0].isFirstField, m1, wf[1].isFirstField, mode == CHD_DROPOUT_OVERCORRECT);
    return CHD_OK;
}

// maskFormatFor (c_api_dropout_detect.cpp:70-82)
bool mask_is_float(chd_pixel_format_t committed)
{
    return committed == CHD_PIXEL_GRAYS || committed == CHD_PIXEL_YUV444PS || committed == CHD_PIXEL_RGBS ||
           committed == CHD_PIXEL_YUV440PS;
}

chd_status_t cuda_fail(const char *what, cudaError_t e)
{
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? CHD_E_OOM : CHD_E_INTERNAL,
                std::string("chd_decode_dropout_mask: ") + what + ": " + cudaGetErrorString(e));
}

chd_status_t raster(const chd_decoder_t *d, const std::vector<Span> &spans, bool isFloat, void *host)
{
    const int w = d->outWidth, h = d->outHeight;
    const size_t bytes = (size_t)w * h * (isFloat ? 4 : 2);
    cudaError_t e;
    int dev = d->device;
    if (d->resolvedKind == CHD_DEC_NONE && (e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_fail("no CUDA device", e);
    if ((e = cudaSetDevice(dev)) != cudaSuccess) return cuda_fail("cudaSetDevice", e);
    cudaStream_t s;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail("stream", e);
    void *plane = nullptr;
    Span *ds = nullptr;
    chd_status_t rc = CHD_OK;
    if ((e = cudaMallocAsync(&plane, bytes, s)) != cudaSuccess) rc = cuda_fail("plane", e);
    if (rc == CHD_OK && !spans.empty()) {
        if ((e = cudaMallocAsync((void **)&ds, spans.size() * sizeof(Span), s)) != cudaSuccess) rc = cuda_fail("spans", e);
        else if ((e = cudaMemcpyAsync(ds, spans.data(), spans.size() * sizeof(Span), cudaMemcpyHostToDevice, s)) !=
                 cudaSuccess)
            rc = cuda_fail("H2D", e);
    }
    if (rc == CHD_OK && mask_raster(plane, isFloat, w, h, ds, (int)spans.size(), s) != 0)
        rc = cuda_fail("raster kernel", cudaGetLastError());
    if (rc == CHD_OK && (e = cudaMemcpyAsync(host, plane, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        rc = cuda_fail("D2H", e);
    if (ds) cudaFreeAsync(ds, s);
    if (plane) cudaFreeAsync(plane, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess && rc == CHD_OK) rc = cuda_fail("sync", e);
    cudaStreamDestroy(s);
    return rc;
}

}  // namespace

// c_api_dropout.cpp:24-43
CHD_API chd_status_t chd_decoder_set_dropout(chd_decoder_t *d, const chd_dropout_opts_t *opts)
{
    if (d == nullptr || opts == nullptr) return fail(CHD_E_INVALID_ARG, "chd_decoder_set_dropout: null argument");
    d->dropoutOpts = *opts;
    d->dropoutOptsSet = true;
    d->dropoutRevision.fetch_add(1, std::memory_order_release);
    return CHD_OK;
}

CHD_API chd_status_t chd_decoder_get_last_dropout_stats(const chd_decoder_t *d, chd_dropout_stats_t *out)
{
    if (d == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_decoder_get_last_dropout_stats: null argument");
    std::lock_guard<std::mutex> l(const_cast<chd_decoder_t *>(d)->statsMutex);
    *out = d->lastDropoutStats;
    return CHD_OK;
}

// c_api_dropout_detect.cpp:185-203
CHD_API chd_status_t chd_decoder_get_output_info(const chd_decoder_t *d, chd_output_info_t *out)
{
    if (d == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_get_output_info: null argument");
    if (!d->committed) return fail(CHD_E_INVALID_ARG, "chd_decoder_get_output_info: chd_decoder_commit not called");
    out->format = d->outputPixelFormat;
    out->width = d->outWidth;
    out->height = d->outHeight;
    out->num_planes = (d->outputPixelFormat == CHD_PIXEL_GRAY16 || d->outputPixelFormat == CHD_PIXEL_GRAYS) ? 1 : 3;
    out->num_frames = d->numFrames;
    return CHD_OK;
}

// c_api_dropout_detect.cpp:205-239
CHD_API chd_status_t chd_decoder_get_dropout_spans(chd_decoder_t *d, int64_t frame_index,
                                                   chd_dropout_detect_mode_t mode, chd_dropout_span_t **out_spans,
                                                   size_t *out_count)
{
    if (d == nullptr || out_spans == nullptr || out_count == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_decoder_get_dropout_spans: null argument");
    *out_spans = nullptr;
    *out_count = 0;
    if (!d->committed) return fail(CHD_E_INVALID_ARG, "chd_decoder_get_dropout_spans: chd_decoder_commit not called");
    if (!valid_mode(mode)) return fail(CHD_E_INVALID_ARG, "chd_decoder_get_dropout_spans: unknown detect mode");
    std::vector<Span> spans;
    if (const chd_status_t rc = collect(d, frame_index, mode, spans); rc != CHD_OK) return rc;
    if (spans.empty()) return CHD_OK;
    static_assert(sizeof(Span) == sizeof(chd_dropout_span_t), "span layouts differ");
    auto *arr = static_cast<chd_dropout_span_t *>(std::malloc(spans.size() * sizeof(chd_dropout_span_t)));
    if (arr == nullptr) return fail(CHD_E_OOM, "chd_decoder_get_dropout_spans: out of memory");
    for (size_t i = 0; i < spans.size(); i++)
        arr[i] = {spans[i].y, spans[i].x_start, spans[i].x_end, CHD_DROPOUT_ORIGIN_SOURCE_METADATA};
    *out_spans = arr;
    *out_count = spans.size();
    return CHD_OK;
}

CHD_API void chd_dropout_spans_free(chd_dropout_span_t *spans) { std::free(spans); }

// c_api_dropout_detect.cpp:245-294
CHD_API chd_status_t chd_decode_dropout_mask(chd_decoder_t *d, int64_t frame_index, chd_dropout_detect_mode_t mode,
                                             chd_frame_t **out)
{
    if (d == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_decode_dropout_mask: null argument");
    *out = nullptr;
    if (!d->committed) return fail(CHD_E_INVALID_ARG, "chd_decode_dropout_mask: chd_decoder_commit not called");
    if (!valid_mode(mode)) return fail(CHD_E_INVALID_ARG, "chd_decode_dropout_mask: unknown detect mode");
    std::vector<Span> spans;
    if (const chd_status_t rc = collect(d, frame_index, mode, spans); rc != CHD_OK) return rc;
    if (d->outWidth <= 0 || d->outHeight <= 0)
        return fail(CHD_E_INTERNAL, "chd_decode_dropout_mask: invalid output geometry");
    const bool isFloat = mask_is_float(d->outputPixelFormat);
    auto f = std::make_unique<chd_frame>();
    f->format = isFloat ? CHD_PIXEL_GRAYS : CHD_PIXEL_GRAY16;
    f->width = d->outWidth;
    f->height = d->outHeight;
    const size_t pixels = (size_t)f->width * f->height;
    void *host;
    if (isFloat) {
        f->maskf.resize(pixels);
        host = f->maskf.data();
    } else {
        f->mask16.resize(pixels);
        host = f->mask16.data();
    }
    if (const chd_status_t rc = raster(d, spans, isFloat, host); rc != CHD_OK) return rc;
    f->pixels = host;
    f->info.format = f->format;
    f->info.width = f->width;
    f->info.height = f->height;
    f->info.num_planes = 1;
    f->info.frame_index = frame_index;
    *out = f.release();
    return CHD_OK;
}
