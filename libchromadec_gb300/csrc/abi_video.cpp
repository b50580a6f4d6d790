// abi_video.cpp -- library lifecycle, version, cancellation and composite
// sources of the chd_* ABI (include/chromadec/video.h, version.h,
// pipeline.h). Behaviour follows the reference's src/abi/c_api_video.cpp,
// c_api_lifecycle.cpp and c_api_pipeline.cpp; each function cites the
// reference lines it mirrors.
#include <cmath>
#include <cstring>
#include <memory>
#include <string>

#include <sys/stat.h>

#include "abi_handles.h"
#include "error_state.h"

namespace {

chd_status_t fail(chd_status_t s, const std::string &msg)
{
    chd::detail::set_last_error(msg);
    return s;
}

chd_video_standard_t abi_standard(int system)
{
    switch (system) {
    case chdg::SYS_PAL: return CHD_STD_PAL;
    case chdg::SYS_NTSC: return CHD_STD_NTSC;
    case chdg::SYS_PAL_M: return CHD_STD_PAL_M;
    case chdg::SYS_SECAM: return CHD_STD_SECAM;
    }
    return CHD_STD_UNKNOWN;
}

// nativeSamplesPerFrame (c_api_video.cpp:240-256) with the standards'
// frame totals (src/format/video_standards.cpp:55-100).
int32_t native_samples_per_frame(int system)
{
    switch (system) {
    case chdg::SYS_PAL:
    case chdg::SYS_SECAM: return 709379;
    case chdg::SYS_NTSC: return 477750;
    case chdg::SYS_PAL_M: return 477750 - 525;
    }
    return 0;
}

// standardSampleRotation (c_api_video.cpp:794-823): where standard sample 0
// sits in a stored row. Line-locked .tbc rows start at 0H (sync start); a
// subcarrier-locked .tbc starts at the first digital blanking sample
// (src/reader/tbc_source.cpp:165-175). Presets: 625-line 1135 samples per
// line, 948 digital active samples, blanking start 9.5 samples before 0H;
// 525-line 910 (PAL-M 909) samples per line, 768 active, blanking start
// 16.3667 (PAL-M x 909/910) (src/format/video_standards.cpp:55-100).
chd_status_t sample_rotation(const chd_video_t *v, const char *caller, int32_t &rowWidth, int32_t &zeroAt)
{
    const chdg::VideoParams &vp = v->cap.vp();
    double samplesPerLine, active, blankStart;
    if (vp.system == chdg::SYS_NTSC) {
        samplesPerLine = 910.0;
        active = 768.0;
        blankStart = 784.0 + 33.0 / 90.0 - 768.0;
    } else if (vp.system == chdg::SYS_PAL_M) {
        samplesPerLine = 909.0;
        active = 768.0;
        blankStart = (784.0 + 33.0 / 90.0 - 768.0) * (909.0 / 910.0);
    } else {
        samplesPerLine = 1135.0;
        active = 948.0;
        blankStart = 957.5 - 948.0;
    }
    const int32_t spl = (int32_t)samplesPerLine;
    if (vp.fieldWidth != spl)
        return fail(CHD_E_UNSUPPORTED, std::string(caller) + ": source row width " + std::to_string(vp.fieldWidth) +
                                           " is not the standard 4fsc line of " + std::to_string(spl) + " samples");
    zeroAt = vp.isSubcarrierLocked ? spl - (int32_t)active : spl - (int32_t)std::ceil(active + blankStart);
    rowWidth = spl;
    return CHD_OK;
}

}  // namespace

// ---- lifecycle (c_api_lifecycle.cpp) ----------------------------------------

CHD_API chd_status_t chd_init(void) { return CHD_OK; }
CHD_API void chd_shutdown(void) {}
CHD_API const char *chd_version_string(void) { return CHROMADEC_VERSION_STRING; }

CHD_API void chd_version(int *major, int *minor, int *patch)
{
    if (major) *major = CHROMADEC_VERSION_MAJOR;
    if (minor) *minor = CHROMADEC_VERSION_MINOR;
    if (patch) *patch = CHROMADEC_VERSION_PATCH;
}

CHD_API int chd_has_feature(const char *feature)
{
    if (feature == nullptr) return 0;
    return (std::strcmp(feature, "cuda") == 0 || std::strcmp(feature, "gb300") == 0) ? 1 : 0;
}

// ---- cancellation (c_api_pipeline.cpp) --------------------------------------

CHD_API chd_status_t chd_cancel_create(chd_cancel_t **out)
{
    if (out == nullptr) return fail(CHD_E_INVALID_ARG, "chd_cancel_create: null argument");
    *out = new chd_cancel();
    return CHD_OK;
}

CHD_API void chd_cancel_request(chd_cancel_t *c)
{
    if (c != nullptr) c->requested.store(true, std::memory_order_release);
}

CHD_API int chd_cancel_is_requested(const chd_cancel_t *c)
{
    return (c != nullptr && c->requested.load(std::memory_order_acquire)) ? 1 : 0;
}

CHD_API void chd_cancel_free(chd_cancel_t *c) { delete c; }

// ---- sources (c_api_video.cpp:650-897) --------------------------------------

CHD_API chd_status_t chd_video_open_composite(const char *path, const char *metadata_path_or_null,
                                              const chd_video_params_t *override_or_null, chd_video_t **out)
{
    if (path == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chd_video_open_composite: null argument");
    *out = nullptr;
    auto v = std::make_unique<chd_video>();
    const int rc = v->cap.open(path, metadata_path_or_null, override_or_null);
    if (rc != CHD_OK) {
        chd::detail::set_last_error("chd_video_open_composite: " + chd::detail::get_last_error());
        return (chd_status_t)rc;
    }
    *out = v.release();
    return CHD_OK;
}

CHD_API chd_status_t chd_video_open_yc(const char *luma_path, const char *chroma_path, const char *, const
                                       chd_video_params_t *, chd_video_t **out)
{
    if (luma_path == nullptr || chroma_path == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_video_open_yc: null argument");
    *out = nullptr;
    return fail(CHD_E_UNSUPPORTED, "chd_video_open_yc: Y/C captures are not decoded by the Transform-PAL GPU path");
}

CHD_API void chd_video_free(chd_video_t *v) { delete v; }

// chd_video_get_info, c_api_video.cpp:713-756.
CHD_API chd_status_t chd_video_get_info(const chd_video_t *v, chd_video_info_t *out)
{
    if (v == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chd_video_get_info: null argument");
    const chdg::VideoParams &vp = v->cap.vp();
    std::memset(out, 0, sizeof(*out));
    out->standard = abi_standard(vp.system);
    out->encoding = CHD_ENC_CVBS_U16_4FSC;   // .tbc: 10-bit samples << 6 in uint16
    out->signal_state = vp.isSubcarrierLocked ? CHD_SIG_STANDARD_TBC_LOCKED : CHD_SIG_STANDARD_TBC_UNLOCKED;
    out->layout = CHD_FRAME_LAYOUT_FIELD_RASTER;
    out->field_width = vp.fieldWidth;
    out->field_height = vp.fieldHeight;
    out->samples_per_frame = native_samples_per_frame(vp.system);
    out->sample_rate_hz = vp.sampleRate;
    out->fsc_hz = vp.fSC;
    out->first_active_sample = vp.activeVideoStart;
    out->last_active_sample = vp.activeVideoEnd - 1;
    out->first_active_frame_line = vp.firstActiveFrameLine;
    out->last_active_frame_line = vp.lastActiveFrameLine;
    out->black_16b_ire = vp.black16bIre;
    out->white_16b_ire = vp.white16bIre;
    out->blanking_16b_ire = vp.blanking16bIre;
    const bool ff = v->cap.isFirstFieldFirst();
    out->num_frames = v->cap.numFrames(ff);
    out->is_first_field_first = ff ? 1 : 0;
    out->is_widescreen = vp.isWidescreen ? 1 : 0;
    out->is_subcarrier_locked = vp.isSubcarrierLocked ? 1 : 0;
    return CHD_OK;
}

// c_api_video.cpp:758-792.
CHD_API chd_status_t chd_video_frame_line_to_signal_line(const chd_video_t *v, int32_t frame_line, int32_t *out)
{
    if (v == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_video_frame_line_to_signal_line: null argument");
    const int32_t H = v->cap.vp().fieldHeight;
    if (frame_line < 0 || frame_line > 2 * H - 2)
        return fail(CHD_E_OUT_OF_RANGE,
                    "chd_video_frame_line_to_signal_line: frame_line out of range [0, (2 * field_height) - 2]");
    *out = (frame_line % 2 == 0) ? frame_line / 2 + 1 : H + (frame_line + 1) / 2;
    return CHD_OK;
}

CHD_API chd_status_t chd_video_signal_line_to_frame_line(const chd_video_t *v, int32_t signal_line, int32_t *out)
{
    if (v == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_video_signal_line_to_frame_line: null argument");
    const int32_t H = v->cap.vp().fieldHeight;
    if (signal_line < 1 || signal_line > 2 * H - 1)
        return fail(CHD_E_OUT_OF_RANGE,
                    "chd_video_signal_line_to_frame_line: signal_line out of range [1, (2 * field_height) - 1]");
    *out = (signal_line <= H) ? 2 * (signal_line - 1) : 2 * (signal_line - H - 1) + 1;
    return CHD_OK;
}

// c_api_video.cpp:825-857.
CHD_API chd_status_t chd_video_standard_sample_to_row_sample(const chd_video_t *v, int32_t standard_sample,
                                                             int32_t *out)
{
    if (v == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_video_standard_sample_to_row_sample: null argument");
    int32_t w = 0, z = 0;
    if (const chd_status_t s = sample_rotation(v, "chd_video_standard_sample_to_row_sample", w, z); s != CHD_OK)
        return s;
    if (standard_sample < 0 || standard_sample >= w)
        return fail(CHD_E_OUT_OF_RANGE,
                    "chd_video_standard_sample_to_row_sample: standard_sample out of range [0, field_width - 1]");
    *out = (standard_sample + z) % w;
    return CHD_OK;
}

CHD_API chd_status_t chd_video_row_sample_to_standard_sample(const chd_video_t *v, int32_t row_sample, int32_t *out)
{
    if (v == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chd_video_row_sample_to_standard_sample: null argument");
    int32_t w = 0, z = 0;
    if (const chd_status_t s = sample_rotation(v, "chd_video_row_sample_to_standard_sample", w, z); s != CHD_OK)
        return s;
    if (row_sample < 0 || row_sample >= w)
        return fail(CHD_E_OUT_OF_RANGE,
                    "chd_video_row_sample_to_standard_sample: row_sample out of range [0, field_width - 1]");
    *out = (row_sample - z + w) % w;
    return CHD_OK;
}

// ---- extra sources for multi-source concealment (c_api_video.cpp:586-897) ---

namespace {

bool exists(const std::string &p)
{
    struct stat st;
    return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// Open one extra capture the way the primary is opened (no parameter
// override); its failure detail is re-attributed to `fn`.
int open_extra(const std::string &fn, const char *path, const char *sidecar, std::unique_ptr<chdg::Capture> &out)
{
    auto c = std::make_unique<chdg::Capture>();
    const int rc = c->open(path, sidecar, nullptr);
    if (rc != CHD_OK) {
        std::string detail = chd::detail::get_last_error();
        const std::string prefix = "chd_video_open_composite: ";
        if (detail.compare(0, prefix.size(), prefix) == 0) detail.erase(0, prefix.size());
        chd::detail::set_last_error(fn + ": " + detail);
        return rc;
    }
    out = std::move(c);
    return CHD_OK;
}

// The concealment kernel reads an extra's replacement lines with the
// primary's field geometry, so an extra must share it.
int check_geometry(const std::string &fn, const chd_video_t *v, const chdg::Capture &x)
{
    if (x.vp().fieldWidth != v->cap.vp().fieldWidth || x.vp().fieldHeight != v->cap.vp().fieldHeight)
        return fail(CHD_E_FORMAT_UNSUPPORTED, fn + ": the extra source's field geometry differs from the primary's");
    return CHD_OK;
}

}  // namespace

CHD_API chd_status_t chd_video_add_extra_source_composite(chd_video_t *v, const char *path,
                                                          const char *metadata_path_or_null)
{
    const std::string fn = "chd_video_add_extra_source_composite";
    if (v == nullptr || path == nullptr) return fail(CHD_E_INVALID_ARG, fn + ": null argument");
    if (v->extrasFrozen.load(std::memory_order_acquire))
        return fail(CHD_E_INVALID_ARG, fn + ": a decode has already run with dropout correction on");
    if (!exists(path)) return fail(CHD_E_FILE_NOT_FOUND, fn + ": file does not exist: " + path);
    std::unique_ptr<chdg::Capture> x;
    if (const int rc = open_extra(fn, path, metadata_path_or_null, x); rc != CHD_OK) return (chd_status_t)rc;
    if (const int rc = check_geometry(fn, v, *x); rc != CHD_OK) return (chd_status_t)rc;
    v->extras.push_back(std::move(x));
    return CHD_OK;
}

// A luma extra corrects the luma plane and a chroma extra the separately
// decoded chroma plane of a Y/C decode; for the composite decodes of this
// library the luma capture is the extra, as in the reference, and the chroma
// capture is opened and checked but not read.
CHD_API chd_status_t chd_video_add_extra_source_yc(chd_video_t *v, const char *luma_path, const char *chroma_path,
                                                   const char *metadata_path_or_null)
{
    const std::string fn = "chd_video_add_extra_source_yc";
    if (v == nullptr || luma_path == nullptr || chroma_path == nullptr)
        return fail(CHD_E_INVALID_ARG, fn + ": null argument");
    if (v->extrasFrozen.load(std::memory_order_acquire))
        return fail(CHD_E_INVALID_ARG, fn + ": a decode has already run with dropout correction on");
    if (!exists(luma_path) || !exists(chroma_path))
        return fail(CHD_E_FILE_NOT_FOUND, fn + ": luma/chroma file does not exist");
    // openYcPair (c_api_video.cpp:586-629): the chroma plane's own sidecar,
    // else the luma's
    const std::string lumaSidecar =
        metadata_path_or_null != nullptr ? std::string(metadata_path_or_null) : std::string(luma_path) + ".json";
    std::unique_ptr<chdg::Capture> luma, chroma;
    if (const int rc = open_extra(fn + " (luma)", luma_path, metadata_path_or_null, luma); rc != CHD_OK)
        return (chd_status_t)rc;
    const bool chromaOwn = exists(std::string(chroma_path) + ".json") || exists(std::string(chroma_path) + ".db");
    if (const int rc = open_extra(fn + " (chroma)", chroma_path, chromaOwn ? nullptr : lumaSidecar.c_str(), chroma);
        rc != CHD_OK)
        return (chd_status_t)rc;
    if (luma->vp().fieldWidth != chroma->vp().fieldWidth || luma->vp().fieldHeight != chroma->vp().fieldHeight)
        return fail(CHD_E_FORMAT_UNSUPPORTED, fn + ": luma and chroma have mismatched dimensions");
    if (luma->numFrames(luma->isFirstFieldFirst()) != chroma->numFrames(chroma->isFirstFieldFirst()))
        return fail(CHD_E_FORMAT_UNSUPPORTED, fn + ": luma and chroma have different frame counts");
    if (const int rc = check_geometry(fn, v, *luma); rc != CHD_OK) return (chd_status_t)rc;
    v->extras.push_back(std::move(luma));
    v->chromaExtras.push_back(std::move(chroma));
    return CHD_OK;
}

CHD_API int chdg_video_source_frame(const chd_video_t *v, int32_t reverse_field_order, int32_t source,
                                    int32_t primary_frame, int32_t *out_frame)
{
    if (v == nullptr || out_frame == nullptr) return fail(CHD_E_INVALID_ARG, "chdg_video_source_frame: null argument");
    if (source < 0 || (size_t)source > v->extras.size())
        return fail(CHD_E_OUT_OF_RANGE, "chdg_video_source_frame: no such source");
    const bool rev = reverse_field_order != 0;
    std::vector<chdg::AlignedSource> all;
    all.push_back({&v->cap, v->cap.isFirstFieldFirst() != rev});
    for (const auto &x : v->extras) all.push_back({x.get(), x->isFirstFieldFirst() != rev});
    const chdg::SourceAlignment a(all, false);
    const int32_t f = a.frameFor(primary_frame + 1, source);
    const int frames = all[(size_t)source].cap->numFrames(all[(size_t)source].firstFieldFirst);
    *out_frame = (f >= 1 && f <= frames) ? f - 1 : -1;
    return CHD_OK;
}
