// abi_frame.cpp -- decoded-frame accessors of the chd_* ABI
// (include/chromadec/frame.h; reference: src/abi/c_api_frame.cpp). Planes
// are borrowed from the frame: yuv444p16 is [Y | Cb | Cr] with a row stride
// of width * 2 bytes, yuv444ps and rgbs three float planes, rgb48 packed
// R'G'B' (row pitch width * 6 bytes); gray16 / grays frames and dropout
// masks are one plane.
#include "abi_handles.h"
#include "error_state.h"

namespace {

chd_status_t fail(chd_status_t s, const std::string &msg)
{
    chd::detail::set_last_error(msg);
    return s;
}

bool is_float(chd_pixel_format_t f)
{
    return f == CHD_PIXEL_YUV444PS || f == CHD_PIXEL_GRAYS || f == CHD_PIXEL_RGBS || f == CHD_PIXEL_YUV440PS;
}

}  // namespace

CHD_API chd_status_t chd_frame_get_info(const chd_frame_t *f, chd_frame_info_t *out)
{
    if (f == nullptr || out == nullptr) return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_get_info: null argument");
    *out = f->info;
    return CHD_OK;
}

// c_api_frame.cpp:36-75
CHD_API chd_status_t chd_frame_get_plane_info(const chd_frame_t *f, chd_plane_t plane, chd_plane_info_t *out)
{
    if (f == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_get_plane_info: null argument");
    bool valid = false;
    switch (f->format) {
    case CHD_PIXEL_YUV444P16:
    case CHD_PIXEL_YUV444PS:
    case CHD_PIXEL_YUV440P16:
    case CHD_PIXEL_YUV440PS: valid = plane == CHD_PLANE_Y || plane == CHD_PLANE_CB || plane == CHD_PLANE_CR; break;
    case CHD_PIXEL_GRAY16:
    case CHD_PIXEL_GRAYS: valid = plane == CHD_PLANE_Y; break;
    case CHD_PIXEL_RGB48:
    case CHD_PIXEL_RGBS: valid = plane == CHD_PLANE_R || plane == CHD_PLANE_G || plane == CHD_PLANE_B; break;
    }
    if (!valid)
        return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane_info: plane not valid for the frame's pixel format");
    out->width = f->width;
    out->height = f->height;
    out->first_frame_row = 0;
    return CHD_OK;
}

// Line-sequential (SECAM) chroma only (c_api_frame.cpp:77-107).
CHD_API chd_status_t chd_frame_chroma_row_component(const chd_frame_t *f, int32_t, chd_chroma_row_component_t *out)
{
    if (f == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_chroma_row_component: null argument");
    return fail(CHD_E_UNSUPPORTED, "chd_frame_chroma_row_component: frame does not carry line-sequential chroma");
}

CHD_API chd_status_t chd_frame_get_chroma_ident(const chd_frame_t *f, chd_chroma_ident_report_t *out)
{
    if (f == nullptr || out == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_get_chroma_ident: null argument");
    return fail(CHD_E_UNSUPPORTED, "chd_frame_get_chroma_ident: frame does not carry line-sequential chroma");
}

// c_api_frame.cpp:109-189
CHD_API chd_status_t chd_frame_get_plane(const chd_frame_t *f, chd_plane_t plane, const void **out_data,
                                         ptrdiff_t *out_stride_bytes)
{
    if (f == nullptr || out_data == nullptr || out_stride_bytes == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_get_plane: null argument");
    *out_data = nullptr;
    *out_stride_bytes = 0;
    const size_t wh = (size_t)f->width * (size_t)f->height;
    const auto *base = static_cast<const uint16_t *>(f->pixels);
    switch (f->format) {
    case CHD_PIXEL_YUV444P16:
        switch (plane) {
        case CHD_PLANE_Y: *out_data = base; break;
        case CHD_PLANE_CB: *out_data = base + wh; break;
        case CHD_PLANE_CR: *out_data = base + 2 * wh; break;
        default: return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane: plane not valid for YUV444P16");
        }
        *out_stride_bytes = (ptrdiff_t)f->width * 2;
        return CHD_OK;
    case CHD_PIXEL_GRAY16:
        if (plane != CHD_PLANE_Y) return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane: GRAY16 only has CHD_PLANE_Y");
        *out_data = base;
        *out_stride_bytes = (ptrdiff_t)f->width * 2;
        return CHD_OK;
    case CHD_PIXEL_RGB48:
        // packed R'G'B': the three accessors share the row pitch, offset 0/1/2 samples
        switch (plane) {
        case CHD_PLANE_R: *out_data = base; break;
        case CHD_PLANE_G: *out_data = base + 1; break;
        case CHD_PLANE_B: *out_data = base + 2; break;
        default: return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane: plane not valid for RGB48");
        }
        *out_stride_bytes = (ptrdiff_t)f->width * 3 * 2;
        return CHD_OK;
    default:
        if (is_float(f->format))
            return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane: use chd_frame_get_plane_float for float pixel formats");
        return fail(CHD_E_INTERNAL, "chd_frame_get_plane: unknown pixel format");
    }
}

// c_api_frame.cpp:191-234
CHD_API chd_status_t chd_frame_get_plane_float(const chd_frame_t *f, chd_plane_t plane, const float **out_data,
                                               ptrdiff_t *out_stride_bytes)
{
    if (f == nullptr || out_data == nullptr || out_stride_bytes == nullptr)
        return fail(CHD_E_INVALID_ARG, "chromadec: chd_frame_get_plane_float: null argument");
    if (!is_float(f->format))
        return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane_float: frame is not a float pixel format");
    if (f->format == CHD_PIXEL_GRAYS && plane != CHD_PLANE_Y)
        return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane_float: CHD_PIXEL_GRAYS only has CHD_PLANE_Y");
    int idx;
    if (f->format == CHD_PIXEL_RGBS) {
        switch (plane) {
        case CHD_PLANE_R: idx = 0; break;
        case CHD_PLANE_G: idx = 1; break;
        case CHD_PLANE_B: idx = 2; break;
        default: return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane_float: CHD_PIXEL_RGBS plane must be R, G, or B");
        }
    } else {
        switch (plane) {
        case CHD_PLANE_Y: idx = 0; break;
        case CHD_PLANE_CB: idx = 1; break;
        case CHD_PLANE_CR: idx = 2; break;
        default:
            return fail(CHD_E_INVALID_ARG, "chd_frame_get_plane_float: Y'CbCr float frame plane must be Y, Cb, or Cr");
        }
    }
    *out_data = static_cast<const float *>(f->pixels) + (size_t)idx * f->width * f->height;
    *out_stride_bytes = (ptrdiff_t)f->width * (ptrdiff_t)sizeof(float);
    return CHD_OK;
}

CHD_API void chd_frame_free(chd_frame_t *f) { delete f; }
