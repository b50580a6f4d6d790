"""ctypes binding of the reference-compatible chd_* ABI (include/chromadec/*.h).

This is the binding a Python consumer of the reference would write against
its C ABI: the same calls, structs and status codes (reference
include/chromadec/{video,decoder,frame,dropout,pipeline,errors}.h), with thin
classes that raise ChdError on a non-OK status. The library underneath
decodes CHD_DEC_PAL_2D, CHD_DEC_TRANSFORM_2D and CHD_DEC_TRANSFORM_3D on the
GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import device

# chd_status_t (errors.h)
OK = 0
E_INVALID_ARG = 1
E_FILE_NOT_FOUND = 2
E_IO = 3
E_FORMAT_UNSUPPORTED = 4
E_METADATA_MISSING = 5
E_METADATA_CORRUPT = 6
E_DECODER_UNKNOWN = 8
E_DECODER_INCOMPATIBLE = 9
E_OUT_OF_RANGE = 13
E_CANCELLED = 14
E_INTERNAL = 15
E_OOM = 16
E_UNSUPPORTED = 17

# chd_decoder_kind_t (decoder.h)
DEC_AUTO = 0
DEC_MONO = 1
DEC_NTSC_2D = 3
DEC_PAL_2D = 6
DEC_TRANSFORM_2D = 7
DEC_TRANSFORM_3D = 8
DEC_NONE = 13

# chd_pixel_format_t, chd_plane_t, detect modes
PIXEL_YUV444P16 = 0
PIXEL_YUV444PS = 1
PIXEL_RGB48 = 2
PIXEL_RGBS = 3
PIXEL_GRAY16 = 4
PIXEL_GRAYS = 5
PLANE_Y, PLANE_CB, PLANE_CR = 0, 1, 2
PLANE_R, PLANE_G, PLANE_B = 3, 4, 5
DROPOUT_DETECTED = 0
DROPOUT_OVERCORRECT = 1


class VideoParams(C.Structure):
    _fields_ = [("standard", C.c_int), ("encoding", C.c_int), ("signal_state", C.c_int), ("layout", C.c_int),
                ("is_subcarrier_locked", C.c_int), ("is_second_field_first", C.c_int)]


class VideoInfo(C.Structure):
    _fields_ = [("standard", C.c_int), ("encoding", C.c_int), ("signal_state", C.c_int), ("layout", C.c_int),
                ("field_width", C.c_int32), ("field_height", C.c_int32), ("samples_per_frame", C.c_int32),
                ("sample_rate_hz", C.c_double), ("fsc_hz", C.c_double),
                ("first_active_sample", C.c_int32), ("last_active_sample", C.c_int32),
                ("first_active_frame_line", C.c_int32), ("last_active_frame_line", C.c_int32),
                ("black_16b_ire", C.c_int32), ("white_16b_ire", C.c_int32), ("blanking_16b_ire", C.c_int32),
                ("num_frames", C.c_int64), ("is_widescreen", C.c_int), ("is_subcarrier_locked", C.c_int),
                ("is_first_field_first", C.c_int)]


class FrameInfo(C.Structure):
    _fields_ = [("format", C.c_int), ("width", C.c_int32), ("height", C.c_int32), ("num_planes", C.c_int32),
                ("frame_index", C.c_int64)]


class PlaneInfo(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("first_frame_row", C.c_int32)]


class OutputInfo(C.Structure):
    _fields_ = [("format", C.c_int), ("width", C.c_int32), ("height", C.c_int32), ("num_planes", C.c_int32),
                ("num_frames", C.c_int64)]


class DropoutOpts(C.Structure):
    _fields_ = [("enabled", C.c_int), ("overcorrect", C.c_int), ("intra_field_only", C.c_int),
                ("reserved", C.c_void_p * 4)]


class DropoutStats(C.Structure):
    _fields_ = [("corrected", C.c_int32), ("failed", C.c_int32), ("total_distance", C.c_int64)]


class DropoutSpan(C.Structure):
    _fields_ = [("y", C.c_int32), ("x_start", C.c_int32), ("x_end", C.c_int32), ("origin", C.c_int)]


FRAME_DONE_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int64, C.c_void_p)
LOG_FN = C.CFUNCTYPE(None, C.c_int, C.c_uint, C.c_char_p, C.c_void_p)

_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_SIGS = {
    "chd_init": ([], C.c_int), "chd_shutdown": ([], None),
    "chd_status_str": ([C.c_int], C.c_char_p), "chd_last_error": ([], C.c_char_p),
    "chd_clear_last_error": ([], None),
    "chd_version_string": ([], C.c_char_p),
    "chd_version": ([C.POINTER(C.c_int)] * 3, None), "chd_has_feature": ([C.c_char_p], C.c_int),
    "chd_video_open_composite": ([C.c_char_p, C.c_char_p, C.POINTER(VideoParams), _PP], C.c_int),
    "chd_video_open_yc": ([C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(VideoParams), _PP], C.c_int),
    "chd_video_free": ([_P], None),
    "chd_video_get_info": ([_P, C.POINTER(VideoInfo)], C.c_int),
    "chd_video_frame_line_to_signal_line": ([_P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "chd_video_signal_line_to_frame_line": ([_P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "chd_video_standard_sample_to_row_sample": ([_P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "chd_video_row_sample_to_standard_sample": ([_P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "chd_video_add_extra_source_composite": ([_P, C.c_char_p, C.c_char_p], C.c_int),
    "chd_video_add_extra_source_yc": ([_P, C.c_char_p, C.c_char_p, C.c_char_p], C.c_int),
    "chdg_video_source_frame": ([_P, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "chdg_decoder_concealed_fields": ([_P, C.c_int64, _P], C.c_int),
    "chd_decoder_create": ([_P, C.c_int, _PP], C.c_int), "chd_decoder_free": ([_P], None),
    "chd_decoder_set_option_f64": ([_P, C.c_char_p, C.c_double], C.c_int),
    "chd_decoder_set_option_i32": ([_P, C.c_char_p, C.c_int32], C.c_int),
    "chd_decoder_set_option_bool": ([_P, C.c_char_p, C.c_int], C.c_int),
    "chd_decoder_set_option_str": ([_P, C.c_char_p, C.c_char_p], C.c_int),
    "chd_decoder_has_option": ([_P, C.c_char_p], C.c_int),
    "chd_decoder_set_nn_model": ([_P, _P], C.c_int),
    "chd_decoder_commit": ([_P], C.c_int),
    "chd_decoder_get_output_info": ([_P, C.POINTER(OutputInfo)], C.c_int),
    "chd_decoder_get_chroma_click_thresholds": ([_P, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "chd_decode_frame": ([_P, C.c_int64, _PP], C.c_int),
    "chd_decode_frames_async": ([_P, C.POINTER(C.c_int64), C.c_size_t, FRAME_DONE_CB, _P, _P], C.c_int),
    "chd_frame_get_info": ([_P, C.POINTER(FrameInfo)], C.c_int),
    "chd_frame_get_plane_info": ([_P, C.c_int, C.POINTER(PlaneInfo)], C.c_int),
    "chd_frame_chroma_row_component": ([_P, C.c_int32, C.POINTER(C.c_int)], C.c_int),
    "chd_frame_get_chroma_ident": ([_P, _P], C.c_int),
    "chd_frame_get_plane": ([_P, C.c_int, _PP, C.POINTER(C.c_ssize_t)], C.c_int),
    "chd_frame_get_plane_float": ([_P, C.c_int, _PP, C.POINTER(C.c_ssize_t)], C.c_int),
    "chd_frame_free": ([_P], None),
    "chd_decoder_set_dropout": ([_P, C.POINTER(DropoutOpts)], C.c_int),
    "chd_decoder_get_last_dropout_stats": ([_P, C.POINTER(DropoutStats)], C.c_int),
    "chd_decoder_get_dropout_spans": ([_P, C.c_int64, C.c_int, C.POINTER(C.POINTER(DropoutSpan)),
                                       C.POINTER(C.c_size_t)], C.c_int),
    "chd_dropout_spans_free": ([C.POINTER(DropoutSpan)], None),
    "chd_decode_dropout_mask": ([_P, C.c_int64, C.c_int, _PP], C.c_int),
    "chd_cancel_create": ([_PP], C.c_int), "chd_cancel_request": ([_P], None),
    "chd_cancel_is_requested": ([_P], C.c_int), "chd_cancel_free": ([_P], None),
    "chd_set_log_callback": ([LOG_FN, _P], None), "chd_log_to_stderr": ([], None),
    "chd_set_log_level": ([C.c_int], None), "chd_get_log_level": ([], C.c_int),
    "chd_log_is_enabled": ([C.c_int], C.c_int), "chd_log_level_str": ([C.c_int], C.c_char_p),
}

_lib = None


def lib():
    """The loaded library with every chd_* signature declared."""
    global _lib
    if _lib is None:
        L = device.lib()
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


class ChdError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        detail = lib().chd_last_error().decode(errors="replace")
        name = lib().chd_status_str(status).decode()
        super().__init__(f"{where}: {name}: {detail}")


def check(status: int, where: str) -> None:
    if status != OK:
        raise ChdError(status, where)


def status_name(status: int) -> str:
    return lib().chd_status_str(status).decode()


class Frame:
    """A decoded frame; planes are copied out as numpy arrays."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        info = FrameInfo()
        check(lib().chd_frame_get_info(self._h, C.byref(info)), "chd_frame_get_info")
        self.info = info

    @property
    def index(self) -> int:
        return self.info.frame_index

    def plane(self, p: int) -> np.ndarray:
        L = lib()
        data = C.c_void_p()
        stride = C.c_ssize_t()
        w, h = self.info.width, self.info.height
        if self.info.format == PIXEL_RGB48:
            check(L.chd_frame_get_plane(self._h, p, C.byref(data), C.byref(stride)), "chd_frame_get_plane")
            n = (h - 1) * (stride.value // 2) + 3 * w - 2
            buf = (C.c_uint16 * n).from_address(data.value)
            a = np.frombuffer(buf, dtype=np.uint16)
            rows = [a[y * (stride.value // 2):y * (stride.value // 2) + 3 * w:3] for y in range(h)]
            return np.stack(rows).copy()
        if self.info.format in (PIXEL_YUV444PS, PIXEL_GRAYS, PIXEL_RGBS):
            check(L.chd_frame_get_plane_float(self._h, p, C.byref(data), C.byref(stride)), "chd_frame_get_plane_float")
            buf = (C.c_float * (h * stride.value // 4)).from_address(data.value)
            return np.frombuffer(buf, dtype=np.float32).reshape(h, stride.value // 4)[:, :w].copy()
        check(L.chd_frame_get_plane(self._h, p, C.byref(data), C.byref(stride)), "chd_frame_get_plane")
        buf = (C.c_uint16 * (h * stride.value // 2)).from_address(data.value)
        return np.frombuffer(buf, dtype=np.uint16).reshape(h, stride.value // 2)[:, :w].copy()

    def planes(self) -> np.ndarray:
        """Y'CbCr / gray formats: (planes, h, w); rgbs: (3, h, w) R, G, B;
        rgb48: (h, w, 3), the packed layout."""
        if self.info.format == PIXEL_RGB48:
            return np.stack([self.plane(p) for p in (PLANE_R, PLANE_G, PLANE_B)], axis=-1)
        if self.info.format == PIXEL_RGBS:
            return np.stack([self.plane(p) for p in (PLANE_R, PLANE_G, PLANE_B)])
        n = self.info.num_planes
        return np.stack([self.plane(p) for p in range(n)])

    def close(self) -> None:
        if self._h:
            lib().chd_frame_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Video:
    def __init__(self, path: str, meta: Optional[str] = None, override: Optional[VideoParams] = None):
        self._h = C.c_void_p()
        check(lib().chd_video_open_composite(path.encode(), meta.encode() if meta else None,
                                             C.byref(override) if override is not None else None,
                                             C.byref(self._h)), "chd_video_open_composite")

    def info(self) -> VideoInfo:
        out = VideoInfo()
        check(lib().chd_video_get_info(self._h, C.byref(out)), "chd_video_get_info")
        return out

    def close(self) -> None:
        if self._h:
            lib().chd_video_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Decoder:
    def __init__(self, video: Video, kind: int):
        self.video = video
        self._h = C.c_void_p()
        check(lib().chd_decoder_create(video._h, kind, C.byref(self._h)), "chd_decoder_create")

    def set(self, name: str, value) -> None:
        L = lib()
        n = name.encode()
        if isinstance(value, bool):
            check(L.chd_decoder_set_option_bool(self._h, n, int(value)), name)
        elif isinstance(value, int):
            check(L.chd_decoder_set_option_i32(self._h, n, value), name)
        elif isinstance(value, float):
            check(L.chd_decoder_set_option_f64(self._h, n, value), name)
        else:
            check(L.chd_decoder_set_option_str(self._h, n, str(value).encode()), name)

    def commit(self) -> None:
        check(lib().chd_decoder_commit(self._h), "chd_decoder_commit")

    def output_info(self) -> OutputInfo:
        out = OutputInfo()
        check(lib().chd_decoder_get_output_info(self._h, C.byref(out)), "chd_decoder_get_output_info")
        return out

    def set_dropout(self, enabled: bool = True, overcorrect: bool = False, intra: bool = False) -> None:
        o = DropoutOpts(int(enabled), int(overcorrect), int(intra))
        check(lib().chd_decoder_set_dropout(self._h, C.byref(o)), "chd_decoder_set_dropout")

    def last_dropout_stats(self) -> Tuple[int, int, int]:
        s = DropoutStats()
        check(lib().chd_decoder_get_last_dropout_stats(self._h, C.byref(s)), "chd_decoder_get_last_dropout_stats")
        return s.corrected, s.failed, s.total_distance

    def decode(self, index: int) -> Frame:
        h = C.c_void_p()
        check(lib().chd_decode_frame(self._h, index, C.byref(h)), "chd_decode_frame")
        return Frame(h.value)

    def decode_async(self, indices: Sequence[int], cancel_after: Optional[int] = None
                     ) -> List[Tuple[int, int, Optional[np.ndarray]]]:
        """chd_decode_frames_async; returns (status, index, planes) in
        completion order. With cancel_after=k, cancellation is requested from
        inside the k-th callback."""
        L = lib()
        results: List[Tuple[int, int, Optional[np.ndarray]]] = []
        cancel = C.c_void_p()
        check(L.chd_cancel_create(C.byref(cancel)), "chd_cancel_create")

        def cb(user, status, idx, frame):
            planes = None
            if frame:
                f = Frame(frame)
                planes = f.planes()
                f.close()
            results.append((status, idx, planes))
            if cancel_after is not None and len(results) == cancel_after:
                L.chd_cancel_request(cancel)

        arr = (C.c_int64 * len(indices))(*indices)
        fn = FRAME_DONE_CB(cb)
        try:
            check(L.chd_decode_frames_async(self._h, arr, len(indices), fn, None, cancel),
                  "chd_decode_frames_async")
        finally:
            L.chd_cancel_free(cancel)
        return results

    def dropout_spans(self, index: int, mode: int = DROPOUT_DETECTED) -> List[Tuple[int, int, int, int]]:
        L = lib()
        arr = C.POINTER(DropoutSpan)()
        n = C.c_size_t()
        check(L.chd_decoder_get_dropout_spans(self._h, index, mode, C.byref(arr), C.byref(n)),
              "chd_decoder_get_dropout_spans")
        out = [(arr[i].y, arr[i].x_start, arr[i].x_end, arr[i].origin) for i in range(n.value)]
        if n.value:
            L.chd_dropout_spans_free(arr)
        return out

    def dropout_mask(self, index: int, mode: int = DROPOUT_DETECTED) -> np.ndarray:
        h = C.c_void_p()
        check(lib().chd_decode_dropout_mask(self._h, index, mode, C.byref(h)), "chd_decode_dropout_mask")
        f = Frame(h.value)
        try:
            return f.plane(PLANE_Y)
        finally:
            f.close()

    def concealed_fields(self, index: int) -> np.ndarray:
        """Frame `index`'s two fields after the GPU concealment (device-level
        chdg_decoder_concealed_fields), shape (2, field_height, field_width)."""
        vi = self.video.info()
        out = np.empty((2, vi.field_height, vi.field_width), dtype=np.uint16)
        check(lib().chdg_decoder_concealed_fields(self._h, index, out.ctypes.data), "chdg_decoder_concealed_fields")
        return out

    def close(self) -> None:
        if self._h:
            lib().chd_decoder_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
