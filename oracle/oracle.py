"""ctypes front end of the CPU oracle (oracle/tpal_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker or the timed CPU stand-in,
never as the product path. ``build()`` compiles the C restatement with the
recipe in oracle/Makefile (gcc, -ffp-contract=off).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtpal_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "chd_ref_harness")

FMT_P16 = 0
FMT_PS = 1
FMT_RGB48 = 2
FMT_RGBS = 3
FMT_GRAY16 = 4
FMT_GRAYS = 5


class Params(C.Structure):
    _fields_ = [
        ("field_width", C.c_int32), ("field_height", C.c_int32),
        ("active_start", C.c_int32), ("active_end", C.c_int32),
        ("first_active_frame_line", C.c_int32), ("last_active_frame_line", C.c_int32),
        ("burst_start", C.c_int32), ("burst_end", C.c_int32),
        ("black", C.c_int32), ("white", C.c_int32),
        ("sample_rate", C.c_double), ("fsc", C.c_double),
        ("is_pal_m", C.c_int32),
        ("kind", C.c_int32),
        ("threshold", C.c_double),
        ("thresholds", C.POINTER(C.c_double)), ("n_thresholds", C.c_int32),
        ("chroma_gain", C.c_double), ("chroma_phase_deg", C.c_double),
        ("output_format", C.c_int32), ("clamp_mode", C.c_int32), ("padding_multiple", C.c_int32),
        ("ecb_from_u", C.c_double), ("ecr_from_v", C.c_double),
        ("kr", C.c_double), ("kb", C.c_double), ("u_reduction", C.c_double), ("v_reduction", C.c_double),
        ("y_nr_level", C.c_double), ("first_field_offset", C.c_int32), ("sc_locked", C.c_int32),
    ]


class Dropout(C.Structure):
    _fields_ = [("field", C.c_int32), ("startx", C.c_int32), ("endx", C.c_int32), ("field_line", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("corrected", C.c_int64), ("failed", C.c_int64), ("total_distance", C.c_int64)]


class Span(C.Structure):
    _fields_ = [("y", C.c_int32), ("x_start", C.c_int32), ("x_end", C.c_int32), ("origin", C.c_int32)]


def build(force: bool = False) -> str:
    """Compile the C restatement (no reference sources needed)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                             for f in ("tpal_oracle.c", "tpal_oracle.h", "fft64.c", "fft64.h")):
        subprocess.run(["make", "-s", "-C", HERE, "restatement"], check=True)
    return LIB_PATH


def build_reference(ref_root: str = "/root/reference") -> Optional[str]:
    """Compile the reference's own hot-path sources into oracle/_ref (only
    where the reference checkout exists)."""
    if not os.path.isdir(os.path.join(ref_root, "src", "decoders", "palcolour")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return REF_HARNESS


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.tpo_default_params.argtypes = [C.POINTER(Params), C.c_int32]
        L.tpo_output_geometry.argtypes = [C.POINTER(Params)] + [C.POINTER(C.c_int32)] * 4
        L.tpo_frame_bytes.argtypes = [C.POINTER(Params)]
        L.tpo_frame_bytes.restype = C.c_size_t
        L.tpo_decode_frames.argtypes = [C.POINTER(Params), C.c_void_p, C.c_int32, C.POINTER(Dropout), C.c_int32,
                                        C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                        C.POINTER(Stats)]
        L.tpo_transform_chroma.argtypes = [C.POINTER(Params), C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
        L.tpo_dropout_correct_frame.argtypes = [C.POINTER(Params), C.c_void_p, C.c_int32, C.POINTER(Dropout),
                                                C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                                C.POINTER(Stats)]
        L.tpo_dropout_spans.argtypes = [C.POINTER(Params), C.POINTER(Dropout), C.c_int32, C.c_int32, C.c_int32,
                                        C.POINTER(Span), C.c_int32]
        L.tpo_dropout_spans.restype = C.c_int32
        _lib = L
    return _lib


def params(kind: int = 3, fmt: int = FMT_P16, threshold: float = 0.4,
           thresholds: Optional[Sequence[float]] = None, **kw) -> Params:
    p = Params()
    lib().tpo_default_params(C.byref(p), kind)
    p.output_format = fmt
    p.threshold = threshold
    if thresholds is not None:
        arr = (C.c_double * len(thresholds))(*thresholds)
        p._thr_keepalive = arr
        p.thresholds = arr
        p.n_thresholds = len(thresholds)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def frame_dtype(p: Params):
    return np.float32 if p.output_format in (FMT_PS, FMT_RGBS, FMT_GRAYS) else np.uint16


def frame_shape(p: Params, count: int, w: int, h: int):
    """Array shape of `count` output frames: planar formats (count, planes,
    h, w); RGB48 is interleaved (count, h, w, 3) as OutputWriter packs it."""
    if p.output_format == FMT_RGB48:
        return (count, h, w, 3)
    planes = 1 if p.output_format in (FMT_GRAY16, FMT_GRAYS) else 3
    return (count, planes, h, w)


def colour_precision(p: Params, difference: str = "modern", scaling: str = "scientific") -> None:
    """ColorConversion for the two precision options (color_conversion.cpp:33-66)."""
    p.kr, p.kb = (0.30, 0.11) if difference == "classic" else (0.299, 0.114)
    p.u_reduction, p.v_reduction = {"classic": (0.493, 0.877), "modern": (0.492111, 0.877283),
                                    "scientific": (0.49211104112248356308804691718185,
                                                   0.87728321993817866838972487283129)}[scaling]
    p.ecb_from_u = 1.0 / ((2.0 * (1.0 - p.kb)) * p.u_reduction)
    p.ecr_from_v = 1.0 / ((2.0 * (1.0 - p.kr)) * p.v_reduction)


def output_geometry(p: Params) -> Tuple[int, int, int, int]:
    w, h, lp, tp = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    lib().tpo_output_geometry(C.byref(p), C.byref(w), C.byref(h), C.byref(lp), C.byref(tp))
    return w.value, h.value, lp.value, tp.value


def _dropout_array(dropouts):
    if not dropouts:
        return None, 0
    arr = (Dropout * len(dropouts))()
    for i, (f, sx, ex, fl) in enumerate(dropouts):
        arr[i].field, arr[i].startx, arr[i].endx, arr[i].field_line = f, sx, ex, fl
    return arr, len(dropouts)


def flatten_dropouts(per_field) -> List[Tuple[int, int, int, int]]:
    """[[(startx, endx, fieldLine)...] per field] -> [(field, startx, endx, fieldLine)]"""
    out = []
    for f, spans in enumerate(per_field):
        for s in spans:
            out.append((f, s[0], s[1], s[2]))
    return out


def decode_frames(p: Params, fields: np.ndarray, first: int, count: int, dropouts=None,
                  overcorrect: bool = False, intra: bool = False, threads: int = 1):
    """Decoded frames as an array (count, 3, h, w) of uint16 (p16) or float32 (ps),
    plus the summed dropout stats of the decoded frames."""
    fields = np.ascontiguousarray(fields, dtype=np.uint16)
    nfields = fields.shape[0]
    w, h, _, _ = output_geometry(p)
    out = np.empty(frame_shape(p, count, w, h), dtype=frame_dtype(p))
    arr, nd = _dropout_array(dropouts)
    st = Stats()
    rc = lib().tpo_decode_frames(C.byref(p), fields.ctypes.data, nfields, arr, nd, int(overcorrect), int(intra),
                                 first, count, out.ctypes.data, threads, C.byref(st))
    if rc != 0:
        raise RuntimeError("tpo_decode_frames failed")
    return out, (st.corrected, st.failed, st.total_distance)


def transform_chroma(p: Params, fields: np.ndarray, first: int, count: int) -> np.ndarray:
    fields = np.ascontiguousarray(fields, dtype=np.uint16)
    out = np.empty((2 * count, p.field_height, p.field_width), dtype=np.float64)
    if lib().tpo_transform_chroma(C.byref(p), fields.ctypes.data, fields.shape[0], first, count,
                                  out.ctypes.data) != 0:
        raise RuntimeError("tpo_transform_chroma failed")
    return out


def dropout_correct_frame(p: Params, fields: np.ndarray, frame: int, dropouts, overcorrect=False, intra=False):
    fields = np.ascontiguousarray(fields, dtype=np.uint16)
    out = np.empty((2, p.field_height, p.field_width), dtype=np.uint16)
    arr, nd = _dropout_array(dropouts)
    st = Stats()
    if lib().tpo_dropout_correct_frame(C.byref(p), fields.ctypes.data, fields.shape[0], arr, nd, int(overcorrect),
                                       int(intra), frame, out.ctypes.data, C.byref(st)) != 0:
        raise RuntimeError("tpo_dropout_correct_frame failed")
    return out, (st.corrected, st.failed, st.total_distance)


def dropout_spans(p: Params, dropouts, frame: int, mode: int = 0):
    arr, nd = _dropout_array(dropouts)
    cap = max(16, 4 * nd)
    spans = (Span * cap)()
    n = lib().tpo_dropout_spans(C.byref(p), arr, nd, frame, mode, spans, cap)
    return [(spans[i].y, spans[i].x_start, spans[i].x_end, spans[i].origin) for i in range(min(n, cap))]
