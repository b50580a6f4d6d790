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


class Extra(C.Structure):
    _fields_ = [("fields", C.c_void_p), ("nfields", C.c_int32), ("dropouts", C.POINTER(Dropout)),
                ("ndropouts", C.c_int32), ("bpsnr", C.POINTER(C.c_double)), ("frame_map", C.POINTER(C.c_int32)),
                ("nframe_map", C.c_int32)]


class Sources(C.Structure):
    _fields_ = [("bpsnr", C.POINTER(C.c_double)), ("extras", C.POINTER(Extra)), ("nextras", C.c_int32)]


class Span(C.Structure):
    _fields_ = [("y", C.c_int32), ("x_start", C.c_int32), ("x_end", C.c_int32), ("origin", C.c_int32)]


def build(force: bool = False) -> str:
    """Compile the C restatement (no reference sources needed)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                             for f in ("tpal_oracle.c", "tpal_oracle.h", "fft64.c", "fft64.h")):
        subprocess.run(["make", "-s", "-C", HERE, "restatement"], check=True)
    return LIB_PATH


def build_reference(ref_root: Optional[str] = None) -> Optional[str]:
    """Compile the reference's own hot-path sources into oracle/_ref from the
    reference checkout at ``ref_root`` (default: the CHROMADEC_REFERENCE
    environment variable); None when no checkout is given or found."""
    ref_root = ref_root or os.environ.get("CHROMADEC_REFERENCE")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src", "decoders", "palcolour")):
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
        L.tpo_decode_frames_ms.argtypes = [C.POINTER(Params), C.c_void_p, C.c_int32, C.POINTER(Dropout), C.c_int32,
                                           C.POINTER(Sources), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_void_p, C.c_int32, C.POINTER(Stats)]
        L.tpo_dropout_correct_frame_ms.argtypes = [C.POINTER(Params), C.c_void_p, C.c_int32, C.POINTER(Dropout),
                                                   C.c_int32, C.POINTER(Sources), C.c_int32, C.c_int32, C.c_int32,
                                                   C.c_void_p, C.POINTER(Stats)]
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


def pal_m(p: Params) -> Params:
    """PAL-M geometry and levels: the reference's PAL_M preset
    (src/format/video_standards.cpp:28-52, 85-100, 116-207; active frame
    lines src/metadata/core.cpp:52-70)."""
    p.field_width, p.field_height = 909, 263
    p.active_start, p.active_end = 124, 892
    p.first_active_frame_line, p.last_active_frame_line = 39, 524
    p.burst_start, p.burst_end = 75, 95
    p.black, p.white = 282 * 64, 800 * 64
    p.sample_rate = 4.0 * 525.0 * (30000.0 / 1001.0) * (909.0 / 4.0)
    p.fsc = 5.0e6 * (63.0 / 88.0) * (909.0 / 910.0)
    p.is_pal_m = 1
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


def _sources(bpsnr, extras):
    """ctypes Sources for the primary's per-field bPSNR and extra captures
    [dict(fields=(n, h, w) uint16, dropouts=[(field, startx, endx, fieldLine)],
    bpsnr=[per field] or None, frame_map=[per primary frame] or None)];
    returns (Sources or None, keep-alive list)."""
    if bpsnr is None and not extras:
        return None, []
    keep = []
    src = Sources()
    if bpsnr is not None:
        b = np.ascontiguousarray(bpsnr, dtype=np.float64)
        keep.append(b)
        src.bpsnr = b.ctypes.data_as(C.POINTER(C.c_double))
    ex = (Extra * max(1, len(extras or [])))()
    for i, e in enumerate(extras or []):
        f = np.ascontiguousarray(e["fields"], dtype=np.uint16)
        keep.append(f)
        ex[i].fields = f.ctypes.data
        ex[i].nfields = f.shape[0]
        arr, nd = _dropout_array(e.get("dropouts"))
        keep.append(arr)
        ex[i].dropouts = arr if arr is not None else None
        ex[i].ndropouts = nd
        if e.get("bpsnr") is not None:
            b = np.ascontiguousarray(e["bpsnr"], dtype=np.float64)
            keep.append(b)
            ex[i].bpsnr = b.ctypes.data_as(C.POINTER(C.c_double))
        if e.get("frame_map") is not None:
            m = np.ascontiguousarray(e["frame_map"], dtype=np.int32)
            keep.append(m)
            ex[i].frame_map = m.ctypes.data_as(C.POINTER(C.c_int32))
            ex[i].nframe_map = m.shape[0]
    keep.append(ex)
    src.extras = ex
    src.nextras = len(extras or [])
    return src, keep


def decode_frames(p: Params, fields: np.ndarray, first: int, count: int, dropouts=None,
                  overcorrect: bool = False, intra: bool = False, threads: int = 1, bpsnr=None, extras=None):
    """Decoded frames as an array (count, 3, h, w) of uint16 (p16) or float32 (ps),
    plus the summed dropout stats of the decoded frames. bpsnr / extras: the
    multi-source concealment inputs (see _sources)."""
    fields = np.ascontiguousarray(fields, dtype=np.uint16)
    nfields = fields.shape[0]
    w, h, _, _ = output_geometry(p)
    out = np.empty(frame_shape(p, count, w, h), dtype=frame_dtype(p))
    arr, nd = _dropout_array(dropouts)
    st = Stats()
    src, _keep = _sources(bpsnr, extras)
    rc = lib().tpo_decode_frames_ms(C.byref(p), fields.ctypes.data, nfields, arr, nd,
                                    C.byref(src) if src is not None else None, int(overcorrect), int(intra),
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


def dropout_correct_frame(p: Params, fields: np.ndarray, frame: int, dropouts, overcorrect=False, intra=False,
                          bpsnr=None, extras=None):
    fields = np.ascontiguousarray(fields, dtype=np.uint16)
    out = np.empty((2, p.field_height, p.field_width), dtype=np.uint16)
    arr, nd = _dropout_array(dropouts)
    st = Stats()
    src, _keep = _sources(bpsnr, extras)
    if lib().tpo_dropout_correct_frame_ms(C.byref(p), fields.ctypes.data, fields.shape[0], arr, nd,
                                          C.byref(src) if src is not None else None, int(overcorrect), int(intra),
                                          frame, out.ctypes.data, C.byref(st)) != 0:
        raise RuntimeError("tpo_dropout_correct_frame failed")
    return out, (st.corrected, st.failed, st.total_distance)


def dropout_spans(p: Params, dropouts, frame: int, mode: int = 0):
    arr, nd = _dropout_array(dropouts)
    cap = max(16, 4 * nd)
    spans = (Span * cap)()
    n = lib().tpo_dropout_spans(C.byref(p), arr, nd, frame, mode, spans, cap)
    return [(spans[i].y, spans[i].x_start, spans[i].x_end, spans[i].origin) for i in range(min(n, cap))]


# ---------------------------------------------------------------------------
# Multi-source alignment: LaserDisc VBI codes and MultiSourceAlignment,
# restated for the tests (src/metadata/vbi_decoder.cpp,
# src/dropout/multi_source_alignment.cpp, src/metadata/core.cpp).
# ---------------------------------------------------------------------------

def _bcd(v: int):
    """VbiDecoder::decodeBCD (vbi_decoder.cpp:650-668); None when a nibble is not a digit."""
    value, place = 0, 1
    while v:
        d = v & 0xF
        if d > 9:
            return None
        value += d * place
        place *= 10
        v >>= 4
    return value


def vbi_decode_field(l16: int, l17: int, l18: int) -> dict:
    """VbiDecoder::decode's CAV picture number and CLV time code
    (vbi_decoder.cpp:131-232, 575-604)."""
    r = dict(picNo=-1, clvHr=-1, clvMin=-1, clvSec=-1, clvPicNo=-1)
    if l16 == -1 and l17 == -1 and l18 == -1:
        return r
    for line in (l17, l18):
        line &= 0xFFFFFFFF
        if line & 0xF00000 == 0xF00000:
            v = _bcd(line & 0x07FFFF)
            if v is not None:
                r["picNo"] = v
    for line in (l17, l18):
        line &= 0xFFFFFFFF
        if line & 0xF0FF00 == 0xF0DD00:
            h = _bcd((line & 0x0F0000) >> 16)
            m = _bcd(line & 0xFF) if h is not None else None
            if m is not None:
                r["clvMin"], r["clvHr"] = m, h
    line = l16 & 0xFFFFFFFF
    if line & 0xF0F000 == 0x80E000:
        x1 = (line & 0x0F0000) >> 16
        if x1 >= 0xA:
            sec = _bcd((line & 0xF00) >> 8)
            pic = _bcd(line & 0xFF) if sec is not None else None
            if pic is not None:
                r["clvPicNo"], r["clvSec"], r["picNo"] = pic, 10 * (x1 - 0xA) + sec, -1
    return r


def vbi_decode_frame(first, second) -> dict:
    """VbiDecoder::decodeFrame (vbi_decoder.cpp:49-80): first field's code, else the second's."""
    a, b = vbi_decode_field(*first), vbi_decode_field(*second)
    return {k: (a[k] if a[k] != -1 else b[k]) for k in a}


def num_frames(is_first, first_field_first: bool) -> int:
    """LdDecodeMetaData::getNumberOfFrames (core.cpp:1092-1110)."""
    f1 = bool(is_first[0]) if is_first else False
    off = (0 if f1 else 1) if first_field_first else (1 if f1 else 0)
    return len(is_first) // 2 - off


def field_number(is_first, frame: int, which: int, first_field_first: bool) -> int:
    """getFirstFieldNumber / getSecondFieldNumber (core.cpp:1112-1190), 1-based; -1 when none."""
    if frame < 1:
        return -1
    if first_field_first:
        first = frame * 2 - 1
        second = first + 1
    else:
        second = frame * 2 - 1
        first = second + 1
    n = len(is_first)

    def isf(k):
        return 1 <= k <= n and bool(is_first[k - 1])

    while not isf(first):
        first += 1
        second += 1
        if first > n or second > n:
            return -1
    if first > n or second > n:
        return -1
    return first if which == 1 else second


def align_sources(sources):
    """MultiSourceAlignment over sources [(is_first per field, vbi per field
    [l16, l17, l18], first_field_first, is_pal)], source 0 the primary.
    Returns frame_for(primary_frame_1based, s) -> 1-based frame or -1
    (setMinAndMaxVbiFrames / sourceFrameForPrimaryFrame,
    multi_source_alignment.cpp:54-177)."""
    info = []
    for is_first, vbi, ffF, is_pal in sources:
        cav = []
        clv = []
        for f in range(1, num_frames(is_first, ffF) + 1):
            a, b = field_number(is_first, f, 1, ffF), field_number(is_first, f, 2, ffF)
            va = vbi[a - 1] if 1 <= a <= len(vbi) else (0, 0, 0)
            vb = vbi[b - 1] if 1 <= b <= len(vbi) else (0, 0, 0)
            v = vbi_decode_frame(va, vb)
            if v["picNo"] > 0:
                cav.append(v["picNo"])
            if -1 not in (v["clvHr"], v["clvMin"], v["clvSec"], v["clvPicNo"]):
                fps = 25 if is_pal else 30
                clv.append(v["clvHr"] * 3600 * fps + v["clvMin"] * 60 * fps + v["clvSec"] * fps + v["clvPicNo"])
        if not cav and not clv:
            info.append(None)
        elif len(cav) > len(clv):
            info.append((min(cav), max(cav)))
        else:
            info.append((min(clv), max(clv)))

    def frame_for(frame: int, s: int) -> int:
        if s == 0 or info[0] is None or info[s] is None:
            return frame
        v = info[0][0] - 1 + frame
        if info[s][0] <= v <= info[s][1]:
            return v - info[s][0] + 1
        return -1

    return frame_for
