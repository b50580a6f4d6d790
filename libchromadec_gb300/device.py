"""ctypes binding of the device-level entry points (include/chromadec_gb300.h).

Device buffers are torch CUDA tensors (plumbing only: allocation, streams);
all compute runs in libchromadec_gb300.so. There is no CPU fallback: loading
fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

from . import _build

KIND_TRANSFORM_2D = 7
KIND_TRANSFORM_3D = 8
FMT_P16 = 0
FMT_PS = 1


class Geometry(C.Structure):
    _fields_ = [
        ("field_width", C.c_int32), ("field_height", C.c_int32),
        ("active_start", C.c_int32), ("active_end", C.c_int32),
        ("first_active_frame_line", C.c_int32), ("last_active_frame_line", C.c_int32),
        ("burst_start", C.c_int32), ("burst_end", C.c_int32),
        ("black", C.c_int32), ("white", C.c_int32),
        ("sample_rate", C.c_double), ("fsc", C.c_double),
    ]


class Config(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("threshold", C.c_double),
        ("thresholds", C.POINTER(C.c_double)), ("n_thresholds", C.c_int32),
        ("chroma_gain", C.c_double), ("chroma_phase_deg", C.c_double),
        ("output_format", C.c_int32), ("clamp_mode", C.c_int32), ("padding_multiple", C.c_int32),
        ("ecb_from_u", C.c_double), ("ecr_from_v", C.c_double),
        ("kr", C.c_double), ("kb", C.c_double), ("u_reduction", C.c_double), ("v_reduction", C.c_double),
        ("y_nr_level", C.c_double), ("first_field_offset", C.c_int32),
    ]


class Dropout(C.Structure):
    """chdg_dropout: one dropout span of a capture's field (field 0-based, field_line 1-based)."""
    _fields_ = [("field", C.c_int32), ("startx", C.c_int32), ("endx", C.c_int32), ("field_line", C.c_int32)]


CONCEAL = 1
CONCEAL_OVERCORRECT = 2
CONCEAL_INTRA = 4


class Capture(C.Structure):
    """chdg_capture: one capture of a batch (device buffers; dropouts on the host)."""
    _fields_ = [("fields", C.c_void_p), ("field_stride", C.c_int64), ("nfields", C.c_int32), ("kind", C.c_int32),
                ("threshold", C.c_double), ("out", C.c_void_p), ("dropouts", C.POINTER(Dropout)),
                ("ndropouts", C.c_int32), ("conceal", C.c_int32), ("mask_out", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("chunk_frames", C.c_int32), ("max_blocks", C.c_int32), ("ms", C.c_float)]


_lib = None


def lib(build: bool = True):
    """Load libchromadec_gb300.so (building it in-tree if needed)."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("libchromadec_gb300.so is missing; run __graft_entry__.build()")
        L = C.CDLL(path)
        L.chdg_default_geometry.argtypes = [C.POINTER(Geometry)]
        L.chdg_default_config.argtypes = [C.POINTER(Config), C.c_int32]
        L.chdg_engine_create.argtypes = [C.POINTER(Geometry), C.POINTER(Config), C.POINTER(C.c_void_p)]
        L.chdg_engine_free.argtypes = [C.c_void_p]
        L.chdg_output_geometry.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.POINTER(C.c_size_t)]
        L.chdg_decode_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_void_p, C.c_void_p]
        L.chdg_chroma_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_void_p, C.c_void_p]
        L.chdg_engine_stats.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.chdg_decode_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_void_p, C.c_void_p]
        L.chdg_engine_set_profiling.argtypes = [C.c_void_p, C.c_int]
        L.chdg_batch_create.argtypes = [C.POINTER(Geometry), C.POINTER(Config), C.POINTER(C.c_void_p)]
        L.chdg_batch_free.argtypes = [C.c_void_p]
        L.chdg_batch_decode.argtypes = [C.c_void_p, C.POINTER(Capture), C.c_int32, C.c_void_p]
        L.chdg_batch_autotune.argtypes = [C.c_void_p, C.POINTER(Capture), C.c_int32, C.c_void_p,
                                          C.POINTER(BatchTuning)]
        L.chdg_engine_kernel_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.POINTER(C.c_int64)]
        L.chdg_tc3d_spectra.argtypes = [C.POINTER(Geometry), C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                                        C.c_int32, C.c_void_p, C.c_void_p]
        L.chdg_tc3d_sync.argtypes = [C.c_void_p]
        L.chdg_engine_set_tc_form.argtypes = [C.c_void_p, C.c_int32]
        L.chdg_engine_set_max_batch_frames.argtypes = [C.c_void_p, C.c_int32]
        L.chdg_tc3d_operand.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]
        L.chdg_masknet_create.argtypes = [C.POINTER(C.c_void_p)]
        L.chdg_masknet_free.argtypes = [C.c_void_p]
        L.chdg_masknet_set_weights.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64]
        L.chdg_masknet_get_weights.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64]
        L.chdg_masknet_set_confidence.argtypes = [C.c_void_p, C.c_float]
        L.chdg_masknet_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
        L.chdg_masknet_train_step.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float,
                                              C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_void_p]
        L.chdg_masknet_set_tensor_cores.argtypes = [C.c_void_p, C.c_int32]
        L.chdg_masknet_sync.argtypes = [C.c_void_p, C.c_void_p]
        L.chdg_masknet_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.chdg_learned_features.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.chdg_learned_chroma.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.chdg_engine_set_masknet.argtypes = [C.c_void_p, C.c_void_p]
        L.chdg_engine_learned_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.chd_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def last_error() -> str:
    return lib().chd_last_error().decode(errors="replace")


def default_geometry() -> Geometry:
    g = Geometry()
    lib().chdg_default_geometry(C.byref(g))
    return g


def default_config(kind: int = KIND_TRANSFORM_3D, fmt: int = FMT_P16, threshold: float = 0.4,
                   thresholds: Optional[Sequence[float]] = None, **kw) -> Config:
    c = Config()
    lib().chdg_default_config(C.byref(c), kind)
    c.output_format = fmt
    c.threshold = threshold
    if thresholds is not None:
        arr = (C.c_double * len(thresholds))(*thresholds)
        c._keep = arr
        c.thresholds = arr
        c.n_thresholds = len(thresholds)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class Engine:
    """One device pipeline (constant tables + scratch) for a geometry/config."""

    def __init__(self, geometry: Optional[Geometry] = None, config: Optional[Config] = None):
        self.geometry = geometry or default_geometry()
        self.config = config or default_config()
        h = C.c_void_p()
        rc = lib().chdg_engine_create(C.byref(self.geometry), C.byref(self.config), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"chdg_engine_create failed ({rc}): {last_error()}")
        self._h = h
        w, hh, fb = C.c_int32(), C.c_int32(), C.c_size_t()
        lib().chdg_output_geometry(self._h, C.byref(w), C.byref(hh), C.byref(fb))
        self.out_width, self.out_height, self.frame_bytes = w.value, hh.value, fb.value

    def close(self):
        if getattr(self, "_h", None):
            lib().chdg_engine_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _stream_ptr(stream):
        return C.c_void_p(stream.cuda_stream if stream is not None else 0)

    def decode(self, fields, frame_begin: int, frame_end: int, out, stream=None, field_stride: Optional[int] = None,
               nfields: Optional[int] = None):
        """fields: uint16 CUDA tensor (nfields, stride) or (nfields, h, w); out: CUDA tensor of
        (frame_end-frame_begin) frames."""
        stride = field_stride if field_stride is not None else fields[0].numel()
        nf = nfields if nfields is not None else fields.shape[0]
        rc = lib().chdg_decode_device(self._h, C.c_void_p(fields.data_ptr()), stride, nf, frame_begin, frame_end,
                                      C.c_void_p(out.data_ptr()), self._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_decode_device failed ({rc}): {last_error()}")

    def chroma(self, fields, frame_begin: int, frame_end: int, out, stream=None, field_stride: Optional[int] = None,
               nfields: Optional[int] = None):
        stride = field_stride if field_stride is not None else fields[0].numel()
        nf = nfields if nfields is not None else fields.shape[0]
        rc = lib().chdg_chroma_device(self._h, C.c_void_p(fields.data_ptr()), stride, nf, frame_begin, frame_end,
                                      C.c_void_p(out.data_ptr()), self._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_chroma_device failed ({rc}): {last_error()}")

    def set_max_batch_frames(self, frames: int):
        """Frames per GPU batch of decode() (default 256): bounds the scratch memory."""
        rc = lib().chdg_engine_set_max_batch_frames(self._h, frames)
        if rc != 0:
            raise RuntimeError(f"chdg_engine_set_max_batch_frames failed ({rc}): {last_error()}")

    def set_tc_form(self, variant: int):
        """-1: the plain form; TC_3XTF32 / TC_BF16X3: the tensor-core form."""
        rc = lib().chdg_engine_set_tc_form(self._h, variant)
        if rc != 0:
            raise RuntimeError(f"chdg_engine_set_tc_form failed ({rc}): {last_error()}")

    def stats(self):
        a, b = C.c_uint64(), C.c_uint64()
        lib().chdg_engine_stats(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_masknet(self, net: Optional["MaskNet"]):
        """The learned form with `net`, or the plain form (None)."""
        rc = lib().chdg_engine_set_masknet(self._h, net._h if net is not None else None)
        if rc != 0:
            raise RuntimeError(f"chdg_engine_set_masknet failed ({rc}): {last_error()}")
        self._net = net   # borrowed by the engine: keep it alive

    def learned_stats(self):
        t, f = C.c_int64(), C.c_int64()
        rc = lib().chdg_engine_learned_stats(self._h, C.byref(t), C.byref(f))
        if rc != 0:
            raise RuntimeError(f"chdg_engine_learned_stats failed ({rc}): {last_error()}")
        return t.value, f.value

    def ntiles(self) -> int:
        """Spatial tiles of the 3D transform (chdg_tc3d_spectra's order)."""
        g = self.geometry
        ntx = (g.active_end - g.active_start + 8 + 7) // 8
        nty = (g.last_active_frame_line - g.first_active_frame_line + 16) // 16 + 1
        return ntx * nty

    def learned_features(self, fields, frame_begin: int, frame_end: int, feat, spec=None, threshold_p=None,
                         stream=None):
        """Features (bf16 bits as int16/uint16 tensor) of the Z tiles of
        frames [frame_begin, frame_end): (frame_end - frame_begin + 2) x ntiles x 1280."""
        rc = lib().chdg_learned_features(self._h, C.c_void_p(fields.data_ptr()), fields[0].numel(), fields.shape[0],
                                         frame_begin, frame_end, C.c_void_p(feat.data_ptr()),
                                         C.c_void_p(spec.data_ptr()) if spec is not None else None,
                                         C.c_void_p(threshold_p.data_ptr()) if threshold_p is not None else None,
                                         self._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_learned_features failed ({rc}): {last_error()}")

    def learned_chroma(self, fields, frame_begin: int, frame_end: int, p, fallback, out, stream=None):
        rc = lib().chdg_learned_chroma(self._h, C.c_void_p(fields.data_ptr()), fields[0].numel(), fields.shape[0],
                                       frame_begin, frame_end, C.c_void_p(p.data_ptr()),
                                       C.c_void_p(fallback.data_ptr()), C.c_void_p(out.data_ptr()),
                                       self._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_learned_chroma failed ({rc}): {last_error()}")


class Batch:
    """chdg_batch: many captures (mixed Transform 2D/3D, one threshold each)
    decoded by one launch per mode, replayed from a CUDA graph."""

    def __init__(self, geometry: Optional[Geometry] = None, config: Optional[Config] = None):
        self.geometry = geometry or default_geometry()
        self.config = config or default_config()
        h = C.c_void_p()
        rc = lib().chdg_batch_create(C.byref(self.geometry), C.byref(self.config), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"chdg_batch_create failed ({rc}): {last_error()}")
        self._h = h

    @staticmethod
    def captures(items):
        """items: (fields tensor (n, stride), kind, threshold, out tensor) tuples, optionally followed by
        (dropouts [(field, startx, endx, fieldLine)], conceal flags, mask tensor or None)."""
        arr = (Capture * len(items))()
        keep = []
        for i, it in enumerate(items):
            f, kind, thr, out = it[:4]
            drops, conceal, mask = (list(it[4]), int(it[5]), it[6]) if len(it) > 4 else ([], 0, None)
            d = (Dropout * max(1, len(drops)))(*[Dropout(*x) for x in drops])
            keep.append(d)
            arr[i] = Capture(f.data_ptr(), f[0].numel(), f.shape[0], kind, thr, out.data_ptr(),
                             C.cast(d, C.POINTER(Dropout)), len(drops), conceal,
                             mask.data_ptr() if mask is not None else None)
        arr._keep = keep
        return arr

    def decode(self, caps, stream=None):
        rc = lib().chdg_batch_decode(self._h, caps, len(caps), Engine._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_batch_decode failed ({rc}): {last_error()}")

    def autotune(self, caps, stream=None) -> BatchTuning:
        t = BatchTuning()
        rc = lib().chdg_batch_autotune(self._h, caps, len(caps), Engine._stream_ptr(stream), C.byref(t))
        if rc != 0:
            raise RuntimeError(f"chdg_batch_autotune failed ({rc}): {last_error()}")
        return t

    def close(self):
        if self._h:
            lib().chdg_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TC_3XTF32 = 0
TC_BF16X3 = 1


def tc3d_spectra(fields, m_begin: int, m_end: int, spec, variant: int = TC_3XTF32, stream=None,
                 geometry: Optional[Geometry] = None, field_stride: Optional[int] = None,
                 nfields: Optional[int] = None):
    """chdg_tc3d_spectra: tensor-core spectra of Z tiles [m_begin, m_end) into
    spec, a complex64 (or float32 (..., 2)) CUDA tensor of
    (m_end - m_begin) x ntiles x 8 x 5 x 32 bins."""
    g = geometry or default_geometry()
    stride = field_stride if field_stride is not None else fields[0].numel()
    nf = nfields if nfields is not None else fields.shape[0]
    ntx = (g.active_end - g.active_start + 8 + 7) // 8
    nty = (g.last_active_frame_line - g.first_active_frame_line + 16) // 16 + 1
    need = (m_end - m_begin) * ntx * nty * 8 * 5 * 32 * 8
    if m_end <= m_begin or spec.numel() * spec.element_size() < need or not spec.is_contiguous():
        raise ValueError(f"spec must be a contiguous buffer of at least {need} bytes")
    rc = lib().chdg_tc3d_spectra(C.byref(g), variant, C.c_void_p(fields.data_ptr()), stride, nf, m_begin, m_end,
                                 C.c_void_p(spec.data_ptr()), Engine._stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"chdg_tc3d_spectra failed ({rc}): {last_error()}")


def tc3d_sync(stream=None):
    rc = lib().chdg_tc3d_sync(Engine._stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"chdg_tc3d_sync failed ({rc}): {last_error()}")


def tc3d_operand(variant: int, stage: int, y0: int = 0, split: int = 0) -> bytes:
    """Host-built shared-memory image of one tensor-core coefficient operand."""
    buf = (C.c_uint8 * 65536)()
    n = lib().chdg_tc3d_operand(variant, stage, y0, split, buf, len(buf))
    if n < 0:
        raise RuntimeError(f"chdg_tc3d_operand failed ({n}): {last_error()}")
    return bytes(buf[:n])


MASKNET_PARAMS = 14753
MASKNET_BINS = 1280


class MaskNet:
    """chdg_masknet: the learned form's per-bin chroma-fraction network."""

    def __init__(self, weights=None):
        h = C.c_void_p()
        rc = lib().chdg_masknet_create(C.byref(h))
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_create failed ({rc}): {last_error()}")
        self._h = h
        if weights is not None:
            self.set_weights(weights)

    def set_weights(self, w):
        import numpy as np
        a = np.ascontiguousarray(w, dtype=np.float32)
        if a.size != MASKNET_PARAMS:
            raise ValueError(f"expected {MASKNET_PARAMS} parameters, got {a.size}")
        rc = lib().chdg_masknet_set_weights(self._h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size)
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_set_weights failed ({rc}): {last_error()}")

    def weights(self):
        import numpy as np
        a = np.empty(MASKNET_PARAMS, dtype=np.float32)
        rc = lib().chdg_masknet_get_weights(self._h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size)
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_get_weights failed ({rc}): {last_error()}")
        return a

    def set_confidence(self, limit: float):
        rc = lib().chdg_masknet_set_confidence(self._h, limit)
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_set_confidence failed ({rc}): {last_error()}")

    def set_tensor_cores(self, on: bool):
        rc = lib().chdg_masknet_set_tensor_cores(self._h, 1 if on else 0)
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_set_tensor_cores failed ({rc}): {last_error()}")

    def sync(self, stream=None):
        rc = lib().chdg_masknet_sync(self._h, Engine._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_sync failed ({rc}): {last_error()}")

    def forward(self, feat, ntiles: int, p, fallback=None, stream=None):
        rc = lib().chdg_masknet_forward(self._h, C.c_void_p(feat.data_ptr()), ntiles, C.c_void_p(p.data_ptr()),
                                        C.c_void_p(fallback.data_ptr()) if fallback is not None else None,
                                        Engine._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_forward failed ({rc}): {last_error()}")

    def train_step(self, feat, ac, ntiles: int, lr: float, want_loss: bool = True, want_grad: bool = False,
                   stream=None):
        """One step (lr = 0: gradient only). Returns (loss or None, grad or None)."""
        import numpy as np
        loss = C.c_double()
        grad = np.empty(MASKNET_PARAMS, dtype=np.float32) if want_grad else None
        rc = lib().chdg_masknet_train_step(self._h, C.c_void_p(feat.data_ptr()), C.c_void_p(ac.data_ptr()), ntiles,
                                           lr, C.byref(loss) if want_loss else None,
                                           grad.ctypes.data_as(C.POINTER(C.c_float)) if want_grad else None,
                                           Engine._stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"chdg_masknet_train_step failed ({rc}): {last_error()}")
        return (loss.value if want_loss else None), grad

    def close(self):
        if getattr(self, "_h", None):
            lib().chdg_masknet_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def masknet_pairs(spec_x, spec_c, nbins: int, ac, stream=None):
    rc = lib().chdg_masknet_pairs(C.c_void_p(spec_x.data_ptr()), C.c_void_p(spec_c.data_ptr()), nbins,
                                  C.c_void_p(ac.data_ptr()), Engine._stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"chdg_masknet_pairs failed ({rc}): {last_error()}")
