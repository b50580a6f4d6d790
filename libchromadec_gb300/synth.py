"""Seeded synthetic PAL / PAL-M 4fsc composite generator (line-locked fields:
1135x313 for 625-line PAL, 909x263 for 525-line PAL-M).

The modulation follows the PAL maths the reference's own test encoder uses
(src/legacy/ld-chroma-decoder/encoder/palencoder.cpp:173-324): chroma is
U*sin(a) + V*cos(a)*Vsw with a = 2*pi*(fSC*t + prevCycles), prevCycles =
prevLines * 283.7516, Vsw = +1 on even prevLines, and a colourburst at
+/-135 degrees with peak-to-peak amplitude 3/7 of black..white. At 4fsc the
sample-index part of the phase is exactly x/4 cycles, so the subcarrier is
phased by integer sample index; the per-line remainder comes from prevCycles.

Levels are the reference's PAL preset (src/format/video_standards.cpp:18-26):
black 0x4000, white 0xD300, sync tip 0x0100. Geometry is the line-locked
preset (sync-start rows): burst [98, 138), active samples [177, 1125), active
frame lines 44..619. PAL-M (SynthConfig.standard = "PAL_M") follows the
reference's PAL_M preset (video_standards.cpp:28-40, 44-52, 85-100,
116-207): 909 samples x 263 lines per field at 4 fSC with fSC = 227.25 fH,
SMPTE ST 244 levels (black 282 x 64, white 800 x 64, sync tip 16 x 64),
burst [75, 95), active samples [124, 892), active frame lines 39..524.

Content (all seeded):
  * 75% colour bars in the top third of the picture (static);
  * a luma zone plate (radial chirp, 0 to 5 MHz at its rim);
  * Gaussian-blurred random U/V patches (sigma 20 px, amplitude +/-0.3);
  * optional panning of the zone plate and patches (px/field, line/field);
  * additive white Gaussian noise, sigma a fraction of white-black;
  * optional dropouts: runs of samples forced to 0x0100, returned as sidecar
    spans (startx, endx, fieldLine 1-based) like ld-decode's metadata.

The ground-truth component planes (Y, U, V) and the chroma-only composite
are available for the learned form and for PSNR measurement.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

FIELD_WIDTH = 1135
FIELD_HEIGHT = 313
BLACK = 0x4000
WHITE = 0xD300
BLANKING = 0x4000
SYNC_TIP = 0x0100
ACTIVE_START = 177
ACTIVE_END = 1125
BURST_START = 98
BURST_END = 138
FIRST_ACTIVE_FRAME_LINE = 44
LAST_ACTIVE_FRAME_LINE = 619
SAMPLE_RATE = 4.0 * 625.0 * 25.0 * (1135.0 / 4.0 + 1.0 / 625.0)
FSC = 283.75 * 15625.0 + 25.0

@dataclass(frozen=True)
class Standard:
    name: str                 # the sidecar's "system"
    field_width: int
    field_height: int
    lines_per_frame: int
    sample_rate: float
    fsc: float
    cycles_per_line: float    # subcarrier cycles per line (the encoder's phase step)
    black: int
    white: int
    blanking: int
    sync_tip: int
    active_start: int
    active_end: int
    burst_start: int
    burst_end: int
    first_active_frame_line: int
    last_active_frame_line: int
    sync_width: int           # samples of sync tip at the start of each line
    sync_level: float         # sync tip relative to black, in units of white - black
    zone_plate_y: float       # the zone plate's centre (frame line)


PAL = Standard("PAL", FIELD_WIDTH, FIELD_HEIGHT, 625, SAMPLE_RATE, FSC, 283.7516, BLACK, WHITE, BLANKING, SYNC_TIP,
               ACTIVE_START, ACTIVE_END, BURST_START, BURST_END, FIRST_ACTIVE_FRAME_LINE, LAST_ACTIVE_FRAME_LINE, 83,
               -0.3 / 0.7, 420.0)
PAL_M = Standard("PAL_M", 909, 263, 525, 4.0 * 525.0 * (30000.0 / 1001.0) * (909.0 / 4.0),
                 5.0e6 * (63.0 / 88.0) * (909.0 / 910.0), 909.0 / 4.0, 282 * 64, 800 * 64, 240 * 64, 16 * 64,
                 124, 892, 75, 95, 39, 524, 67, -(282.0 - 16.0) / (800.0 - 282.0), 356.0)
STANDARDS = {"PAL": PAL, "PAL_M": PAL_M}

# Composite U/V reduction factors at the "scientific" precision
# (src/common/color_conversion.cpp:25-27).
U_REDUCTION = 0.49211104112248356308804691718185
V_REDUCTION = 0.87728321993817866838972487283129


@dataclass
class SynthConfig:
    seed: int = 1
    pan_x: float = 0.0          # samples per field
    pan_y: float = 0.0          # frame lines per field
    noise: float = 0.005        # AWGN sigma as a fraction of white-black
    bars: bool = True
    zone_plate: bool = True
    patches: bool = True
    patch_amplitude: float = 0.3
    patch_sigma: float = 20.0
    dropout_line_fraction: float = 0.0
    dropout_min_len: int = 20
    dropout_max_len: int = 400
    saturation_edges: bool = False
    # Another capture of the same disc: the same pictures (content seeded by
    # `seed`) with its own noise and dropouts.
    noise_seed: Optional[int] = None
    dropout_seed: Optional[int] = None
    standard: str = "PAL"


@dataclass
class SynthCapture:
    fields: np.ndarray                       # (nfields, field_height, field_width) uint16
    dropouts: List[List[Tuple[int, int, int]]]  # per field: (startx, endx, fieldLine)
    y: Optional[np.ndarray] = None           # ground truth, same shape, float32
    u: Optional[np.ndarray] = None
    v: Optional[np.ndarray] = None
    chroma: Optional[np.ndarray] = None      # chroma-only composite, sample units
    standard: str = "PAL"


def _gaussian_kernel(sigma: float) -> np.ndarray:
    radius = max(1, int(np.ceil(3.0 * sigma)))
    t = np.arange(-radius, radius + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    return k / k.sum()


def _blur_periodic_2d(a: np.ndarray, sigma: float) -> np.ndarray:
    """Gaussian blur with wrap-around edges, via the Fourier transform."""
    ky = np.fft.fftfreq(a.shape[0])[:, None]
    kx = np.fft.rfftfreq(a.shape[1])[None, :]
    g = np.exp(-2.0 * (np.pi * sigma) ** 2 * (ky * ky + kx * kx))
    return np.fft.irfft2(np.fft.rfft2(a) * g, s=a.shape)


def _blur_axis(a: np.ndarray, sigma: float, axis: int) -> np.ndarray:
    k = _gaussian_kernel(sigma)
    r = (len(k) - 1) // 2
    pad = [(0, 0)] * a.ndim
    pad[axis] = (r, r)
    ap = np.pad(a, pad, mode="wrap")
    out = np.zeros_like(a)
    n = a.shape[axis]
    for i, w in enumerate(k):
        sl = [slice(None)] * a.ndim
        sl[axis] = slice(i, i + n)
        out += w * ap[tuple(sl)]
    return out


def _bars_rgb() -> np.ndarray:
    # white, yellow, cyan, green, magenta, red, blue, black at 75%
    bits = [(1, 1, 1), (1, 1, 0), (0, 1, 1), (0, 1, 0), (1, 0, 1), (1, 0, 0), (0, 0, 1), (0, 0, 0)]
    return 0.75 * np.array(bits, dtype=np.float64)


def _rgb_to_yuv(rgb: np.ndarray):
    r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
    y = 0.299 * r + 0.587 * g + 0.114 * b
    return y, U_REDUCTION * (b - y), V_REDUCTION * (r - y)


class PalEncoder:
    """Builds fields one at a time from a seeded content description."""

    def __init__(self, cfg: SynthConfig):
        self.cfg = cfg
        self.std = std = STANDARDS[cfg.standard]
        rng = np.random.default_rng(cfg.seed)
        self.rng = rng
        # Patch canvas, larger than the frame so panning never runs out.
        ch, cw = 640, 1280
        self.canvas_h, self.canvas_w = ch, cw
        if cfg.patches:
            cu = rng.standard_normal((ch, cw))
            cv = rng.standard_normal((ch, cw))
            cu = _blur_periodic_2d(cu, cfg.patch_sigma)
            cv = _blur_periodic_2d(cv, cfg.patch_sigma)
            cu *= cfg.patch_amplitude / (3.0 * cu.std())
            cv *= cfg.patch_amplitude / (3.0 * cv.std())
            self.canvas_u = np.clip(cu, -cfg.patch_amplitude, cfg.patch_amplitude)
            self.canvas_v = np.clip(cv, -cfg.patch_amplitude, cfg.patch_amplitude)
        else:
            self.canvas_u = np.zeros((ch, cw))
            self.canvas_v = np.zeros((ch, cw))
        self.zp_cx = 0.5 * (std.active_start + std.active_end) + rng.uniform(-40, 40)
        self.zp_cy = std.zone_plate_y + rng.uniform(-20, 20)
        self.zp_r = 240.0 * (std.active_end - std.active_start) / 948.0
        self.noise_rng = np.random.default_rng(cfg.seed + 7919 if cfg.noise_seed is None else cfg.noise_seed)
        x = np.arange(std.field_width, dtype=np.float64)
        # Raised-cosine gate for the active region (4-sample edges).
        self.active_gate = np.clip(np.minimum(x - (std.active_start - 4), (std.active_end + 3) - x) / 4.0, 0.0, 1.0)
        self.active_gate = 0.5 - 0.5 * np.cos(np.pi * self.active_gate)
        bg = np.clip(np.minimum(x - (std.burst_start - 2), (std.burst_end + 1) - x) / 3.0, 0.0, 1.0)
        self.burst_gate = 0.5 - 0.5 * np.cos(np.pi * bg)
        self.sync_gate = (x < std.sync_width).astype(np.float64)
        # Bars are static: build one band-limited row of Y, U, V.
        bar_w = (std.active_end - std.active_start) / 8.0
        idx = np.clip(np.floor((x - std.active_start) / bar_w), 0, 7).astype(np.int64)
        by, bu, bv = _rgb_to_yuv(_bars_rgb()[idx])
        # chroma band-limited like the encoder's 1.3 MHz Gaussian low-pass
        self.bar_row = (by, _blur_axis(bu[None, :], 1.5, 1)[0], _blur_axis(bv[None, :], 1.5, 1)[0])

    def components(self, field_index: int):
        """Y (0=black, 1=white), U, V planes for one field, (field_height, field_width)."""
        cfg = self.cfg
        std = self.std
        parity = field_index % 2
        fl = np.arange(std.field_height, dtype=np.float64)
        frame_y = 2.0 * fl + parity                      # frame line of each field line
        x = np.arange(std.field_width, dtype=np.float64)
        Y = np.full((std.field_height, std.field_width), 0.45)
        U = np.zeros_like(Y)
        V = np.zeros_like(Y)
        # Panned coordinates.
        px = x[None, :] - cfg.pan_x * field_index
        py = frame_y[:, None] - cfg.pan_y * field_index
        if cfg.zone_plate:
            # only the zone plate's bounding box is evaluated
            cxp = self.zp_cx + cfg.pan_x * field_index
            cyp = self.zp_cy + cfg.pan_y * field_index
            x0 = max(0, int(cxp - self.zp_r) - 1)
            x1 = min(std.field_width, int(cxp + self.zp_r) + 2)
            l0 = max(0, int((cyp - self.zp_r / 1.23 - parity) / 2) - 1)
            l1 = min(std.field_height, int((cyp + self.zp_r / 1.23 - parity) / 2) + 2)
            if x1 > x0 and l1 > l0:
                dx = px[:, x0:x1] - self.zp_cx
                dy = (py[l0:l1, :] - self.zp_cy) * 1.23
                r2 = dx * dx + dy * dy
                kmax = (5.0e6 / std.sample_rate) / self.zp_r   # cycles/sample per sample of radius
                zp = 0.25 * np.cos(np.pi * kmax * r2)
                Y[l0:l1, x0:x1] += np.where(r2 <= self.zp_r ** 2, zp, 0.0)
        if cfg.patches:
            # bilinear sample of the canvas at (py, px) offset into the canvas
            cy = py + 200.0
            cx = px + 300.0
            iy = np.floor(cy).astype(np.int64)
            ix = np.floor(cx).astype(np.int64)
            fy = cy - iy
            fx = cx - ix
            iy0 = np.mod(iy, self.canvas_h)
            iy1 = np.mod(iy + 1, self.canvas_h)
            ix0 = np.mod(ix, self.canvas_w)
            ix1 = np.mod(ix + 1, self.canvas_w)
            for canvas, dst in ((self.canvas_u, U), (self.canvas_v, V)):
                a = canvas[iy0, ix0] * (1 - fx) + canvas[iy0, ix1] * fx
                b = canvas[iy1, ix0] * (1 - fx) + canvas[iy1, ix1] * fx
                dst += a * (1 - fy) + b * fy
        if cfg.saturation_edges:
            # high-saturation vertical stripes moving with the pan
            stripe = (np.floor((px - 200.0) / 37.0) % 3 == 0) & (py > 300) & (py < 360)
            U = np.where(stripe, 0.45, U)
            V = np.where(stripe, -0.4, V)
        if cfg.saturation_edges:
            U = _blur_axis(U, 1.5, 1)
            V = _blur_axis(V, 1.5, 1)
        if cfg.bars:
            top = std.first_active_frame_line
            bottom = top + (std.last_active_frame_line - top + 1) // 3
            rows = (frame_y >= top) & (frame_y < bottom)
            by, bu, bv = self.bar_row
            Y[rows, :] = by[None, :]
            U[rows, :] = bu[None, :]
            V[rows, :] = bv[None, :]
        return Y, U, V

    def encode_field(self, field_index: int):
        """Composite uint16 field plus its ground truth (Y, U, V, chroma)."""
        std = self.std
        Y, U, V = self.components(field_index)
        fl = np.arange(std.field_height)
        field_id = field_index % 8
        prev_lines = (field_id // 2) * std.lines_per_frame + (field_id % 2) * std.field_height + fl
        vsw = np.where(prev_lines % 2 == 0, 1.0, -1.0)
        line_phase = np.mod(prev_lines * std.cycles_per_line, 1.0)        # cycles at 0H
        x = np.arange(std.field_width)
        # a = 2*pi*(x/4 + phase): sin/cos repeat every 4 samples, so build them
        # from each line's sin/cos of the 0H phase.
        th = 2.0 * np.pi * line_phase
        st, ct = np.sin(th), np.cos(th)
        s4 = np.stack([st, ct, -st, -ct], axis=1)            # sin(th + k*pi/2)
        c4 = np.stack([ct, -st, -ct, st], axis=1)            # cos(th + k*pi/2)
        s = s4[:, x % 4]
        c = c4[:, x % 4]
        active_rows = ((2 * fl + field_index % 2) >= std.first_active_frame_line) & \
                      ((2 * fl + field_index % 2) <= std.last_active_frame_line)
        gate = self.active_gate[None, :] * active_rows[:, None]
        chroma = (U * s + V * c * vsw[:, None]) * gate
        luma = Y * gate
        burst_rows = (fl >= 6) & (fl <= std.field_height - 4)
        off = vsw[:, None] * (135.0 * np.pi / 180.0)
        burst = (s * np.cos(off) + c * np.sin(off)) * (3.0 / 7.0) / 2.0
        burst = burst * self.burst_gate[None, :] * burst_rows[:, None]
        sync = std.sync_level * self.sync_gate[None, :]
        sig = luma + chroma + burst + sync
        if self.cfg.noise > 0:
            sig = sig + self.noise_rng.standard_normal(sig.shape) * self.cfg.noise
        samples = np.rint(std.black + (std.white - std.black) * sig)
        samples = np.clip(samples, std.sync_tip, 0xFEFF).astype(np.uint16)
        return samples, (Y * gate, U * gate, V * gate, chroma * (std.white - std.black))


def make_capture(nfields: int, cfg: SynthConfig, truth: bool = False) -> SynthCapture:
    enc = PalEncoder(cfg)
    std = enc.std
    fields = np.empty((nfields, std.field_height, std.field_width), dtype=np.uint16)
    ys = us = vs = cs = None
    if truth:
        ys = np.empty((nfields, std.field_height, std.field_width), dtype=np.float32)
        us = np.empty_like(ys)
        vs = np.empty_like(ys)
        cs = np.empty_like(ys)
    for f in range(nfields):
        samples, (Y, U, V, C) = enc.encode_field(f)
        fields[f] = samples
        if truth:
            ys[f], us[f], vs[f], cs[f] = Y, U, V, C
    dropouts: List[List[Tuple[int, int, int]]] = [[] for _ in range(nfields)]
    if cfg.dropout_line_fraction > 0:
        drng = np.random.default_rng(cfg.seed + 104729 if cfg.dropout_seed is None else cfg.dropout_seed)
        for f in range(nfields):
            for line in range(std.field_height):
                if drng.random() >= cfg.dropout_line_fraction:
                    continue
                length = int(drng.integers(cfg.dropout_min_len, cfg.dropout_max_len + 1))
                start = int(drng.integers(0, std.field_width - length))
                fields[f, line, start:start + length] = std.sync_tip
                dropouts[f].append((start, start + length, line + 1))
    return SynthCapture(fields=fields, dropouts=dropouts, y=ys, u=us, v=vs, chroma=cs, standard=cfg.standard)


def video_parameters_json(nfields: int, standard: str = "PAL") -> dict:
    std = STANDARDS[standard]
    return {
        "system": std.name,
        "fieldWidth": std.field_width,
        "fieldHeight": std.field_height,
        "sampleRate": std.sample_rate,
        "activeVideoStart": std.active_start,
        "activeVideoEnd": std.active_end,
        "colourBurstStart": std.burst_start,
        "colourBurstEnd": std.burst_end,
        "white16bIre": std.white,
        "black16bIre": std.black,
        "blanking16bIre": std.blanking,
        "isSubcarrierLocked": False,
        "isWidescreen": False,
        "isMapped": False,
        "numberOfSequentialFields": nfields,
    }


def _bcd(v: int) -> int:
    out, shift = 0, 0
    while True:
        out |= (v % 10) << shift
        v //= 10
        shift += 4
        if v == 0:
            return out


def cav_vbi(picture: int):
    """VBI lines 16-18 of a field carrying CAV picture number `picture`
    (IEC 60857-1986 10.1.3: 0xF00000 | BCD on lines 17 and 18)."""
    code = 0xF00000 | _bcd(picture)
    return [0, code, code]


def clv_vbi(hours: int, minutes: int, seconds: int, picture: int):
    """VBI lines 16-18 carrying a CLV time code (IEC 60857-1986 10.1.6 on
    line 17: 0xF0DD00 | BCD hour << 16 | BCD minutes; 10.1.10 on line 16:
    0x80E000 | (0xA + tens of seconds) << 16 | units << 8 | BCD picture)."""
    l17 = 0xF0DD00 | (_bcd(hours) << 16) | _bcd(minutes)
    l16 = 0x80E000 | ((0xA + seconds // 10) << 16) | ((seconds % 10) << 8) | _bcd(picture)
    return [l16, l17, 0]


def write_tbc(path: str, cap: SynthCapture, vbi=None, bpsnr=None) -> str:
    """Write an ld-decode style .tbc and its .tbc.json sidecar; returns the
    json path. vbi: per field [line16, line17, line18] or None; bpsnr: per
    field VITS bPSNR or None."""
    nfields = cap.fields.shape[0]
    with open(path, "wb") as fp:
        fp.write(np.ascontiguousarray(cap.fields).tobytes())
    meta = {
        "videoParameters": video_parameters_json(nfields, cap.standard),
        "fields": [],
    }
    for i in range(nfields):
        spans = cap.dropouts[i]
        fm = {
            "seqNo": i + 1,
            "isFirstField": (i % 2) == 0,
            "syncConf": 100,
            "dropOuts": {
                "startx": [s[0] for s in spans],
                "endx": [s[1] for s in spans],
                "fieldLine": [s[2] for s in spans],
            },
        }
        if vbi is not None and vbi[i] is not None:
            fm["vbi"] = {"vbiData": [int(v) for v in vbi[i]]}
        if bpsnr is not None:
            fm["vitsMetrics"] = {"bPSNR": float(bpsnr[i]), "wSNR": 0.0}
        meta["fields"].append(fm)
    jpath = path + ".json"
    with open(jpath, "w") as fp:
        json.dump(meta, fp)
    return jpath


def write_dropout_list(path: str, cap: SynthCapture) -> None:
    """Dropouts as text lines "field_index startx endx fieldLine"."""
    with open(path, "w") as fp:
        for i, spans in enumerate(cap.dropouts):
            for s in spans:
                fp.write(f"{i} {s[0]} {s[1]} {s[2]}\n")
