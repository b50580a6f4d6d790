"""Host-side behaviour of the chd_* ABI, no GPU needed.

Covers what the reference's own ABI tests check without decoding
(tests/unit/test_dropout_spans_abi.cpp, test_error_propagation.cpp,
test_log_abi.cpp, test_tbc_json_reader.cpp): every declared symbol is
exported, sources open with the reference's statuses, options are accepted
and rejected per kind, commit validates in the reference's order, and
dropout spans of a CHD_DEC_NONE decoder match the oracle bit for bit.
"""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from libchromadec_gb300 import abi, synth
from oracle import oracle
from tests._capture import capture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    hdrs = [os.path.join(ROOT, "include", "chromadec_gb300.h")]
    d = os.path.join(ROOT, "include", "chromadec")
    hdrs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".h")]
    for h in hdrs:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(chdg?_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = abi.lib()
    missing = [n for n in _declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert len(_declared_functions()) >= 70


def test_version_features_status_names():
    L = abi.lib()
    assert L.chd_version_string() == b"0.2.1"
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    L.chd_version(C.byref(a), C.byref(b), C.byref(c))
    assert (a.value, b.value, c.value) == (0, 2, 1)
    assert L.chd_has_feature(b"cuda") == 1 and L.chd_has_feature(b"nn") == 0 and L.chd_has_feature(None) == 0
    assert abi.status_name(abi.E_OUT_OF_RANGE) == "CHD_E_OUT_OF_RANGE"
    assert abi.status_name(999) == "CHD_E_UNKNOWN"
    assert L.chd_init() == 0


def test_log_api_levels_and_sink():
    L = abi.lib()
    assert L.chd_get_log_level() == 1                    # INFO by default
    assert L.chd_log_is_enabled(3) == 0                   # no sink installed yet
    got = []
    fn = abi.LOG_FN(lambda lvl, flags, msg, user: got.append((lvl, flags, msg)))
    L.chd_set_log_callback(fn, None)
    try:
        assert L.chd_log_is_enabled(3) == 1 and L.chd_log_is_enabled(0) == 0
        L.chd_set_log_level(-5)
        assert L.chd_get_log_level() == 0                 # clamped to DEBUG
        L.chd_set_log_level(99)
        assert L.chd_get_log_level() == 4                 # clamped to OFF
        assert L.chd_log_is_enabled(3) == 0
        assert L.chd_log_is_enabled(4) == 0               # OFF is never a message level
        assert L.chd_log_level_str(2) == b"WARN" and L.chd_log_level_str(77) == b"UNKNOWN"
    finally:
        L.chd_set_log_level(1)
        L.chd_set_log_callback(abi.LOG_FN(), None)


def test_nn_calls_answer_as_a_build_without_backend():
    L = abi.lib()
    L.chd_nn_backend_set_library_path.argtypes = [C.c_int, C.c_char_p]
    assert L.chd_nn_backend_set_library_path(12, None) == abi.E_UNSUPPORTED
    assert L.chd_nn_backend_set_library_path(3, None) == abi.E_INVALID_ARG
    L.chd_nn_backend_is_available.argtypes = [C.c_int]
    assert L.chd_nn_backend_is_available(12) == 0
    L.chd_nn_model_load_from_file.argtypes = [C.c_char_p, C.c_void_p, C.POINTER(C.c_void_p)]
    m = C.c_void_p()
    assert L.chd_nn_model_load_from_file(b"x.onnx", None, C.byref(m)) == abi.E_INTERNAL


@pytest.fixture(scope="module")
def pal_tbc(tmp_path_factory):
    d = tmp_path_factory.mktemp("pal")
    cap = capture(8, 7, dropouts=0.02)
    path = str(d / "cap.tbc")
    synth.write_tbc(path, cap)
    return path, cap


def test_open_statuses(tmp_path, pal_tbc):
    L = abi.lib()
    v = C.c_void_p()
    assert L.chd_video_open_composite(str(tmp_path / "none.tbc").encode(), None, None, C.byref(v)) == \
        abi.E_FILE_NOT_FOUND
    raw = tmp_path / "raw.tbc"
    raw.write_bytes(b"\0" * 16)
    assert L.chd_video_open_composite(str(raw).encode(), None, None, C.byref(v)) == abi.E_METADATA_MISSING
    (tmp_path / "raw.tbc.db").write_bytes(b"SQLite format 3\0")
    assert L.chd_video_open_composite(str(raw).encode(), None, None, C.byref(v)) == abi.E_FORMAT_UNSUPPORTED
    bad = tmp_path / "bad.json"
    bad.write_text("{ not json")
    assert L.chd_video_open_composite(str(raw).encode(), str(bad).encode(), None, C.byref(v)) == \
        abi.E_METADATA_CORRUPT
    assert b"bad.json" in L.chd_last_error()
    assert L.chd_video_open_composite(None, None, None, C.byref(v)) == abi.E_INVALID_ARG
    path, _ = pal_tbc
    assert L.chd_video_open_yc(path.encode(), path.encode(), None, None, C.byref(v)) == abi.E_UNSUPPORTED


def test_video_info_and_conversions(pal_tbc):
    path, cap = pal_tbc
    v = abi.Video(path)
    i = v.info()
    assert (i.standard, i.encoding, i.signal_state, i.layout) == (2, 2, 2, 1)
    assert (i.field_width, i.field_height, i.samples_per_frame) == (1135, 313, 709379)
    assert (i.first_active_sample, i.last_active_sample) == (177, 1124)
    assert (i.first_active_frame_line, i.last_active_frame_line) == (44, 619)
    assert (i.black_16b_ire, i.white_16b_ire, i.num_frames, i.is_first_field_first) == (0x4000, 0xD300, 4, 1)
    assert abs(i.fsc_hz - 4433618.75) < 1e-6 and abs(i.sample_rate_hz - 4 * 4433618.75) < 1e-3
    L = abi.lib()
    o = C.c_int32()
    # woven frame line <-> field-sequential signal line
    for fl, sl in ((0, 1), (1, 314), (2, 2), (624, 313)):
        assert L.chd_video_frame_line_to_signal_line(v._h, fl, C.byref(o)) == 0 and o.value == sl
        assert L.chd_video_signal_line_to_frame_line(v._h, sl, C.byref(o)) == 0 and o.value == fl
    assert L.chd_video_frame_line_to_signal_line(v._h, 625, C.byref(o)) == abi.E_OUT_OF_RANGE
    assert L.chd_video_signal_line_to_frame_line(v._h, 0, C.byref(o)) == abi.E_OUT_OF_RANGE
    # line-locked rows start at 0H: standard sample 0 is row sample 1135 - ceil(948 + 9.5) = 177
    assert L.chd_video_standard_sample_to_row_sample(v._h, 0, C.byref(o)) == 0 and o.value == 177
    assert L.chd_video_standard_sample_to_row_sample(v._h, 1000, C.byref(o)) == 0 and o.value == 42
    assert L.chd_video_row_sample_to_standard_sample(v._h, 42, C.byref(o)) == 0 and o.value == 1000
    assert L.chd_video_row_sample_to_standard_sample(v._h, 1135, C.byref(o)) == abi.E_OUT_OF_RANGE


def test_option_applicability(pal_tbc):
    path, _ = pal_tbc
    v = abi.Video(path)
    L = abi.lib()
    d3 = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    assert L.chd_decoder_set_option_f64(d3._h, b"transform_threshold", 0.5) == 0
    assert L.chd_decoder_set_option_str(d3._h, b"transform_thresholds_file", b"t.txt") == 0
    assert L.chd_decoder_set_option_f64(d3._h, b"chroma_gain", 1.5) == 0
    assert L.chd_decoder_set_option_f64(d3._h, b"chroma_nr_level", 1.0) == abi.E_INVALID_ARG
    assert L.chd_decoder_set_option_i32(d3._h, b"transform_threshold", 1) == abi.E_INVALID_ARG   # wrong type
    assert L.chd_decoder_set_option_str(d3._h, b"output_format", None) == abi.E_INVALID_ARG
    assert L.chd_decoder_has_option(d3._h, b"padding_multiple") == 0
    assert L.chd_decoder_has_option(d3._h, b"comb_show_map") == abi.E_INVALID_ARG
    d2p = abi.Decoder(v, abi.DEC_PAL_2D)
    assert L.chd_decoder_set_option_f64(d2p._h, b"transform_threshold", 0.5) == abi.E_INVALID_ARG
    assert L.chd_decoder_set_option_f64(d2p._h, b"luma_nr_level", 1.0) == 0
    auto = abi.Decoder(v, abi.DEC_AUTO)
    assert L.chd_decoder_set_option_f64(auto._h, b"chroma_phase_deg", 3.0) == 0
    assert L.chd_decoder_set_option_f64(auto._h, b"transform_threshold", 0.5) == abi.E_INVALID_ARG


def _commit_status(v, kind, **opts):
    d = abi.Decoder(v, kind)
    for k, val in opts.items():
        d.set(k, val)
    st = abi.lib().chd_decoder_commit(d._h)
    return st, d


def test_commit_validation_order(pal_tbc, tmp_path):
    path, _ = pal_tbc
    v = abi.Video(path)
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, padding_multiple=0)[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, padding_multiple=1025)[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, output_format="yuv420p")[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, output_clamp="loud")[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, color_difference_precision="x")[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, broadcast_scaling_precision="x")[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, output_format="yuv440ps")[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, first_active_sample=2000)[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, last_active_frame_line=625)[0] == abi.E_INVALID_ARG
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, first_active_frame_line=300,
                          last_active_frame_line=200)[0] == abi.E_INVALID_ARG
    assert _commit_status(v, 99)[0] == abi.E_DECODER_UNKNOWN
    assert _commit_status(v, abi.DEC_MONO)[0] == abi.E_UNSUPPORTED
    assert _commit_status(v, abi.DEC_NTSC_2D)[0] == abi.E_UNSUPPORTED
    # supported configurations pass validation; without a GPU the commit
    # then stops at the device (no CPU fallback)
    for kind, opts in ((abi.DEC_AUTO, {}), (abi.DEC_PAL_2D, {"luma_nr_level": 2.0}),
                       (abi.DEC_TRANSFORM_3D, {"output_format": "rgb48"}),
                       (abi.DEC_TRANSFORM_2D, {"output_format": "grays", "reverse_field_order": True})):
        assert _commit_status(v, kind, **opts)[0] in (abi.OK, abi.E_INTERNAL)
    thr = tmp_path / "short.txt"
    thr.write_text(" ".join(["0.5"] * 100))
    assert _commit_status(v, abi.DEC_TRANSFORM_3D, transform_thresholds_file=str(thr))[0] == \
        abi.E_DECODER_INCOMPATIBLE
    # decode before commit
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    f = C.c_void_p()
    assert abi.lib().chd_decode_frame(d._h, 0, C.byref(f)) == abi.E_INVALID_ARG
    o = abi.OutputInfo()
    assert abi.lib().chd_decoder_get_output_info(d._h, C.byref(o)) == abi.E_INVALID_ARG


def test_ntsc_source_is_incompatible(tmp_path):
    ntsc = _write_ntsc_capture(tmp_path, [])
    v = abi.Video(ntsc)
    assert _commit_status(v, abi.DEC_TRANSFORM_3D)[0] == abi.E_DECODER_INCOMPATIBLE


def _write_ntsc_capture(tmp_path, dropouts, nfields=4):
    w, h = 910, 263
    path = str(tmp_path / "do.tbc")
    np.full((nfields, h, w), 17920, dtype=np.uint16).tofile(path)
    fields = []
    for i in range(nfields):
        mine = [d for d in dropouts if d[0] == i]
        fields.append({"seqNo": i + 1, "isFirstField": i % 2 == 0,
                       "dropOuts": {"startx": [d[1] for d in mine], "endx": [d[2] for d in mine],
                                    "fieldLine": [d[3] for d in mine]}})
    meta = {"videoParameters": {"system": "NTSC", "fieldWidth": w, "fieldHeight": h, "sampleRate": 14318181.8,
                                "activeVideoStart": 147, "activeVideoEnd": 894, "colourBurstStart": 78,
                                "colourBurstEnd": 110, "white16bIre": 51200, "black16bIre": 17920,
                                "numberOfSequentialFields": nfields},
            "fields": fields}
    with open(path + ".json", "w") as fp:
        json.dump(meta, fp)
    return path


def _write_vbi_capture(tmp_path, name, nframes, vbi_of_frame, nfields=None, first_is_first=True):
    """A small PAL .tbc whose fields carry VBI lines from vbi_of_frame(k)
    (frame k = fields 2k, 2k+1; both fields carry the frame's code, as in the
    reference's test_multi_source_alignment.cpp), or none when it returns None."""
    n = nfields if nfields is not None else 2 * nframes
    cap = synth.SynthCapture(fields=np.full((n, 313, 1135), 0x4000, dtype=np.uint16), dropouts=[[] for _ in range(n)])
    vbi = [vbi_of_frame(i // 2) for i in range(n)]
    path = str(tmp_path / name)
    synth.write_tbc(path, cap, vbi=vbi)
    if not first_is_first:
        meta = json.load(open(path + ".json"))
        for i, f in enumerate(meta["fields"]):
            f["isFirstField"] = (i % 2) == 1
        json.dump(meta, open(path + ".json", "w"))
    return path


def test_extra_source_statuses(tmp_path, pal_tbc):
    """chd_video_add_extra_source_* (src/abi/c_api_video.cpp:631-897): null
    arguments, missing files, the Y/C pair checks, and this library's own
    rule that an extra shares the primary's field geometry."""
    path, _ = pal_tbc
    v = abi.Video(path)
    L = abi.lib()
    assert L.chd_video_add_extra_source_composite(None, path.encode(), None) == abi.E_INVALID_ARG
    assert L.chd_video_add_extra_source_composite(v._h, None, None) == abi.E_INVALID_ARG
    assert L.chd_video_add_extra_source_composite(v._h, str(tmp_path / "none.tbc").encode(), None) == \
        abi.E_FILE_NOT_FOUND
    ntsc = _write_ntsc_capture(tmp_path, [])
    assert L.chd_video_add_extra_source_composite(v._h, ntsc.encode(), None) == abi.E_FORMAT_UNSUPPORTED
    assert b"geometry" in L.chd_last_error()
    assert L.chd_video_add_extra_source_composite(v._h, path.encode(), None) == 0
    # Y/C: luma sidecar shared by the chroma plane
    luma = _write_vbi_capture(tmp_path, "yc.tbc", 2, lambda k: None)
    chroma = str(tmp_path / "yc_chroma.tbc")
    np.full((4, 313, 1135), 0x4000, dtype=np.uint16).tofile(chroma)
    assert L.chd_video_add_extra_source_yc(v._h, luma.encode(), None, None) == abi.E_INVALID_ARG
    assert L.chd_video_add_extra_source_yc(v._h, luma.encode(), str(tmp_path / "x").encode(), None) == \
        abi.E_FILE_NOT_FOUND
    short = str(tmp_path / "short_chroma.tbc")
    np.full((2, 313, 1135), 0x4000, dtype=np.uint16).tofile(short)
    meta = json.load(open(luma + ".json"))
    meta["fields"] = meta["fields"][:2]
    json.dump(meta, open(short + ".json", "w"))
    assert L.chd_video_add_extra_source_yc(v._h, luma.encode(), short.encode(), None) == abi.E_FORMAT_UNSUPPORTED
    assert L.chd_video_add_extra_source_yc(v._h, luma.encode(), chroma.encode(), None) == 0
    o = C.c_int32()
    assert L.chdg_video_source_frame(v._h, 0, 3, 0, C.byref(o)) == abi.E_OUT_OF_RANGE
    assert L.chdg_video_source_frame(v._h, 0, 2, 1, C.byref(o)) == 0 and o.value == 1   # no VBI: positional


def _cav(pic):
    return None if pic is None else [0, 0xF00000 | int(str(pic), 16), 0]


def test_multi_source_alignment_known_answers(tmp_path):
    """The reference's own alignment test (tests/unit/test_multi_source_alignment.cpp)
    through chdg_video_source_frame: a primary holding CAV pictures 100..109,
    extra A 105..114, extra B without VBI; then the reversed pairing."""
    L = abi.lib()
    prim = _write_vbi_capture(tmp_path, "p.tbc", 10, lambda k: _cav(100 + k))
    a = _write_vbi_capture(tmp_path, "a.tbc", 10, lambda k: _cav(105 + k))
    b = _write_vbi_capture(tmp_path, "b.tbc", 10, lambda k: None)
    v = abi.Video(prim)
    assert L.chd_video_add_extra_source_composite(v._h, a.encode(), None) == 0
    assert L.chd_video_add_extra_source_composite(v._h, b.encode(), None) == 0
    o = C.c_int32()

    def fr(rev, s, f):
        assert L.chdg_video_source_frame(v._h, rev, s, f, C.byref(o)) == 0
        return o.value

    # 0-based here: the reference's sequential frame 6 is frame 5
    assert fr(0, 1, 5) == 0          # disc 105 is extra A's first frame
    assert fr(0, 1, 0) == -1         # disc 100 precedes extra A
    assert fr(0, 0, 5) == 5          # the primary maps to itself
    assert fr(0, 2, 5) == 5          # no VBI: positional
    assert fr(0, 1, 9) == 4
    # reversed pairing: sequential frame 1 is fields (3, 2), disc 101
    assert fr(1, 1, 5) == 0          # disc 106: the reversed primary's frame 6, extra A's frame 1
    assert fr(1, 1, 4) == -1


def test_multi_source_alignment_matches_oracle(tmp_path):
    """CAV and CLV codes, invalid BCD digits, codes on only one field, a
    CLV picture number on line 16 cancelling a CAV one, sources with no
    codes, and both pairings: the library's alignment against the oracle's
    restatement of VbiDecoder / MultiSourceAlignment."""
    L = abi.lib()
    rng = np.random.default_rng(17)

    def clv(fn):
        s_, p_ = divmod(fn, 25)
        m_, s_ = divmod(s_, 60)
        h_, m_ = divmod(m_, 60)
        return synth.clv_vbi(h_, m_, s_, p_)

    layouts = {
        "cav": lambda base: (lambda k: _cav(base + k)),
        "clv": lambda base: (lambda k: clv(base + k)),
        "noisy": lambda base: (lambda k: [int(rng.integers(0, 1 << 24)) for _ in range(3)] if k % 3 == 0
                               else _cav(base + k)),
        "none": lambda base: (lambda k: None),
        "cav_then_clv16": lambda base: (lambda k: [clv(base + k)[0], 0xF00000 | int(str(base + k), 16), 0]),
    }
    names = list(layouts)
    for trial in range(6):
        srcs = []
        paths = []
        for s in range(3):
            kind = names[int(rng.integers(0, len(names)))] if s or trial % 2 else "cav"
            base = int(rng.integers(1, 200))
            nfr = int(rng.integers(4, 9))
            fn = layouts[kind](base)
            p = _write_vbi_capture(tmp_path, f"t{trial}_{s}.tbc", nfr, fn)
            meta = json.load(open(p + ".json"))
            srcs.append(([f["isFirstField"] for f in meta["fields"]],
                         [tuple(f.get("vbi", {}).get("vbiData", [0, 0, 0])) for f in meta["fields"]], nfr))
            paths.append(p)
        v = abi.Video(paths[0])
        for p in paths[1:]:
            assert L.chd_video_add_extra_source_composite(v._h, p.encode(), None) == 0
        for rev in (0, 1):
            frame_for = oracle.align_sources([(f, vb, not rev, True) for f, vb, _ in srcs])
            for s in range(3):
                nfr_s = oracle.num_frames(srcs[s][0], not rev)
                for f in range(oracle.num_frames(srcs[0][0], not rev)):
                    want = frame_for(f + 1, s)
                    want = want - 1 if 1 <= want <= nfr_s else -1
                    o = C.c_int32()
                    assert L.chdg_video_source_frame(v._h, rev, s, f, C.byref(o)) == 0
                    assert o.value == want, (trial, rev, s, f)


def test_dropout_spans_known_answers(tmp_path):
    """The reference's testDropoutSpansAndMask span checks
    (tests/unit/test_dropout_spans_abi.cpp:204-339) on the same geometry and
    dropouts: A = field 0 line 100 [300, 400), B = field 1 line 50 [147, 200)."""
    path = _write_ntsc_capture(tmp_path, [(0, 300, 400, 100), (1, 147, 200, 50)])
    v = abi.Video(path)
    vi = v.info()
    avs, first = vi.first_active_sample, vi.first_active_frame_line
    d = abi.Decoder(v, abi.DEC_NONE)
    d.set("padding_multiple", 1)
    assert abi.lib().chd_decoder_set_option_f64(d._h, b"chroma_nr_level", 0.0) == abi.E_INVALID_ARG
    d.commit()
    oi = d.output_info()
    assert (oi.format, oi.num_planes, oi.num_frames) == (abi.PIXEL_YUV444P16, 3, 2)
    assert (oi.width, oi.height) == (vi.last_active_sample + 1 - avs, vi.last_active_frame_line - first + 1)
    # a NONE decoder never decodes, and the async callback never fires
    f = C.c_void_p()
    assert abi.lib().chd_decode_frame(d._h, 0, C.byref(f)) == abi.E_DECODER_INCOMPATIBLE and not f.value
    hits = []
    cb = abi.FRAME_DONE_CB(lambda u, s, i, fr: hits.append(i))
    idx = (C.c_int64 * 1)(0)
    assert abi.lib().chd_decode_frames_async(d._h, idx, 1, cb, None, None) == abi.E_DECODER_INCOMPATIBLE
    assert hits == []
    yA = 2 * 99 + 0 - first
    yB = 2 * 49 + 1 - first
    assert d.dropout_spans(0) == [(yB, 0, 200 - avs, 0), (yA, 300 - avs, 400 - avs, 0)]
    assert d.dropout_spans(0, abi.DROPOUT_OVERCORRECT) == [(yB, 0, 224 - avs, 0), (yA, 276 - avs, 424 - avs, 0)]
    assert d.dropout_spans(1) == []
    L = abi.lib()
    arr = C.POINTER(abi.DropoutSpan)()
    n = C.c_size_t()
    assert L.chd_decoder_get_dropout_spans(d._h, 99, 0, C.byref(arr), C.byref(n)) == abi.E_OUT_OF_RANGE
    assert L.chd_decoder_get_dropout_spans(d._h, 0, 99, C.byref(arr), C.byref(n)) == abi.E_INVALID_ARG
    assert not arr


@pytest.mark.parametrize("padding", [1, 16])
@pytest.mark.parametrize("mode", [0, 1])
def test_dropout_spans_match_oracle(pal_tbc, padding, mode):
    path, cap = pal_tbc
    oracle.build()
    v = abi.Video(path)
    d = abi.Decoder(v, abi.DEC_NONE)
    d.set("padding_multiple", padding)
    d.commit()
    p = oracle.params(3, oracle.FMT_P16)
    p.padding_multiple = padding
    w, h, _, _ = oracle.output_geometry(p)
    oi = d.output_info()
    assert (oi.width, oi.height) == (w, h)
    flat = oracle.flatten_dropouts(cap.dropouts)
    assert len(flat) > 0
    total = 0
    for frame in range(oi.num_frames):
        mine = d.dropout_spans(frame, mode)
        ref = oracle.dropout_spans(p, flat, frame, mode)
        assert sorted(mine) == sorted(ref)
        assert [s[:2] for s in mine] == sorted(s[:2] for s in mine)
        total += len(mine)
    assert total > 0
