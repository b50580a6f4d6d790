"""PAL-M (525 lines, 909 samples per line, 4 fSC) through the chd_* ABI on
the GPU: the reference's PalDecoder accepts PAL and PAL-M for
CHD_DEC_PAL_2D, CHD_DEC_TRANSFORM_2D and CHD_DEC_TRANSFORM_3D
(src/decoders/palcolour/pal_decoder.cpp:38-51), with the PAL-M preset's
raster and levels (src/format/video_standards.cpp:28-52, 85-100), the
demodulator's PAL-M table exchange (palcolour.cpp:158-173), its filter size
at the PAL-M sample rate, and the PAL-M luma filter of the dropout corrector
(dropout_corrector.cpp:498-506). A seeded PAL-M capture is written as a
.tbc + JSON sidecar (system "PAL_M") and every frame compared with the
oracle, itself pinned to the reference's own code by the PAL-M golden cases.
"""
import numpy as np
import pytest

from libchromadec_gb300 import abi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NF = 16


@pytest.fixture(scope="module")
def palm(tmp_path_factory):
    cfg = synth.SynthConfig(seed=71, pan_x=1.5, pan_y=0.5, dropout_line_fraction=0.015, standard="PAL_M")
    cap = synth.make_capture(NF, cfg)
    path = str(tmp_path_factory.mktemp("palm") / "m.tbc")
    synth.write_tbc(path, cap)
    return path, cap


def _compare(got, ref, fmt):
    if fmt == "yuv444ps":
        err = np.abs(got.astype(np.float64) - ref.astype(np.float64)).max()
        assert err < 1e-4, err
    else:
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1, (d.max(), (d > 0).mean())


@pytest.mark.parametrize("kind,okind", [(abi.DEC_TRANSFORM_3D, 3), (abi.DEC_TRANSFORM_2D, 2), (abi.DEC_PAL_2D, 1)])
@pytest.mark.parametrize("fmt", ["yuv444p16", "yuv444ps"])
def test_palm_decodes_match_oracle(cuda, palm, kind, okind, fmt):
    path, cap = palm
    v = abi.Video(path)
    vi = v.info()
    assert (vi.field_width, vi.field_height) == (909, 263)
    d = abi.Decoder(v, kind)
    d.set("output_format", fmt)
    d.commit()
    oi = d.output_info()
    assert (oi.width, oi.height, oi.num_frames) == (768, 486, NF // 2)
    p = O.pal_m(O.params(okind, O.FMT_PS if fmt == "yuv444ps" else O.FMT_P16))
    ref, _ = O.decode_frames(p, cap.fields, 0, NF // 2, threads=8)
    got = {i: pl for s, i, pl in d.decode_async(list(range(NF // 2)))}
    for k in range(NF // 2):
        _compare(got[k], ref[k], fmt)


def test_palm_concealment_and_decode_with_dropouts(cuda, palm):
    path, cap = palm
    v = abi.Video(path)
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    d.commit()
    p = O.pal_m(O.params(3, O.FMT_P16))
    flat = O.flatten_dropouts(cap.dropouts)
    assert len(flat) > 0
    blended = 0
    for overcorrect, intra in ((False, False), (True, False), (False, True)):
        d.set_dropout(True, overcorrect, intra)
        for k in range(NF // 2):
            got = d.concealed_fields(k)
            ref, st = O.dropout_correct_frame(p, cap.fields, k, flat, overcorrect=overcorrect, intra=intra)
            assert np.array_equal(got, ref), (k, overcorrect, intra)
            # the PAL-M luma filter shows where a replacement line is blended
            blended += int((ref != cap.fields[2 * k:2 * k + 2]).sum())
            dec, st2 = O.decode_frames(p, cap.fields, k, 1, dropouts=flat, overcorrect=overcorrect, intra=intra,
                                       threads=8)
            f = d.decode(k)
            _compare(f.planes(), dec[0], "yuv444p16")
            assert d.last_dropout_stats() == tuple(st2)
            f.close()
    assert blended > 0
