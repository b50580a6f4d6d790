"""The oracle's C restatement against golden vectors from the reference.

tests/golden/golden.json holds, per case, the SHA-256 of what the
reference's own Transform-PAL / PALcolour / OutputWriter / DropoutCorrector
sources output (compiled unmodified, oracle/_ref; generator
tests/golden/make_golden.py). The restatement must reproduce every byte and
the reference's dropout statistics; the GPU path is then checked against the
restatement.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.cases import CASES, case_inputs, case_sources, thresholds_for

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]


FMTS = {"p16": O.FMT_P16, "ps": O.FMT_PS, "rgb48": O.FMT_RGB48, "rgbs": O.FMT_RGBS, "gray16": O.FMT_GRAY16,
        "grays": O.FMT_GRAYS}


def _params(case):
    p = O.params(case["kind"], FMTS[case.get("fmt", "p16")], threshold=case.get("threshold", 0.4),
                 thresholds=thresholds_for(case))
    if case.get("std") == "palm":
        O.pal_m(p)
    for k in ("chroma_gain", "chroma_phase_deg", "clamp_mode", "padding_multiple", "active_start", "active_end",
              "first_active_frame_line", "last_active_frame_line", "y_nr_level"):
        if k in case:
            setattr(p, k, case[k])
    p.first_field_offset = int(case.get("sff", 0))
    p.sc_locked = int(case.get("sc_locked", 0))
    O.colour_precision(p, case.get("cdp", "modern"), case.get("bsp", "scientific"))
    return p


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_matches_reference_golden(name):
    case, gold = CASES[name], GOLDEN[name]
    fields, drops = case_inputs(case)
    assert hashlib.sha256(fields.tobytes()).hexdigest() == gold["input_sha256"], "synthetic input changed"
    p = _params(case)
    oc, intra = bool(case.get("overcorrect", 0)), bool(case.get("intra", 0))
    bpsnr, extras = case_sources(case)
    if extras:
        assert [hashlib.sha256(e["fields"].tobytes()).hexdigest() for e in extras] == gold["extras_sha256"]
    nframes = fields.shape[0] // 2
    # positional alignment with each extra's leading frames: window frame f is the extra's f + offset
    ex = [dict(fields=e["fields"], dropouts=e["dropouts"], bpsnr=e["bpsnr"],
               frame_map=[f + e["offset"] for f in range(nframes)]) for e in extras]
    if case["mode"] == "decode":
        out, st = O.decode_frames(p, fields, case["first"], case["count"], dropouts=drops, overcorrect=oc,
                                  intra=intra, threads=8, bpsnr=bpsnr, extras=ex)
        data = out.tobytes()
    elif case["mode"] == "chroma":
        data = O.transform_chroma(p, fields, case["first"], case["count"]).tobytes()
        st = (0, 0, 0)
    else:
        parts, tot = [], np.zeros(3, dtype=np.int64)
        for k in range(case["first"], case["first"] + case["count"]):
            f2, s = O.dropout_correct_frame(p, fields, k, drops, oc, intra, bpsnr=bpsnr, extras=ex)
            parts.append(f2.tobytes())
            tot += s
        data, st = b"".join(parts), tuple(int(x) for x in tot)
    assert len(data) == gold["output_bytes"]
    assert hashlib.sha256(data).hexdigest() == gold["output_sha256"]
    assert list(st) == gold["stats"]
