"""Cases of the golden vectors (tests/golden/golden.json).

Each case names the reference code path (decode / chroma-only / dropout
concealment), the Transform-PAL kind (2 or 3), the output format, the frames
decoded and the options. Inputs are seeded synthetic PAL captures from
libchromadec_gb300.synth; frames at both ends of a capture exercise the black
padding of the 3D field window.
"""
from __future__ import annotations

import functools

import numpy as np

from libchromadec_gb300 import synth

CASES = {
    "t2d_p16": dict(mode="decode", kind=2, fmt="p16", nfields=8, seed=31, first=0, count=4),
    "t2d_ps": dict(mode="decode", kind=2, fmt="ps", nfields=8, seed=31, first=0, count=4),
    "t2d_thr": dict(mode="decode", kind=2, fmt="p16", nfields=8, seed=31, first=1, count=2, thr_seed=5),
    "t2d_opts_ps": dict(mode="decode", kind=2, fmt="ps", nfields=8, seed=31, first=2, count=2, threshold=0.55,
                        chroma_gain=0.8, chroma_phase_deg=-12.0, clamp_mode=1),
    "t3d_p16": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=0, count=6),
    "t3d_ps": dict(mode="decode", kind=3, fmt="ps", nfields=12, seed=32, first=0, count=6),
    "t3d_thr": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=2, count=2, thr_seed=6),
    "t3d_opts": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=0, count=3, chroma_gain=1.25,
                     chroma_phase_deg=7.5, clamp_mode=3, padding_multiple=32, active_start=185, active_end=1101,
                     first_active_frame_line=50, last_active_frame_line=601),
    "t3d_drop": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02),
    "t3d_drop_oc": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02,
                        overcorrect=1),
    "t3d_drop_intra": dict(mode="decode", kind=3, fmt="ps", nfields=12, seed=33, first=1, count=4, dropouts=0.02,
                           intra=1),
    "conceal": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02),
    "conceal_oc": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02,
                       overcorrect=1),
    "chroma2d": dict(mode="chroma", kind=2, nfields=8, seed=31, first=0, count=4),
    "chroma3d": dict(mode="chroma", kind=3, nfields=12, seed=32, first=0, count=6),
    # PALcolour 2D filter alone (CHD_DEC_PAL_2D)
    "pal2d_p16": dict(mode="decode", kind=1, fmt="p16", nfields=8, seed=34, first=0, count=4),
    "pal2d_ps_ynr": dict(mode="decode", kind=1, fmt="ps", nfields=8, seed=34, first=1, count=2, y_nr_level=2.5),
    # luma noise coring on the Transform paths
    "t3d_ynr": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=1, count=3, y_nr_level=1.5),
    "t2d_ynr_ps": dict(mode="decode", kind=2, fmt="ps", nfields=8, seed=31, first=0, count=2, y_nr_level=4.0),
    # output formats and colour-conversion precisions
    "t3d_rgb48": dict(mode="decode", kind=3, fmt="rgb48", nfields=12, seed=32, first=2, count=2),
    "t3d_rgbs_bt601": dict(mode="decode", kind=3, fmt="rgbs", nfields=12, seed=32, first=2, count=2, clamp_mode=3,
                           cdp="classic", bsp="modern"),
    "t3d_rgbs_hdr": dict(mode="decode", kind=3, fmt="rgbs", nfields=12, seed=32, first=3, count=1, clamp_mode=2),
    "t2d_gray16_pad": dict(mode="decode", kind=2, fmt="gray16", nfields=8, seed=31, first=0, count=2,
                           padding_multiple=16, clamp_mode=1),
    "t2d_grays": dict(mode="decode", kind=2, fmt="grays", nfields=8, seed=31, first=1, count=2, clamp_mode=3),
    "t3d_p16_classic": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=2, count=1,
                            cdp="classic", bsp="classic"),
    # reversed field pairing (reverse_field_order): slot 0 holds second fields
    "t3d_rev": dict(mode="decode", kind=3, fmt="p16", nfields=13, seed=35, first=0, count=6, sff=1,
                    dropouts=0.02),
    "t2d_rev_ps": dict(mode="decode", kind=2, fmt="ps", nfields=9, seed=35, first=0, count=4, sff=1),
    "conceal_rev": dict(mode="dropout", kind=3, fmt="p16", nfields=13, seed=35, first=0, count=6, sff=1,
                        dropouts=0.02),
    # subcarrier-locked PAL: second fields shifted by 2 samples
    "t3d_sclocked": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, sc_locked=1,
                         dropouts=0.02),
    "conceal_sclocked": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6,
                             sc_locked=1, dropouts=0.02, overcorrect=1),
    # multi-source concealment: extra captures of the same pictures with their
    # own noise and dropouts; `offset` frames of other content lead an extra
    # (window frame f is its frame f + offset), `trim` frames are cut off its
    # end; bpsnr is each source's VITS bPSNR (one value per source, or a
    # per-field list)
    "conceal_multi": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.03,
                          bpsnr=40.5, extras=[dict(noise_seed=61, dropout_seed=71, dropouts=0.03, bpsnr=38.0),
                                              dict(noise_seed=62, dropout_seed=72, dropouts=0.02, offset=1,
                                                   bpsnr=42.25)]),
    "conceal_multi_tie": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=36, first=0, count=6,
                              dropouts=0.04, overcorrect=1,
                              extras=[dict(noise_seed=63, dropout_seed=73, dropouts=0.05, trim=2),
                                      dict(noise_seed=64, dropout_seed=74, dropouts=0.05, offset=2)]),
    "conceal_multi_intra_sclocked": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6,
                                         dropouts=0.03, intra=1, sc_locked=1, bpsnr=[30.0 + 0.5 * i for i in range(12)],
                                         extras=[dict(noise_seed=65, dropout_seed=75, dropouts=0.04, bpsnr=33.0)]),
    "t3d_drop_multi": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.03,
                           bpsnr=39.0, extras=[dict(noise_seed=61, dropout_seed=71, dropouts=0.03, bpsnr=41.0),
                                               dict(noise_seed=66, dropout_seed=76, dropouts=0.02, offset=1, trim=1)]),
    "t2d_drop_multi_rev_ps": dict(mode="decode", kind=2, fmt="ps", nfields=9, seed=35, first=0, count=4, sff=1,
                                  dropouts=0.03, extras=[dict(noise_seed=67, dropout_seed=77, dropouts=0.03)]),
    # PAL-M (525 lines, 909 samples, ST 244 levels): the same decoders on the other raster
    "palm_t3d_p16": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=37, first=0, count=6, std="palm"),
    "palm_t3d_ps": dict(mode="decode", kind=3, fmt="ps", nfields=12, seed=37, first=1, count=3, std="palm"),
    "palm_t2d_p16": dict(mode="decode", kind=2, fmt="p16", nfields=8, seed=38, first=0, count=4, std="palm"),
    "palm_pal2d_ps": dict(mode="decode", kind=1, fmt="ps", nfields=8, seed=38, first=0, count=4, std="palm"),
    "palm_chroma3d": dict(mode="chroma", kind=3, nfields=12, seed=37, first=0, count=4, std="palm"),
    "palm_t3d_drop": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=39, first=0, count=6, dropouts=0.02,
                          std="palm"),
    "palm_conceal": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=39, first=0, count=6, dropouts=0.02,
                         overcorrect=1, std="palm"),
}

# harness argument of each optional case key
HARNESS_ARGS = {"chroma_gain": "gain", "chroma_phase_deg": "phase", "clamp_mode": "clamp",
                "padding_multiple": "padding", "active_start": "avs", "active_end": "ave",
                "first_active_frame_line": "fafl", "last_active_frame_line": "lafl", "y_nr_level": "ynr",
                "sff": "sff", "sc_locked": "sclocked", "cdp": "cdp", "bsp": "bsp", "std": "std"}

SYNTH_STANDARD = {"pal": "PAL", "palm": "PAL_M"}


@functools.lru_cache(maxsize=8)
def _capture(nfields: int, seed: int, dropouts: float, standard: str = "PAL"):
    cfg = synth.SynthConfig(seed=seed, pan_x=1.5, pan_y=0.5, dropout_line_fraction=dropouts, standard=standard)
    return synth.make_capture(nfields, cfg)


def case_inputs(case: dict):
    """(fields uint16 (n, field_height, field_width), flat dropouts [(field, startx, endx, fieldLine)] or None).

    For the reversed pairing (sff) the capture's first field is dropped, so
    the array starts with a second field and frame k is fields 2k, 2k+1 of
    the array, slot 0 being a second field."""
    cap = _capture(case["nfields"], case["seed"], case.get("dropouts", 0.0), SYNTH_STANDARD[case.get("std", "pal")])
    skip = 1 if case.get("sff") else 0
    flat = None
    if case.get("dropouts", 0.0) > 0:
        flat = [(f - skip, s[0], s[1], s[2]) for f, spans in enumerate(cap.dropouts) for s in spans if f >= skip]
    return np.ascontiguousarray(cap.fields[skip:]), flat


def _per_field(v, n):
    if v is None:
        return None
    if isinstance(v, (list, tuple)):
        return np.asarray(v[:n], dtype=np.float64)
    return np.full(n, float(v))


def case_sources(case: dict):
    """Multi-source inputs of a case: (primary per-field bPSNR or None,
    [dict(fields, dropouts, bpsnr, offset)] extras) laid out like the
    primary from case_inputs (reversed pairing drops the same first field)."""
    if "extras" not in case:
        return None, []
    skip = 1 if case.get("sff") else 0
    n = case["nfields"] - skip
    extras = []
    for e in case["extras"]:
        off, trim = e.get("offset", 0), e.get("trim", 0)
        cfg = synth.SynthConfig(seed=case["seed"], pan_x=1.5, pan_y=0.5, dropout_line_fraction=e["dropouts"],
                                noise_seed=e["noise_seed"], dropout_seed=e["dropout_seed"])
        rc = synth.make_capture(case["nfields"], cfg)
        fields = np.ascontiguousarray(rc.fields[skip:])
        drops = [(f - skip, s[0], s[1], s[2]) for f, spans in enumerate(rc.dropouts) for s in spans if f >= skip]
        if off > 0:   # leading frames of other content
            lead = synth.make_capture(2 * off, synth.SynthConfig(seed=case["seed"] + 1000, noise_seed=e["noise_seed"]))
            fields = np.concatenate([lead.fields, fields])
            drops = [(f + 2 * off, a, b, c) for f, a, b, c in drops]
        if trim > 0:
            keep = fields.shape[0] - 2 * trim
            fields = np.ascontiguousarray(fields[:keep])
            drops = [d for d in drops if d[0] < keep]
        extras.append(dict(fields=fields, dropouts=drops, bpsnr=_per_field(e.get("bpsnr"), fields.shape[0]),
                           offset=off))
    return _per_field(case.get("bpsnr"), n), extras


def thresholds_for(case: dict):
    if "thr_seed" not in case:
        return None
    n = 80 if case["kind"] == 2 else 768
    return np.random.default_rng(case["thr_seed"]).uniform(0.25, 0.65, n)
