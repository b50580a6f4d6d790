"""Evaluation of the learned form against the plain threshold on held-out
fields (measurement code for the tests and the benchmark).

For a seeded capture with ground truth (synth.py), frames are decoded in
chunks: the feature pass gives every Z tile's features and the FP32
threshold decisions; the network gives its fractions and fallback flags.
Then, for both forms, against the encoder's true chroma over the active
area (field lines 22..309, samples 177..1124, peak = white - black):

  * chroma PSNR of the separated chroma (the plain form as the decoder runs
    it, with every threshold decision exact; the learned form as its engine
    decodes);
  * cross-colour: the chroma the form's masks pass from the luma-only signal
    (the same masks applied to the encoder's luma alone), as energy relative
    to the true chroma's, and as dB below the peak;
  * cross-luma: the true chroma the masks reject (the masks applied to the
    chroma-only signal, minus the true chroma), likewise.

The masks of a tile are taken from the composite and applied unchanged to
the luma-only and chroma-only signals, so the two leaks add up to the form's
chroma error.
"""
from __future__ import annotations

import numpy as np

from libchromadec_gb300 import device as D, masknet_train as MT, synth

ROWS = slice(22, 310)
COLS = slice(synth.ACTIVE_START, synth.ACTIVE_END)


def _db(peak2, e):
    return float(10.0 * np.log10(peak2 / e)) if e > 0 else float("inf")


def evaluate(weights, nfields: int = 500, seed: int = 1, pan_x: float = 1.5, pan_y: float = 0.5,
             chunk_frames: int = 50, threshold: float = 0.4, stream=None):
    import torch
    cfg = synth.SynthConfig(seed=seed, pan_x=pan_x, pan_y=pan_y)
    cap = synth.make_capture(nfields, cfg, truth=True)
    n = nfields
    nfr = n // 2
    g = D.default_geometry()
    gc = D.default_geometry()
    gc.black = MT.CHROMA_OFFSET
    cfgd = D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS, threshold=threshold)
    plain = D.Engine(g, cfgd)
    learned = D.Engine(g, cfgd)
    net = D.MaskNet(weights)
    learned.set_masknet(net)
    engc = D.Engine(gc, cfgd)
    comp = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    luma = torch.from_numpy(MT.luma_only_fields(cap).reshape(n, -1).view(np.int16)).cuda()
    chro = torch.from_numpy(MT.chroma_only_fields(cap).reshape(n, -1).view(np.int16)).cuda()
    truth_all = torch.from_numpy(np.ascontiguousarray(cap.chroma[:, ROWS, COLS])).cuda().double()
    nt = plain.ntiles()
    acc = {k: 0.0 for k in ("err_plain", "err_learned", "cc_plain", "cc_learned", "cl_plain", "cl_learned",
                            "truth")}
    fallback_tiles = 0
    tiles = 0
    for fb in range(0, nfr, chunk_frames):
        fe = min(nfr, fb + chunk_frames)
        nz = fe - fb + 2
        feat = torch.empty((nz, nt, D.MASKNET_BINS), dtype=torch.int16, device="cuda")
        thr = torch.empty((nz, nt, D.MASKNET_BINS), dtype=torch.float32, device="cuda")
        plain.learned_features(comp, fb, fe, feat, None, thr, stream)
        p = torch.empty((nz * nt, D.MASKNET_BINS), dtype=torch.float32, device="cuda")
        fbk = torch.empty((nz * nt,), dtype=torch.uint8, device="cuda")
        net.forward(feat, nz * nt, p, fbk, stream)
        zero = torch.zeros_like(fbk)
        shape = (2 * (fe - fb), 288, 948)
        out = {k: torch.empty(shape, dtype=torch.float32, device="cuda") for k in
               ("plain", "learned", "cc_p", "cc_l", "cl_p", "cl_l")}
        plain.chroma(comp, fb, fe, out["plain"], stream)
        learned.chroma(comp, fb, fe, out["learned"], stream)
        plain.learned_chroma(luma, fb, fe, thr, zero, out["cc_p"], stream)
        plain.learned_chroma(luma, fb, fe, p, fbk, out["cc_l"], stream)
        engc.learned_chroma(chro, fb, fe, thr, zero, out["cl_p"], stream)
        engc.learned_chroma(chro, fb, fe, p, fbk, out["cl_l"], stream)
        torch.cuda.synchronize()
        truth = truth_all[2 * fb:2 * fe]
        acc["truth"] += float((truth ** 2).sum())
        acc["err_plain"] += float(((out["plain"].double() - truth) ** 2).sum())
        acc["err_learned"] += float(((out["learned"].double() - truth) ** 2).sum())
        acc["cc_plain"] += float((out["cc_p"].double() ** 2).sum())
        acc["cc_learned"] += float((out["cc_l"].double() ** 2).sum())
        acc["cl_plain"] += float(((out["cl_p"].double() - truth) ** 2).sum())
        acc["cl_learned"] += float(((out["cl_l"].double() - truth) ** 2).sum())
        fallback_tiles += int(fbk.sum())
        tiles += int(fbk.numel())
        del feat, thr, p, fbk, out
    npx = nfields * 288 * 948
    peak2 = float(g.white - g.black) ** 2
    res = {}
    for form in ("plain", "learned"):
        res[form] = {
            "chroma_psnr_db": _db(peak2, acc[f"err_{form}"] / npx),
            "cross_colour_rel_energy": acc[f"cc_{form}"] / acc["truth"],
            "cross_colour_db": _db(peak2, acc[f"cc_{form}"] / npx),
            "cross_luma_rel_energy": acc[f"cl_{form}"] / acc["truth"],
            "cross_luma_db": _db(peak2, acc[f"cl_{form}"] / npx),
        }
    res["learned"]["fallback_tiles"] = fallback_tiles
    res["learned"]["tiles"] = tiles
    res["fields"] = nfields
    res["held_out"] = f"seed {seed}, pan {pan_x} px/field + {pan_y} line/field (training uses seeds >= 1001)"
    net.close()
    return res
