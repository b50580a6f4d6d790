"""Generate tests/golden/golden.json from the reference's own code.

Runs oracle/_ref/chd_ref_harness -- the reference's Transform-PAL,
PALcolour, OutputWriter and DropoutCorrector sources compiled unmodified
from the reference tree (oracle/Makefile, target ``ref``) -- on seeded
synthetic captures, and records for every case the SHA-256 of the raw output
bytes plus the dropout statistics the reference reports. The input captures
are regenerated from their seeds by the tests, and their own SHA-256 is
recorded too, so a changed generator is told apart from a changed oracle.

Usage (needs the reference checkout, so it runs where that exists):
    python tests/golden/make_golden.py --ref /path/to/reference
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.cases import CASES, HARNESS_ARGS, case_inputs, case_sources, thresholds_for  # noqa: E402
from oracle import oracle  # noqa: E402


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def run_case(harness: str, case: dict, tmp: str) -> dict:
    fields, dropouts = case_inputs(case)
    fin = os.path.join(tmp, "in.u16")
    fields.tofile(fin)
    out = os.path.join(tmp, "out.bin")
    args = [harness, f"mode={case['mode']}", f"kind={case['kind']}", f"fmt={case.get('fmt', 'p16')}",
            f"threshold={case.get('threshold', 0.4)}", f"in={fin}", f"nfields={fields.shape[0]}",
            f"first={case['first']}", f"count={case['count']}", f"out={out}"]
    if dropouts:
        dpath = os.path.join(tmp, "drop.txt")
        with open(dpath, "w") as fp:
            for f, sx, ex, fl in dropouts:
                fp.write(f"{f} {sx} {ex} {fl}\n")
        args += [f"dropouts={dpath}", f"overcorrect={int(case.get('overcorrect', 0))}",
                 f"intra={int(case.get('intra', 0))}"]
    bpsnr, extras = case_sources(case)
    blines = []
    if bpsnr is not None:
        blines += [f"0 {i} {float(v)!r}" for i, v in enumerate(bpsnr)]
    for k, e in enumerate(extras):
        epath = os.path.join(tmp, f"extra{k + 1}.u16")
        e["fields"].tofile(epath)
        edrop = os.path.join(tmp, f"extra{k + 1}_drop.txt")
        with open(edrop, "w") as fp:
            for f, sx, ex, fl in e["dropouts"]:
                fp.write(f"{f} {sx} {ex} {fl}\n")
        args.append(f"extra{k + 1}={epath}:{e['fields'].shape[0]}:{edrop}:{e['offset']}")
        if e["bpsnr"] is not None:
            blines += [f"{k + 1} {i} {float(v)!r}" for i, v in enumerate(e["bpsnr"])]
    if blines:
        bpath = os.path.join(tmp, "bpsnr.txt")
        with open(bpath, "w") as fp:
            fp.write("\n".join(blines) + "\n")
        args.append(f"bpsnr={bpath}")
    thr = thresholds_for(case)
    if thr is not None:
        tpath = os.path.join(tmp, "thr.txt")
        with open(tpath, "w") as fp:
            fp.write("\n".join(repr(float(t)) for t in thr))
        args.append(f"thresholds={tpath}")
    for key, arg in HARNESS_ARGS.items():
        if key in case:
            args.append(f"{arg}={case[key]}")
    r = subprocess.run(args, capture_output=True, text=True, check=True)
    stats = json.loads(r.stdout.strip().splitlines()[-1])
    with open(out, "rb") as fp:
        data = fp.read()
    res = {"input_sha256": sha(fields.tobytes()), "output_sha256": sha(data), "output_bytes": len(data),
           "stats": [stats["corrected"], stats["failed"], stats["total_distance"]]}
    if extras:
        res["extras_sha256"] = [sha(e["fields"].tobytes()) for e in extras]
    return res


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CHROMADEC_REFERENCE"),
                    help="reference checkout (default: $CHROMADEC_REFERENCE)")
    a = ap.parse_args()
    harness = oracle.build_reference(a.ref)
    if harness is None:
        raise SystemExit(f"reference checkout not found at {a.ref!r} (pass --ref or set CHROMADEC_REFERENCE)")
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, case in CASES.items():
            res[name] = run_case(harness, case, tmp)
            print(name, res[name]["output_sha256"][:16], res[name]["stats"], flush=True)
    with open(os.path.join(HERE, "golden.json"), "w") as fp:
        json.dump({"generator": "reference sources via oracle/_ref/chd_ref_harness", "cases": res}, fp, indent=1,
                  sort_keys=True)


if __name__ == "__main__":
    main()
