"""Builds libchromadec_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ (CUDA kernels, the host engine and the
chd_* ABI) is compiled in parallel with one -gencode (compute_103a ->
sm_103a) and linked into one shared library that exports only chd_* and
chdg_* symbols (the reference's export map, meson/chromadec.map.in, keeps
chd_* global and everything else local).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libchromadec_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The reference's SONAME and symbol version node for release 0.2.x
# (src/meson.build:238-240, meson.build:53-60: pre-1.0 they track the minor).
SONAME = "libchromadec.so.0.2"
VERSION_NODE = "CHROMADEC_0.2"
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    out = []
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, name))
    return out


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, "chromadec_gb300.h")]
    chd = os.path.join(INCLUDE, "chromadec")
    if os.path.isdir(chd):
        files += [os.path.join(chd, f) for f in os.listdir(chd)]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc] + NVCC_FLAGS + ["-x", "c++", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    vscript = os.path.join(BUILD, "exports.map")
    with open(vscript, "w") as fp:
        # chd_* under the reference's version node (meson/chromadec.map.in,
        # CHROMADEC_<major>.<minor> before 1.0), so binaries linked against
        # the reference bind to these symbols unchanged; chdg_* under our own.
        fp.write(f"{VERSION_NODE} {{ global: chd_*; }};\n"
                 "CHROMADEC_GB300 { global: chdg_*; local: *; };\n")
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + \
          ["-Xlinker", "--version-script=" + vscript, "-Xlinker", "-soname=" + SONAME, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the reference's file names, for consumers that load libchromadec by name
    for alias in (SONAME, "libchromadec.so"):
        ap = os.path.join(HERE, alias)
        if os.path.lexists(ap):
            os.remove(ap)
        os.symlink(os.path.basename(LIB), ap)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
