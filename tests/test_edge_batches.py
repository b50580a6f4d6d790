"""The batch splitter both host paths use (chdg::edge_batches in
libchromadec_gb300/csrc/engine.h: chd_decode_frames_async's pipeline and
chdg_decode_host), compiled on the host and checked over many run lengths:
the batches tile [a, b) in order, none is empty or longer than the batch
size, a run that fits one batch is one batch, and a longer run starts and
ends with a batch of the edge size (at most half a batch), so the copies no
kernel overlaps stay small."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "libchromadec_gb300", "csrc")

DRIVER = r"""
#include "engine.h"
#include <cstdio>
#include <cstdlib>
int main(int argc, char **argv)
{
    // argv: batch edge, then (a, b) pairs; one line of "first:last ..." per pair
    const long long batch = std::atoll(argv[1]), edge = std::atoll(argv[2]);
    for (int i = 3; i + 1 < argc; i += 2) {
        for (const auto &p : chdg::edge_batches(std::atoll(argv[i]), std::atoll(argv[i + 1]), batch, edge))
            std::printf("%lld:%lld ", (long long)p.first, (long long)p.second);
        std::printf("\n");
    }
    return 0;
}
"""


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def splitter(tmp_path_factory):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("no host C++ compiler or CUDA headers")
    d = tmp_path_factory.mktemp("eb")
    src, exe = d / "eb.cpp", d / "eb"
    src.write_text(DRIVER)
    subprocess.run(["g++", "-std=c++17", "-I", CSRC, "-I", inc, str(src), "-o", str(exe)], check=True)

    def run(batch, edge, ranges):
        args = [str(exe), str(batch), str(edge)] + [str(x) for r in ranges for x in r]
        out = subprocess.run(args, capture_output=True, text=True, check=True).stdout.splitlines()
        return [[tuple(int(v) for v in tok.split(":")) for tok in line.split()] for line in out]

    return run


@pytest.mark.parametrize("batch,edge", [(64, 16), (32, 16), (16, 16), (8, 16), (1, 16)])
def test_batches_tile_the_run(splitter, batch, edge):
    ranges = [(a, a + n) for a in (0, 7) for n in range(0, 301)]
    e = max(1, min(edge, max(1, batch // 2)))
    for (a, b), bl in zip(ranges, splitter(batch, edge, ranges)):
        if b == a:
            assert bl == []
            continue
        assert bl[0][0] == a and bl[-1][1] == b
        assert all(s < t and t - s <= batch for s, t in bl)
        assert all(bl[i][1] == bl[i + 1][0] for i in range(len(bl) - 1))
        if b - a <= batch:
            assert bl == [(a, b)]
        else:
            assert bl[0][1] - bl[0][0] == e and bl[-1][1] - bl[-1][0] == e


def test_the_bench_stream(splitter):
    assert splitter(64, 16, [(0, 250)])[0] == [(0, 16), (16, 80), (80, 144), (144, 208), (208, 234), (234, 250)]
