"""A C11 program written against include/chromadec/*.h, linked by the
reference's library name (-lchromadec) and run: the headers compile as C, the
symbols resolve under the reference's version node, and the answers match the
Python binding's."""
import json
import os
import shutil
import subprocess

import pytest

from libchromadec_gb300 import _build, abi, synth
from tests._capture import capture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "libchromadec_gb300")


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    _build.build()
    exe = str(tmp_path_factory.mktemp("c") / "consumer")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_consumer", "consumer.c"), "-L", PKG, "-lchromadec",
                    "-Wl,-rpath," + PKG, "-o", exe], check=True)
    return exe


@pytest.fixture(scope="module")
def tbc(tmp_path_factory):
    cap = capture(8, 7, dropouts=0.02)
    path = str(tmp_path_factory.mktemp("cc") / "cap.tbc")
    synth.write_tbc(path, cap)
    return path


def test_symbols_carry_the_reference_version_node():
    out = subprocess.run(["readelf", "--dyn-syms", "-W", _build.LIB], capture_output=True, text=True).stdout
    assert "chd_decode_frame@@CHROMADEC_0.2" in out
    assert "chdg_decode_device@@CHROMADEC_GB300" in out
    dyn = subprocess.run(["readelf", "-d", _build.LIB], capture_output=True, text=True).stdout
    assert "libchromadec.so.0.2" in dyn


def test_c_consumer_matches_python_binding(consumer, tbc):
    r = subprocess.run([consumer, tbc], capture_output=True, text=True, check=True)
    got = json.loads(r.stdout)
    v = abi.Video(tbc)
    d = abi.Decoder(v, abi.DEC_NONE)
    d.commit()
    assert got["version"] == "0.2.1" and got["field_width"] == 1135 and got["num_frames"] == 4
    assert got["out"] == [948, 576, 3]
    assert [tuple(s) for s in got["spans"]] == d.dropout_spans(0)


@pytest.mark.gpu
def test_c_consumer_decodes(cuda, consumer, tbc):
    r = subprocess.run([consumer, tbc, "decode"], capture_output=True, text=True, check=True)
    got = json.loads(r.stdout)
    assert got["frame"] == [948, 576, 3]
    v = abi.Video(tbc)
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    d.commit()
    planes = d.decode(0).planes()
    assert got["samples"] == [int(planes[p][300, 474]) for p in range(3)]
