"""The C++ drop-in shim (include/nsg.hpp): a C++ program written against
nscale's own names (tests/cpp/shim_segment.cpp) is compiled and linked
against libnsg.so here (no GPU needed), and on a GPU it segments a tile whose
labels, boxes, mask and RBC mask must equal the oracle's."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_shim(nsg, outdir):
    """g++ on the test program: include/, the CUDA runtime, libnsg.so."""
    from nscale_gb300 import _lib
    exe = os.path.join(outdir, "shim_segment")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "shim_segment.cpp"),
           "-o", exe, "-L", libdir, "-lnsg", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_shim_compiles_and_links(nsg, tmp_path):
    exe = build_shim(nsg, str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_shim_segments_like_the_oracle(cuda, orc, tmp_path):
    from nscale_gb300 import _lib, synth
    exe = build_shim(_lib.load(), str(tmp_path))
    img = np.ascontiguousarray(synth.he_tile(257, 203, seed=0x5EED1001))
    rows, cols = img.shape[:2]
    src = tmp_path / "tile.bgr"
    img.tofile(src)
    out = str(tmp_path / "o")
    r = subprocess.run([exe, str(src), str(rows), str(cols), out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    status, count, mstatus, dstatus, dcount = map(int, open(out + ".txt").read().split())
    ost, olab, omask, obox, _ = orc.segment_nuclei(img)
    assert status == mstatus == dstatus == ost == 0
    assert count == dcount == obox.shape[1]
    np.testing.assert_array_equal(np.fromfile(out + ".labels.i32", np.int32).reshape(rows, cols), olab)
    np.testing.assert_array_equal(np.fromfile(out + ".dlabels.i32", np.int32).reshape(rows, cols), olab)
    np.testing.assert_array_equal(np.fromfile(out + ".bbox.i32", np.int32).reshape(5, count), obox)
    np.testing.assert_array_equal(np.fromfile(out + ".mask.u8", np.uint8).reshape(rows, cols), omask)
    np.testing.assert_array_equal(np.fromfile(out + ".rbc.u8", np.uint8).reshape(rows, cols), orc.get_rbc(img))
