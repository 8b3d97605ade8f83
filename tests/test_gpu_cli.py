"""The offline evaluator (pd-flow_gb300/examples/pd_flow_pair.cpp): the
reference CLI's flags, PGM frames in, `<root>_resultsNN.txt` and the PPM
representation out; its flow equals the library's."""
import os
import subprocess

import numpy as np
import pytest

from pdflow import Solver, scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_pgm(path, a):
    a = np.ascontiguousarray(a)
    h, w = a.shape
    with open(path, "wb") as f:
        if a.dtype == np.uint8:
            f.write(b"P5\n%d %d\n255\n" % (w, h))
            f.write(a.tobytes())
        else:
            f.write(b"P5\n%d %d\n65535\n" % (w, h))
            f.write(a.astype(">u2").tobytes())


def test_cli_writes_the_reference_results_format(built_lib, tmp_path):
    exe = str(tmp_path / "pd_flow_pair")
    lib = os.path.join(ROOT, "pd-flow_gb300", "lib")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "pd-flow_gb300", "csrc"),
                        os.path.join(ROOT, "pd-flow_gb300", "examples", "pd_flow_pair.cpp"), "-L", lib,
                        "-lpdflow_gb300", f"-Wl,-rpath,{lib}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    i1, z1, i2, z2 = scenes.make_pair(17, n_objects=3)
    for name, a in (("i1", i1), ("z1", z1), ("i2", i2), ("z2", z2)):
        write_pgm(str(tmp_path / f"{name}.pgm"), a)
    out = str(tmp_path / "run")
    r = subprocess.run([exe, "--rows", "120", "--i1", str(tmp_path / "i1.pgm"), "--i2", str(tmp_path / "i2.pgm"),
                        "--z1", str(tmp_path / "z1.pgm"), "--z2", str(tmp_path / "z2.pgm"), "--out", out,
                        "--no-show"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    res = np.loadtxt(out + "_results01.txt")
    assert res.shape == (120 * 160, 5)
    s = Solver(120, 320, 240).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    v, u = res[:, 0].astype(int), res[:, 1].astype(int)
    idx = v + u * 120
    for c, ref in zip((2, 3, 4), (s.dxp, s.dyp, s.dzp)):
        assert np.allclose(res[:, c], ref[idx], rtol=1e-5, atol=1e-7)
    s.freeGPUMemory()
    with open(out + "_representation01.ppm", "rb") as f:
        assert f.read(15) == b"P6\n160 120\n255\n"
    # a second run does not overwrite the first
    r = subprocess.run([exe, "--rows", "120", "--i1", str(tmp_path / "i1.pgm"), "--i2", str(tmp_path / "i2.pgm"),
                        "--z1", str(tmp_path / "z1.pgm"), "--z2", str(tmp_path / "z2.pgm"), "--out", out],
                       capture_output=True, text=True)
    assert r.returncode == 0 and os.path.exists(out + "_results02.txt")
