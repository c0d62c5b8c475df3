"""The C++ drop-in (include/cgsense/Reco.h): a program written against the
reference's Reco interface compiles against it, and on a GPU reproduces the
reference's own outputs (tests/golden)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, golden, rel_l2

SRC = os.path.join(ROOT, "tests", "drivers", "reco_dropin.cpp")


@pytest.fixture(scope="module")
def dropin_exe(cgs, tmp_path_factory):
    if not os.path.exists(cgs.LIB_PATH):
        cgs.build()
    out = str(tmp_path_factory.mktemp("dropin") / "reco_dropin")
    libdir = os.path.dirname(cgs.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", out,
           "-L", libdir, "-l:libcgsense.so", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True)
    return out


def test_dropin_compiles_and_links(dropin_exe):
    assert os.path.exists(dropin_exe)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ref_ops_24x20x16.npz", "ref_ops_32x24x16_mask.npz",
                                  "ref_ops_40x20x16_stop.npz"])
def test_dropin_matches_reference(gpu_lib, dropin_exe, name):
    z = golden(name)
    grid = [int(v) for v in z["grid"]]
    nch = int(z["nch"])
    ns = z["k"].shape[0]
    d = tempfile.mkdtemp(prefix="dropin_")
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("%d %d %d %d %d %r\n" % (grid[0], grid[1], grid[2], ns, nch, float(z["cg_threshold"])))
    z["k"].astype(np.float64).tofile(os.path.join(d, "traj.bin"))
    z["data"].astype(np.complex64).tofile(os.path.join(d, "data.bin"))
    z["dcf"].astype(np.float32).tofile(os.path.join(d, "dcf.bin"))
    z["smaps"].astype(np.complex64).tofile(os.path.join(d, "smaps.bin"))
    subprocess.run([dropin_exe, d], check=True, stdout=subprocess.DEVNULL)
    x = np.fromfile(os.path.join(d, "x_out.bin"), np.complex64)
    res = np.fromfile(os.path.join(d, "residuals_out.bin"), np.float64)
    it = int(np.fromfile(os.path.join(d, "iters_out.bin"), np.int32)[0])
    kft = np.fromfile(os.path.join(d, "kernelft_out.bin"), np.complex64)
    assert it == int(z["cg_iters"][0])
    assert np.allclose(res, z["cg_residuals"], rtol=2e-4, atol=0)
    assert rel_l2(x, z["cg_x"]) < 2e-4
    assert rel_l2(kft, z["kernelft"]) < 1e-5


def test_dropin_data_input_paths(cgs, tmp_path):
    """Reco::setDataInputPaths (Reco.cpp:63-71): one state file per batch
    entry, root + file name + index + ".bin" (root and file name are empty
    in the reference, which has no setters for them).  Host only."""
    if not os.path.exists(cgs.LIB_PATH):
        cgs.build()
    src = tmp_path / "paths.cpp"
    src.write_text('#include "cgsense/Reco.h"\n#include <cstdio>\n'
                   'int main() { Reco r; r.setBatch(3); r.setDataInputPaths();\n'
                   '  for (const auto& f : r.getBatchFiles()) std::printf("%s\\n", f.c_str());\n'
                   '  return r.getBatchSize() == 3 ? 0 : 1; }\n')
    exe = str(tmp_path / "paths")
    libdir = os.path.dirname(cgs.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe,
                    "-L", libdir, "-l:libcgsense.so", "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["0.bin", "1.bin", "2.bin"]
