"""The drop-in C++ header (include/RCBForceTree_gb300.h) used from C++ the way
Particles::map2 uses the reference tree: it compiles against the reference's
call shape, links to libhacc_sr.so, reports the missing device on a CPU-only
machine and matches the golden fixtures on a GPU."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import hsr
import oracle
import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors, golden_names, load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp")


@pytest.fixture(scope="module")
def shim_exe(hsr_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    libdir = os.path.dirname(hsr.LIB_PATH)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.dirname(SRC), SRC, "-o", exe,
                    "-L", libdir, "-lhacc_sr", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a CUDA device is present")
def test_shim_reports_missing_device(shim_exe, tmp_path):
    p, kp, _ = load_golden(golden_names()[0])
    cin, cout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    oracle.write_case(cin, p, kp)
    r = subprocess.run([shim_exe, cin, cout], capture_output=True, text=True)
    assert r.returncode == 3 and "hsr_create" in r.stderr


@pytest.mark.parametrize("tree,law", [(0, "fit"), (0, "rsm"), (0, "newton"), (1, "fit"),
                                      (1, "newton")])
def test_shim_refuses_other_force_laws(shim_exe, tmp_path, law, tree):
    """HACC without -P passes ForceLawSR over FGridEvalFit (Particles.cxx:
    173-183): the drop-in trees throw before any device work instead of
    running the polynomial law in its place; so does a Newtonian law, and
    RCBForceTree given a polynomial law at another softening than its `r`.
    (RCOForceTree has no softening argument: it takes the law's own.)"""
    p, kp, _ = load_golden(golden_names()[0])
    kp.tree = tree
    cin, cout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    oracle.write_case(cin, p, kp)
    r = subprocess.run([shim_exe, cin, cout, law], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert ("not the polynomial short-range law" in r.stderr
            or "no finite softening" in r.stderr), r.stderr
    assert not os.path.exists(cout)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_shim_matches_golden(shim_exe, name, tmp_path):
    p, kp, out = load_golden(name)
    v_in = p.copy()
    hsr.HostLists(v_in, kp)
    cin, cout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    oracle.write_case(cin, p, kp)
    r = subprocess.run([shim_exe, cin, cout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = oracle.read_case_arrays(cout)
    for k in ("x", "y", "z", "mass", "phi", "id", "mask"):
        assert np.array_equal(got[k].view(np.uint8), out[k].view(np.uint8)), k
    vin = np.stack([v_in.vx, v_in.vy, v_in.vz], 1).astype(np.float64)
    dv = np.stack([got["vx"], got["vy"], got["vz"]], 1) - vin
    dv_ref = np.stack([out["vx"], out["vy"], out["vz"]], 1) - vin
    rms, mx = force_errors(dv, dv_ref)
    slack = 0.0 if not np.abs(vin).max(initial=0) else \
        64 * 2.0 ** -24 * np.abs(vin).max() / np.sqrt((dv_ref ** 2).sum(1).mean())
    assert rms <= RMS_TOL + slack and mx <= MAX_TOL + slack
