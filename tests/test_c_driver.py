"""A C driver of the reference's time loop on the C ABI (tests/c_driver/
driver.c, the binding of INTEGRATION.md): it builds against
include/sclet_gb300.h and libsclet_gb300.so on the host; on a GB300 it runs
the golden cases stage by stage and must give the same states as the
reference's own code (oracle/_ref fixtures, 1e-10) and, bit for bit, the same
as sclet_step through the Python binding."""
import os
import subprocess

import numpy as np
import pytest

import case_defs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_driver", "driver.c")
PKG = os.path.join(ROOT, "energy-stability_gb300")


def build_driver(out_dir: str) -> str:
    exe = os.path.join(out_dir, "sclet_driver")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", PKG, "-lsclet_gb300", f"-Wl,-rpath,{PKG}", "-o", exe], check=True, capture_output=True,
                   text=True)
    return exe


def test_driver_builds_against_the_header(sclet_lib, tmp_path):
    exe = build_driver(str(tmp_path))
    assert os.path.exists(exe)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["full", "formula234"])
def test_driver_runs_golden_case(name, sclet_lib, tmp_path):
    exe = build_driver(str(tmp_path))
    run = tmp_path / "run"
    c = case_defs.write(name, str(run))
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(run), name, str(c.steps), "0", str(out)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    F, n = c.nac + c.nch, c.n
    u = np.fromfile(out, dtype=np.float64).reshape(F, n, n, n)
    g = np.load(os.path.join(case_defs.HERE, f"{name}.npz"))
    for f in range(F):
        assert rel(u[f], g["final"][f]) <= 1e-10, (name, f)
    diag = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("diag")]
    assert len(diag) == c.steps * F
    # the same calls made through the Python binding with sclet_step
    sg = sclet_lib
    p = sg.read_case(str(run), name)
    s = sg.Solver(p, sg.FP64)
    d, v, vi = (np.loadtxt(os.path.join(str(run), f"{k}3{n}.dat")) for k in ("d", "v", "vi"))
    s.set_eigen(d, v, vi)
    s.load_restart_dir(str(run))
    s.step(c.steps)
    np.testing.assert_array_equal(s.get_fields(), u)
    last = np.array([[float(x) for x in ln[3:]] for ln in diag[-F:]])
    np.testing.assert_array_equal(s.check_soln(1), last)
    s.close()
