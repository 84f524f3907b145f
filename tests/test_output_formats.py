"""The alpha driver's checkpoint and 16-bit output formats (write_chk /
read_chk, Dtype2B_E / Dtype2B_CI, write_field2B): host-side file layout and
names on CPU; the device codes and the checkpoint round trip through a
context on the GPU, against the oracle's restatement."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

import bench
import cases
import oracle_py


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def test_chk_file_layout_and_round_trip(sclet_lib, tmp_path):
    L = sclet_lib.lib()
    n = 12
    block = np.random.default_rng(3).standard_normal((n, n, n))
    path = str(tmp_path / "eta0.dat").encode()
    assert L.sclet_write_chk_file(path, 37, n, _dp(block)) == 0
    with open(path, "rb") as fp:
        assert fp.read() == oracle_py.chk_file_bytes(37, block)
    back = np.zeros_like(block)
    irun = ctypes.c_int()
    assert L.sclet_read_chk_file(path, n, ctypes.byref(irun), _dp(back)) == 0
    assert irun.value == 37 and np.array_equal(back, block)
    # a file shorter than the block is an error, not a silent partial read
    with open(path, "r+b") as fp:
        fp.truncate(100)
    assert L.sclet_read_chk_file(path, n, ctypes.byref(irun), _dp(back)) != 0


def test_file_names(sclet_lib):
    L = sclet_lib.lib()
    buf = ctypes.create_string_buffer(256)
    assert L.sclet_chk_path(buf, 256, b"./output/", 2, 1) == 0
    assert buf.value == b"./output/00/eta2_chk1_000000.dat"
    assert L.sclet_field2b_path(buf, 256, b"./data/", sclet_lib.AC, 3, 42) == 0
    assert buf.value == b"./data/00/eta3_000042_000000.dat"
    assert L.sclet_field2b_path(buf, 256, b"./data/", sclet_lib.CH, 0, 7) == 0
    assert buf.value == b"./data/00/c0_000007_000000.dat"
    assert L.sclet_chk_path(buf, 8, b"./output/", 2, 1) != 0  # does not fit


def _params(sg, case):
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        return sg.read_case(td, case.suffix)


@pytest.mark.gpu
@pytest.mark.parametrize("precision_name", ["FP64", "MIXED"])
def test_field_codes_match_oracle(precision_name, sclet_lib):
    sg = sclet_lib
    case = bench.workload(24, seed=4)
    s = sg.Solver(_params(sg, case), getattr(sg, precision_name))
    s.set_fields(bench.block_fields(case))
    s.step(3)
    state = s.get_fields()
    for f in range(s.F):
        kind = 0 if f < s.nac else 1
        np.testing.assert_array_equal(s.field_u16(f), oracle_py.field2b_codes(kind, state[f]))
    s.close()


@pytest.mark.gpu
def test_checkpoint_and_field2b_files(sclet_lib, tmp_path):
    sg = sclet_lib
    case = bench.workload(24, seed=6)
    params = _params(sg, case)
    a = sg.Solver(params, sg.FP64)
    a.set_fields(bench.block_fields(case))
    a.step(2)
    want = a.get_fields()
    out = str(tmp_path) + "/"
    a.write_chk(out, 1, 120)
    a.write_field2b(out, 5, 0)
    for m in range(a.nac):
        with open(os.path.join(out, "00", f"eta{m}_chk1_000000.dat"), "rb") as fp:
            assert fp.read() == oracle_py.chk_file_bytes(120, want[m])
        codes = np.fromfile(os.path.join(out, "00", f"eta{m}_000005_000000.dat"), dtype=np.uint16)
        np.testing.assert_array_equal(codes.reshape(want[m].shape), oracle_py.field2b_codes(0, want[m]))
    # read_chk restores the order parameters into a fresh context
    b = sg.Solver(params, sg.FP64)
    assert b.read_chk(out, 1) == 120
    got = b.get_fields()
    for m in range(a.nac):
        assert np.array_equal(got[m], want[m])
    a.close()
    b.close()


def test_vtk_file_matches_restated_script(sclet_lib, tmp_path):
    L = sclet_lib.lib()
    n, nf = 6, 3
    blocks = np.random.default_rng(9).uniform(-1.0, 1.0, (nf, n, n, n)) * np.array([1.0, 1e-3, 1e5])[:, None, None, None]
    path = str(tmp_path / "time_300.vtk").encode()
    assert L.sclet_write_vtk_file(path, 300, n, nf, _dp(np.ascontiguousarray(blocks))) == 0
    with open(path) as fp:
        assert fp.read() == oracle_py.vtk_text(300, blocks)


@pytest.mark.gpu
def test_vtk_of_context_state(sclet_lib, tmp_path):
    sg = sclet_lib
    case = bench.workload(24, seed=2)
    s = sg.Solver(_params(sg, case), sg.MIXED)
    s.set_fields(bench.block_fields(case))
    s.step(1)
    state = s.get_fields()
    path = str(tmp_path / "time_1.vtk")
    s.write_vtk(path, 1)
    with open(path) as fp:
        assert fp.read() == oracle_py.vtk_text(1, state[:s.nac])
    s.close()


def test_soln_logs_match_restated_check_soln(sclet_lib, tmp_path):
    L = sclet_lib.lib()
    nac, nch = 4, 1
    rng = np.random.default_rng(4)
    want = {}
    for it in (0, 1, 2):
        d = np.ascontiguousarray(rng.normal(0.0, 1e3, (nac + nch, 4)))
        couple = np.array([-1234.5 * (it + 1)])
        assert L.sclet_append_soln_log((str(tmp_path) + "/").encode(), it, nac, nch, _dp(d), _dp(couple)) == 0
        for name, text in oracle_py.soln_log_rows(it, nac, nch, d, couple[0]).items():
            want[name] = want.get(name, "") + text
    assert sorted(p.name for p in tmp_path.iterdir()) == sorted(want)
    for name, text in want.items():
        assert (tmp_path / name).read_text() == text, name


@pytest.mark.gpu
def test_soln_logs_of_context(sclet_lib, tmp_path):
    sg = sclet_lib
    case = bench.workload(24, seed=3)
    s = sg.Solver(_params(sg, case), sg.FP64)
    s.set_fields(bench.block_fields(case))
    work = str(tmp_path) + "/"
    want = {}
    for it in range(3):
        if it:
            s.step(1)
        d0, d1 = s.check_soln(0), s.check_soln(1)
        s.log_soln(work, it, 0)
        for name, text in oracle_py.soln_log_rows(it, s.nac, s.F - s.nac, d0, d1[0, 3]).items():
            want[name] = want.get(name, "") + text
    for name, text in want.items():
        assert (tmp_path / name).read_text() == text, name
    s.close()
