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
