"""Diagnostics without allocation (sclet_check_soln_noalloc): the same
numbers as the context entry point sclet_check_soln for the same state, on two
calls in a row (the fixed scratch is reused), for FP64 and FP32 blocks.  The
state lives in device buffers owned by the test (torch), as a caller with its
own memory would hold it.  Kept in its own file, collected last, so that it
runs both alone in a fresh process and after the other GPU tests."""
import ctypes
import tempfile

import numpy as np
import pytest

import bench
import cases

pytestmark = pytest.mark.gpu


def _params(sg, case):
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        return sg.read_case(td, case.suffix)


def _noalloc(sg, params, precision, dev_fields, form, dev_out):
    msg = ctypes.create_string_buffer(256)
    rc = sg.lib().sclet_check_soln_noalloc(ctypes.byref(params), precision, ctypes.c_void_p(dev_fields.data_ptr()),
                                           form, ctypes.c_void_p(dev_out.data_ptr()), None, msg, len(msg))
    return rc, msg.value.decode()


@pytest.mark.parametrize("anisotropic", [1, 0])
@pytest.mark.parametrize("precision_name", ["FP64", "MIXED"])
def test_noalloc_diagnostics_match_context_path(precision_name, anisotropic, sclet_lib):
    """anisotropic = 1: the energy's gradient tensors are the file tensors;
    0: diag(kk), which the entry point builds itself."""
    torch = pytest.importorskip("torch")
    sg = sclet_lib
    precision = getattr(sg, precision_name)
    case = bench.workload(24, seed=5)  # 4 AC + 1 CH fields
    case.anisotropic = anisotropic
    if not anisotropic:
        case.kk = (0.5, 0.4, 0.3)  # distinct diagonal entries
    params = _params(sg, case)
    u0 = bench.block_fields(case)
    s = sg.Solver(params, precision)
    s.set_fields(u0)
    s.step(3)
    state = s.get_fields()  # FP64 copy of the device state
    if precision == sg.MIXED:
        # FP32 values whose difference from c0 is exact in FP32 too, so that the
        # context (which stores c - c0) and the caller's FP32 block hold the
        # same numbers
        state = state.astype(np.float32).astype(np.float64)
        s.set_fields(state)
    dtype = torch.float64 if precision == sg.FP64 else torch.float32
    dev = torch.from_numpy(np.ascontiguousarray(state)).to(device="cuda:0", dtype=dtype)
    outs = [torch.full((4 * s.F,), float("nan"), dtype=torch.float64, device="cuda:0") for _ in range(4)]
    # a first call does the per-device set-up; later calls must leave the
    # device's free memory as it was
    rc, msg = _noalloc(sg, params, precision, dev, 1, outs[0])
    assert rc == 0, msg
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for form in (0, 1):
        want = s.check_soln(form)
        for call in range(2):
            out = outs[2 * form + call]
            out.fill_(float("nan"))
            rc, msg = _noalloc(sg, params, precision, dev, form, out)
            assert rc == 0, msg
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info(0)[0] == free0, "free device memory changed"
            got = out.cpu().numpy().reshape(s.F, 4)
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=0,
                                       err_msg=f"{precision_name} form {form} call {call}")
    s.close()


def test_noalloc_rejects_sizes_beyond_its_limits(sclet_lib):
    torch = pytest.importorskip("torch")
    sg = sclet_lib
    params = _params(sg, bench.workload(24, seed=5))
    dev = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    out = torch.zeros(20, dtype=torch.float64, device="cuda:0")
    params.nx = params.ny = params.nz = 2000
    rc, msg = _noalloc(sg, params, sg.FP64, dev, 1, out)
    assert rc == 1 and "block edge" in msg
    params.nx = params.ny = params.nz = 28
    params.nac = 6
    rc, msg = _noalloc(sg, params, sg.FP64, dev, 1, out)
    assert rc == 1 and "Allen-Cahn" in msg
