"""Runs the reference's own code (oracle/_ref/libsclet_ref*.so) on a case
directory written by oracle/cases.py and saves arrays to an .npz file.
Test infrastructure; each run is a fresh process (the reference keeps its state
in process globals).

    python oracle/ref_runner.py LIB CASE_DIR SUFFIX STEPS OUT.npz [--probe|--rhs|--check]

Saved arrays (n = block edge incl. ghosts, layout [z, y, x]):
  ac{m} / ch{m}      field after STEPS loop passes
With --rhs, instead of stepping, one right-hand-side evaluation (ref_rhs) on
the initial state:
  ac{m}_rhs0 ...     right-hand side fieldE1 / fieldCI1
  ac{m}_filled0      field after the halo exchange
  ac{m}_felas0       elastic force
  ac{m}_u{face}0     boundary values (faces l,r,t,b,f,k)
  ch{m}_mu{face}0    CH boundary chemical potential
  mats               MPX, MPY, MPZ, MPXI, MPYI, MPZI (n x n, column-major)
  dd                 DDX, DDY, DDZ
With --probe the first pass is replaced by a halo probe: every cell of every
field is set to a unique code (its linear index + 1 + 10^7 * field) before
transfer() and calc_mu(), so the saved ghost cells and boundary values name the
cell they were copied from.
With --check the reference's own check_soln_new runs after every pass, as in
its time loop, and writes its CSV logs under CASE_DIR/output/.
"""
import ctypes
import os
import sys

import numpy as np

FACES = "lrtbfk"


def main(argv):
    lib_path, case_dir, suffix, steps, out = argv[:5]
    probe = "--probe" in argv
    steps = int(steps)
    lib = ctypes.CDLL(os.path.abspath(lib_path))
    lib.ref_ptr.restype = ctypes.POINTER(ctypes.c_double)
    lib.ref_mat.restype = ctypes.POINTER(ctypes.c_double)
    lib.ref_h.restype = ctypes.c_double
    out = os.path.abspath(out)
    os.chdir(case_dir)
    rc = lib.ref_init(suffix.encode())
    if rc != 0:
        raise SystemExit(f"ref_init failed: {rc}")
    n = ctypes.c_int.in_dll(lib, "nx").value
    nac = ctypes.c_int.in_dll(lib, "nac").value
    nch = ctypes.c_int.in_dll(lib, "nch").value
    n3 = n * n * n
    save = {}

    def arr(kind, m, which, size):
        p = lib.ref_ptr(kind, m, which)
        return np.ctypeslib.as_array(p, shape=(size,))

    mats = np.stack([np.ctypeslib.as_array(lib.ref_mat(i), shape=(n * n,)).copy() for i in range(6)])
    dd = np.stack([np.ctypeslib.as_array(lib.ref_mat(6 + i), shape=(n,)).copy() for i in range(3)])
    save["mats"] = mats
    save["dd"] = dd
    save["h"] = np.array([lib.ref_h(0), lib.ref_h(1), lib.ref_h(2)])
    kinds = [(0, "ac", m) for m in range(nac)] + [(1, "ch", m) for m in range(nch)]
    save["init_fields"] = np.stack([arr(k, m, 0, n3).copy() for k, _, m in kinds]).reshape(-1, n, n, n)

    lib.ref_set_check(1 if "--check" in argv else 0)
    if probe:
        for f, (k, _, m) in enumerate(kinds):
            a = arr(k, m, 0, n3)
            a[:] = np.arange(n3, dtype=np.float64) + 1.0 + 1.0e7 * f
        lib.transfer()
        lib.calc_mu()
        for k, name, m in kinds:
            save[f"{name}{m}"] = arr(k, m, 0, n3).copy().reshape(n, n, n)
            for fi, face in enumerate(FACES):
                save[f"{name}{m}_u{face}0"] = arr(k, m, 3 + fi, n * n).copy().reshape(n, n)
                save[f"{name}{m}_e{face}0"] = arr(k, m, 17 + fi, 4 * (n + 4) * (n + 4)).copy()
        np.savez(out, **save)
        return
    if "--rhs" in argv:
        lib.ref_rhs()
        for k, name, m in kinds:
            save[f"{name}{m}_rhs0"] = arr(k, m, 1, n3).copy().reshape(n, n, n)
            save[f"{name}{m}_felas0"] = arr(k, m, 2, n3).copy().reshape(n, n, n)
            save[f"{name}{m}_filled0"] = arr(k, m, 0, n3).copy().reshape(n, n, n)
            for fi, face in enumerate(FACES):
                save[f"{name}{m}_u{face}0"] = arr(k, m, 3 + fi, n * n).copy().reshape(n, n)
                save[f"{name}{m}_mu{face}0"] = arr(k, m, 9 + fi, n * n).copy().reshape(n, n)
        np.savez(out, **save)
        return
    for s in range(steps):
        lib.ref_step()
    for k, name, m in kinds:
        save[f"{name}{m}"] = arr(k, m, 0, n3).copy().reshape(n, n, n)
    np.savez(out, **save)


if __name__ == "__main__":
    main(sys.argv[1:])
