"""Generates the golden fixtures in tests/golden/ by running the reference's
own code (oracle/_ref, built by oracle/Makefile.ref from the reference
sources) on the cases of cases.json.  Run here, where the reference exists:

    python tests/golden/make_golden.py

For each case it stores, from the reference: the right-hand side, the halo-
filled fields, boundary values and elastic force of the first evaluation
(ref_runner --rhs), the state after `steps` loop passes, and the reference
binary's own check_soln_new diagnostics of every pass (its CSV files).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import case_defs  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libsclet_ref.so")
# the reference built with its own formula.c (the 2-3-4 physics)
LIB_ORIG = os.path.join(ROOT, "oracle", "_ref", "libsclet_ref_orig.so")
BIN = os.path.join(ROOT, "oracle", "_ref", "ScLETD_ref")
RUNNER = os.path.join(ROOT, "oracle", "ref_runner.py")


sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ref_paths  # noqa: E402

# the reference checkout: SCLET_REFERENCE_ROOT, else the build recipe's default
EIGEN_DIR = os.path.join(ref_paths.reference_root(), "source_beta_to_alpha")


def eigen260():
    """Summary of the reference's shipped n = 260 eigen files: eigenvalues,
    the stencil rows V diag(d) V^-1 reproduces, and per-column sums of |V|."""
    out = {}
    for k in range(4):
        d = np.loadtxt(os.path.join(EIGEN_DIR, f"d{k}260.dat"))
        v = np.loadtxt(os.path.join(EIGEN_DIR, f"v{k}260.dat"))
        vi = np.loadtxt(os.path.join(EIGEN_DIR, f"vi{k}260.dat"))
        t = v @ np.diag(d) @ vi
        out[f"d{k}"] = d
        out[f"T{k}"] = np.round(t[[0, 1, -2, -1]], 12)
        out[f"colabs{k}"] = np.abs(v).sum(axis=0)
    np.savez_compressed(os.path.join(HERE, "eigen260.npz"), **out)


def main(only=None):
    """All cases of cases.json, or only the named ones.  Cases with physics 1
    run the reference built with its own formula.c; their per-pass
    diagnostics come from its check_soln_new inside the stepping run."""
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref"], cwd=ROOT, check=True)
    if not only:
        eigen260()
    for name in case_defs.load_defs():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            c = case_defs.write(name, td)
            lib = LIB_ORIG if c.physics == 1 else LIB
            # the reference binary itself runs only where its main() is safe:
            # its variable-mobility path writes three concentrations' mobility
            # (update_M_C, mobility.c:860-922), so with nch < 3 only the
            # harness (which gives ch[] three entries) runs it
            own_check = c.physics == 1 or c.variable_mobility == 1
            rhs = os.path.join(td, "rhs.npz")
            run = os.path.join(td, "run.npz")
            subprocess.run([sys.executable, RUNNER, lib, td, name, "0", rhs, "--rhs"], check=True,
                           capture_output=True)
            subprocess.run([sys.executable, RUNNER, lib, td, name, str(c.steps), run]
                           + (["--check"] if own_check else []), check=True, capture_output=True)
            if not own_check:
                subprocess.run([BIN, name], cwd=td, check=True, capture_output=True)
            R, S = np.load(rhs), np.load(run)
            out = {}
            names = [f"ac{m}" for m in range(c.nac)] + [f"ch{m}" for m in range(c.nch)]
            out["rhs0"] = np.stack([R[f"{k}_rhs0"] for k in names])
            out["filled0"] = np.stack([R[f"{k}_filled0"] for k in names])
            if c.elastic:
                out["felas0"] = np.stack([R[f"ac{m}_felas0"] for m in range(c.nac)])
            out["final"] = np.stack([S[k] for k in names])
            diags = []
            for k in names:
                kind = "ac" if k.startswith("ac") else "ch"
                diags.append(np.loadtxt(os.path.join(td, "output", f"phi_{kind}_{k[2:]}.csv"), delimiter=",",
                                        skiprows=1, ndmin=2)[:, 1:])
            out["diag"] = np.stack(diags)  # [field][pass][max,min,vol,eng]
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
            print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv[1:] or None)
