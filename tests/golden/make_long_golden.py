"""Generates tests/golden/beta_omega_64_1000.npz by running the reference's own
code (oracle/_ref/libsclet_ref.so, built by oracle/Makefile.ref from the
reference sources) on the 64^3 beta->omega workload for 1000 steps:

    python tests/golden/make_long_golden.py

Workload: 4 non-conserved order parameters U(-0.01, 0.01) from seed 2024 on a
64^3 periodic grid, Landau 2-4-6 (a2 = -1, a4 = -1, a6 = 2, cross term 1.5),
gradient coefficient 0.5, cubic elasticity C11/C12/C44 = 1.0/0.6/0.4 with the
four <111> eigenstrains, dt = 0.01, first-order ETD.  Stored: the owned cells
of every field after 1000 passes (float64) and the reference's check_soln_new
record of every pass (its CSV logs).  Takes about an hour on one core (the
reference's DGEMM stand-in is sequential).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import cases  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libsclet_ref.so")
RUNNER = os.path.join(ROOT, "oracle", "ref_runner.py")
NAME = "beta_omega_64_1000"


def long_case() -> "cases.Case":
    return cases.Case(big_n=64, nac=4, nch=0, dt=0.01, steps=1000, epn2=0.5, elastic=1, seed=2024,
                      suffix="bo64")


def main():
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref"], cwd=ROOT, check=True)
    c = long_case()
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(c, td)
        run = os.path.join(td, "run.npz")
        subprocess.run([sys.executable, RUNNER, LIB, td, c.suffix, str(c.steps), run, "--check"], check=True,
                       capture_output=True)
        S = np.load(run)
        own = (slice(2, -2),) * 3
        final = np.stack([S[f"ac{m}"][own] for m in range(c.nac)])
        diag = np.stack([np.loadtxt(os.path.join(td, "output", f"phi_ac_{m}.csv"), delimiter=",", skiprows=1,
                                    ndmin=2)[:, 1:] for m in range(c.nac)])
    np.savez_compressed(os.path.join(HERE, f"{NAME}.npz"), final=final, diag=diag)
    print(NAME, final.shape, diag.shape)


if __name__ == "__main__":
    main()
