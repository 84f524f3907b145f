"""Input-case writer for the test oracle (test infrastructure).

Writes a run directory in the reference's own file formats so the same case can
be fed to the reference (oracle/_ref), to the C restatement (oracle/) and to the
CUDA path:

* ``input<suffix>.ini`` -- positional format of
  source_beta_to_omega/src/ScLETD.c:16-34;
* ``elastic_input.txt`` -- ElasticScale, 6x6 Voigt stiffness, four 3x3
  eigenstrains (src/elastic.c:349-439);
* ``anisotropic_input.txt`` -- nac 3x3 gradient tensors (src/anisotropic.c:630-674);
* ``landau_input.txt`` -- the physics plugin's constants
  (a2 a4 a6 g th c0 A LE KE LCI KCI);
* ``d{k}{n}.dat``, ``v{k}{n}.dat``, ``vi{k}{n}.dat`` -- per-axis eigen data in
  the layout read by src/vars.c:370-476 (one eigenvalue per line; matrices
  row by row);
* ``input/field_iter0_ac{m}_000.txt`` / ``..._ch{m}_000.txt`` -- seeded initial
  interior values, read by the restart path (src/field.c:746-754, 137-154).

Seeded values use a counter-based generator (SplitMix64 on seed, field and
global cell index), identical in C (energy-stability_gb300/csrc/sclet_seed.h).
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Optional, Sequence

import numpy as np

MASK64 = (1 << 64) - 1


# ---------------------------------------------------------------------------
# Eigen data for the 1D second-difference matrix (src/vars.c:361-591 reads it)
# ---------------------------------------------------------------------------
def second_difference(n: int, variant: int) -> np.ndarray:
    """1D second-difference matrix of the boundary variant the reference keys
    as ``id = (k-1) + (l-1)*2`` (src/vars.c:488-506): 0 Neumann-Neumann,
    1 Dirichlet-left/Neumann-right, 2 Neumann-left/Dirichlet-right,
    3 Dirichlet-Dirichlet.  Neumann rows use the ghost-reflected stencil
    [-2, 2]."""
    t = np.zeros((n, n))
    for i in range(n):
        t[i, i] = -2.0
        if i > 0:
            t[i, i - 1] = 1.0
        if i < n - 1:
            t[i, i + 1] = 1.0
    if variant in (0, 2):
        t[0, 1] = 2.0
    if variant in (0, 1):
        t[n - 1, n - 2] = 2.0
    return t


def eigen_variant(n: int, variant: int):
    """Returns (d, V, Vi) with V diag(d) Vi = second_difference(n, variant),
    eigenvalues ascending.  Variant 3 is the closed-form DST-I basis
    (orthonormal, Vi = V^T); the others come from a dense eigensolver with
    unit-norm columns and Vi = V^-1."""
    if variant == 3:
        k = np.arange(n, 0, -1, dtype=np.float64)  # ascending eigenvalues
        d = -4.0 * np.sin(k * np.pi / (2.0 * (n + 1))) ** 2
        j = np.arange(1, n + 1, dtype=np.float64)
        v = np.sqrt(2.0 / (n + 1)) * np.sin(np.pi * np.outer(j, k) / (n + 1))
        return d, v, v.T.copy()
    t = second_difference(n, variant)
    w, v = np.linalg.eig(t)
    w = w.real
    v = v.real
    order = np.argsort(w)
    w = w[order]
    v = v[:, order]
    v /= np.linalg.norm(v, axis=0, keepdims=True)
    return w, v, np.linalg.inv(v)


def write_eigen_files(dirpath: str, n: int, variants: Sequence[int] = (0, 1, 2, 3)) -> None:
    for k in variants:
        d, v, vi = eigen_variant(n, k)
        with open(os.path.join(dirpath, f"d{k}{n}.dat"), "w") as fp:
            for x in d:
                fp.write("%25.16e\n" % x)
        for name, m in (("v", v), ("vi", vi)):
            with open(os.path.join(dirpath, f"{name}{k}{n}.dat"), "w") as fp:
                for row in m:
                    fp.write("".join("%25.16e" % x for x in row) + "\n")


# ---------------------------------------------------------------------------
# Seeded values: SplitMix64(seed, field, cell) -> 53-bit uniform in [0, 1)
# ---------------------------------------------------------------------------
def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(MASK64)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def seeded_uniform(seed: int, field: int, count: int) -> np.ndarray:
    """U[0,1) values for cells 0..count-1 of one field (53-bit resolution)."""
    with np.errstate(over="ignore"):
        key = np.uint64((seed * 0xD1B54A32D192ED03 + (field + 1) * 0xA0761D6478BD642F) & MASK64)
        idx = np.arange(count, dtype=np.uint64)
        z = _splitmix64(idx ^ key)
        z = _splitmix64(z)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def seeded_field(seed: int, field: int, big_n: int, lo: float, hi: float) -> np.ndarray:
    """Interior values of one field, shape (N, N, N) indexed [z, y, x]."""
    u = seeded_uniform(seed, field, big_n ** 3)
    return (lo + (hi - lo) * u).reshape(big_n, big_n, big_n)


# ---------------------------------------------------------------------------
# Case description and writer
# ---------------------------------------------------------------------------
def rhombohedral_eigenstrains(diag: float = 0.01, off: float = 0.005) -> List[np.ndarray]:
    """Four <111> variants: eps_ii = diag, eps_ij = off * d_i d_j."""
    out = []
    for d in ((1, 1, 1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1)):
        e = np.full((3, 3), 0.0)
        for i in range(3):
            for j in range(3):
                e[i, j] = diag if i == j else off * d[i] * d[j]
        out.append(e)
    return out


def cubic_voigt(c11: float, c12: float, c44: float) -> np.ndarray:
    c = np.zeros((6, 6))
    c[:3, :3] = c12
    for i in range(3):
        c[i, i] = c11
        c[3 + i, 3 + i] = c44
    return c


# physics plugin names of physics_input.txt (read by sclet_read_case)
PHYSICS_NAMES = {0: "landau246", 1: "formula234"}


@dataclasses.dataclass
class Case:
    big_n: int = 64                 # physical edge N; block edge n = N + 4
    nac: int = 4
    nch: int = 0
    dt: float = 0.01
    steps: int = 1000
    epn2: float = 0.5
    length: Optional[float] = None  # domain edge; default N/2 (h = 0.5)
    etd2: int = 0
    elastic: int = 1                # 0 none, 1 Allen-Cahn (AC_FUNCTION)
    anisotropic: int = 0
    kk: Sequence[float] = (1.0, 1.0, 1.0)
    lambdas: Optional[Sequence[np.ndarray]] = None   # per-AC-field 3x3 (file values)
    elastic_scale: float = 50.0
    voigt: np.ndarray = dataclasses.field(default_factory=lambda: cubic_voigt(1.0, 0.6, 0.4))
    eigenstrains: List[np.ndarray] = dataclasses.field(default_factory=rhombohedral_eigenstrains)
    landau: Sequence[float] = (-1.0, -1.0, 2.0, 1.5, 0.8, 0.5, 1.0, 1.0, 6.0, 1.0, 2.0)
    seed: int = 1234
    eta_range: Sequence[float] = (-0.01, 0.01)
    c_range: Sequence[float] = (0.48, 0.52)
    suffix: str = "case"
    physics: int = 0                # 0 Landau 2-4-6 plugin, 1 the reference's own formula.c
    variable_mobility: int = 0      # VariableMobility of the ini (mobility.c:838-922)

    @property
    def n(self) -> int:
        return self.big_n + 4

    @property
    def domain(self) -> float:
        return self.length if self.length is not None else self.big_n / 2.0

    def initial_fields(self):
        """List of (kind, index, (N,N,N) array [z,y,x]) interior values."""
        out = []
        for m in range(self.nac):
            out.append(("ac", m, seeded_field(self.seed, m, self.big_n, *self.eta_range)))
        for m in range(self.nch):
            out.append(("ch", m, seeded_field(self.seed, self.nac + m, self.big_n, *self.c_range)))
        return out


def write_case(case: Case, dirpath: str, eigen: bool = True, fields: bool = True) -> None:
    os.makedirs(os.path.join(dirpath, "input"), exist_ok=True)
    os.makedirs(os.path.join(dirpath, "output"), exist_ok=True)
    os.makedirs(os.path.join(dirpath, "restart"), exist_ok=True)
    os.makedirs(os.path.join(dirpath, "data"), exist_ok=True)  # outputfield, src/field.c:17-56
    n = case.n
    t_total = (case.steps - 0.5) * case.dt
    with open(os.path.join(dirpath, f"input{case.suffix}.ini"), "w") as fp:
        fp.write(f" {n}, {n}, {n}\n 1, 1, 1\n 2\n ./output/\n ./data/\n")
        fp.write(f" {case.dt!r}, {t_total!r}\n {case.epn2!r}\n 1\n {case.nac}, {case.nch}\n")
        fp.write(" 1, 0, ./restart/\n 0, 0, 0\n")
        L = case.domain
        fp.write(f" {L!r}, {L!r}, {L!r}\n {case.etd2}\n {case.elastic}\n {case.anisotropic}\n")
        fp.write(f" {case.kk[0]!r}, {case.kk[1]!r}, {case.kk[2]!r}\n {case.variable_mobility}\n")
    with open(os.path.join(dirpath, "elastic_input.txt"), "w") as fp:
        fp.write(f"{case.elastic_scale!r}\n\n")
        for row in case.voigt:
            fp.write(" ".join(repr(float(x)) for x in row) + "\n")
        for e in case.eigenstrains:
            fp.write("\n")
            for row in e:
                fp.write(" ".join(repr(float(x)) for x in row) + "\n")
    lambdas = case.lambdas
    if lambdas is None:
        lambdas = [np.zeros((3, 3)) for _ in range(case.nac)]
    with open(os.path.join(dirpath, "anisotropic_input.txt"), "w") as fp:
        for m in range(case.nac):
            for row in np.asarray(lambdas[m]):
                fp.write(" ".join(repr(float(x)) for x in row) + "\n")
            fp.write("\n")
    with open(os.path.join(dirpath, "landau_input.txt"), "w") as fp:
        fp.write(" ".join(repr(float(x)) for x in case.landau) + "\n")
    if case.physics:
        with open(os.path.join(dirpath, "physics_input.txt"), "w") as fp:
            fp.write(PHYSICS_NAMES[case.physics] + "\n")
    for kind, m, vals in (case.initial_fields() if fields else []):
        with open(os.path.join(dirpath, "input", f"field_iter0_{kind}{m}_000.txt"), "w") as fp:
            np.savetxt(fp, vals.reshape(-1), fmt="%.17g")
    if eigen:
        write_eigen_files(dirpath, n)
