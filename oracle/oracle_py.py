"""ctypes front end of the C oracle (oracle/liboracle_sclet.so).

TEST INFRASTRUCTURE: used by tests/, __graft_entry__.smoke() and the bench's
CPU-baseline leg as the oracle; never by the product path.

``load_case(dir, suffix)`` parses a run directory in the reference's formats
(see oracle/cases.py) with numpy, independently of the product's C parser, and
``Oracle`` holds a state and calls the C restatement.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_sclet.so")

_dp = ctypes.POINTER(ctypes.c_double)


class OrcCfg(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("nac", ctypes.c_int), ("nch", ctypes.c_int),
        ("etd2", ctypes.c_int), ("elastic", ctypes.c_int), ("anisotropic", ctypes.c_int),
        ("dt", ctypes.c_double), ("epn2", ctypes.c_double),
        ("h", ctypes.c_double * 3), ("kk", ctypes.c_double * 3),
        ("lam", ctypes.c_double * 36),
        ("elastic_scale", ctypes.c_double),
        ("physics", ctypes.c_int),
        ("K", ctypes.c_double * 16),
        ("LE", ctypes.c_double), ("KE", ctypes.c_double),
        ("LCI", ctypes.c_double), ("KCI", ctypes.c_double),
        ("mp", _dp * 3), ("mpi", _dp * 3), ("dd", _dp * 3),
        ("bn", _dp),
        ("elam", ctypes.c_double * 36),
        ("energy_form", ctypes.c_int),
        ("variable_mobility", ctypes.c_int),
    ]


def build(out_dir: str = HERE) -> str:
    """Compiles the C oracle (gcc, OpenMP when available) into out_dir."""
    import subprocess
    srcs = [os.path.join(HERE, "sclet_oracle.c"), os.path.join(HERE, "ref_shims", "oracle_fft.c")]
    out = os.path.join(out_dir, "liboracle_sclet.so")
    base = ["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-I" + HERE, "-o", out] + srcs + ["-lm"]
    try:
        subprocess.run(base[:4] + ["-fopenmp"] + base[4:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True)
    return out


def _lib():
    lib = ctypes.CDLL(LIB_PATH)
    lib.orc_threads.restype = ctypes.c_int
    return lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _read_numbers(path: str):
    with open(path) as fp:
        return [float(t) for t in fp.read().replace(",", " ").split()]


def load_case(case_dir: str, suffix: str, fields=None) -> Dict:
    """Parses a run directory (ini: source_beta_to_omega/src/ScLETD.c:16-34).
    `fields` (F, n, n, n) replaces the restart files as initial state."""
    with open(os.path.join(case_dir, f"input{suffix}.ini")) as fp:
        lines = [ln.strip() for ln in fp if ln.strip()]
    nums = lambda s: [float(t) for t in s.replace(",", " ").split()]
    p = {}
    p["n"] = int(nums(lines[0])[0])
    p["dt"], p["t_total"] = nums(lines[5])
    p["epn2"] = nums(lines[6])[0]
    p["nac"], p["nch"] = [int(v) for v in nums(lines[8])]
    lo, hi = nums(lines[10]), nums(lines[11])
    p["etd2"] = int(nums(lines[12])[0])
    p["elastic"] = int(nums(lines[13])[0])
    p["anisotropic"] = int(nums(lines[14])[0])
    p["kk"] = nums(lines[15])
    p["variable_mobility"] = int(nums(lines[16])[0]) if len(lines) > 16 else 0
    n = p["n"]
    big_n = n - 4
    p["h"] = [(hi[d] - lo[d]) / big_n for d in range(3)]
    el = _read_numbers(os.path.join(case_dir, "elastic_input.txt"))
    p["elastic_scale"] = el[0]
    p["voigt"] = np.array(el[1:37]).reshape(6, 6)
    p["eps"] = np.array(el[37:73]).reshape(4, 3, 3)
    lam_file = np.zeros((4, 3, 3))
    if p["anisotropic"]:
        an = _read_numbers(os.path.join(case_dir, "anisotropic_input.txt"))
        lam_file[: p["nac"]] = np.array(an[: 9 * p["nac"]]).reshape(p["nac"], 3, 3)
    p["lam_file"] = lam_file
    p["landau"] = _read_numbers(os.path.join(case_dir, "landau_input.txt"))
    p["physics"] = 0
    phys = os.path.join(case_dir, "physics_input.txt")
    if os.path.exists(phys):
        with open(phys) as fp:
            p["physics"] = {"landau246": 0, "formula234": 1}[fp.read().split()[0]]
    # eigen data of the Dirichlet-Dirichlet variant (id 3, src/vars.c:488-582):
    # the case's files when written, else the closed form
    if os.path.exists(os.path.join(case_dir, f"d3{n}.dat")):
        d = np.loadtxt(os.path.join(case_dir, f"d3{n}.dat"))
        v = np.loadtxt(os.path.join(case_dir, f"v3{n}.dat"))
        vi = np.loadtxt(os.path.join(case_dir, f"vi3{n}.dat"))
    else:
        import cases
        d, v, vi = cases.eigen_variant(n, 3)
    p["d"], p["v"], p["vi"] = d, v, vi
    if fields is not None:
        p["fields"] = np.ascontiguousarray(fields, dtype=np.float64)
        return p
    fields = []
    for kind, cnt in (("ac", p["nac"]), ("ch", p["nch"])):
        for m in range(cnt):
            vals = np.loadtxt(os.path.join(case_dir, "input", f"field_iter0_{kind}{m}_000.txt"))
            blk = np.zeros((n, n, n))
            blk[2:-2, 2:-2, 2:-2] = vals.reshape(big_n, big_n, big_n)
            fields.append(blk)
    p["fields"] = np.stack(fields)
    return p


def load_case_params(case_dir: str, suffix: str, fields) -> Dict:
    return load_case(case_dir, suffix, fields=fields)


class Oracle:
    """C oracle state for one case.  ``u`` is (F, n, n, n) incl. ghosts."""

    def __init__(self, p: Dict, energy_form: int = 1):
        self.lib = _lib()
        self.p = p
        n = p["n"]
        self.n = n
        self.F = p["nac"] + p["nch"]
        c = OrcCfg()
        c.n, c.nac, c.nch = n, p["nac"], p["nch"]
        c.etd2, c.elastic, c.anisotropic = p["etd2"], p["elastic"], p["anisotropic"]
        c.dt, c.epn2 = p["dt"], p["epn2"]
        for d in range(3):
            c.h[d] = p["h"][d]
            c.kk[d] = p["kk"][d]
        lam = np.zeros((4, 3, 3))
        for m in range(p["nac"]):
            lam[m] = np.diag(p["kk"]) - p["lam_file"][m]
        self.lam = lam
        for i, v in enumerate(lam.reshape(-1)):
            c.lam[i] = v
        c.elastic_scale = p["elastic_scale"]
        # physics plugin: 0 the Landau 2-4-6 form (landau_input.txt), 1 the
        # reference's own formula.c (2-3-4, LE = 1, KE = 42)
        c.physics = p.get("physics", 0)
        for i, v in enumerate(p["landau"] if c.physics == 0 else []):
            c.K[i] = v
        if self.lib.orc_physics_setup(ctypes.byref(c)) != 0:
            raise ValueError(f"unknown physics plugin {c.physics}")
        # matrices column-major like the reference (element (r, c) at c*n + r)
        self._keep = []
        for d in range(3):
            mp = np.ascontiguousarray(p["v"].T.reshape(-1))
            mpi = np.ascontiguousarray(p["vi"].T.reshape(-1))
            dd = np.ascontiguousarray(p["d"] / p["h"][d] ** 2)
            self._keep += [mp, mpi, dd]
            c.mp[d], c.mpi[d], c.dd[d] = _ptr(mp), _ptr(mpi), _ptr(dd)
        big_n = n - 4
        if p["elastic"]:
            self.bn = np.zeros(16 * big_n ** 3)
            self.lib.orc_compute_bn(ctypes.c_int(big_n), _ptr(np.ascontiguousarray(p["voigt"].reshape(-1))),
                                    _ptr(np.ascontiguousarray(p["eps"].reshape(-1))), _ptr(self.bn))
            c.bn = _ptr(self.bn)
        # energy tensors: the gradient operator of the dynamics (the file
        # tensors when ANISOTROPIC, else diag(kk)); the reference's own
        # check_soln_new uses diag(kk) - file tensor (set_energy_tensors)
        elam = np.zeros((4, 3, 3))
        for m in range(p["nac"]):
            elam[m] = p["lam_file"][m] if p["anisotropic"] else np.diag(p["kk"])
        for i, v in enumerate(elam.reshape(-1)):
            c.elam[i] = v
        c.energy_form = energy_form
        c.variable_mobility = p.get("variable_mobility", 0)
        self.cfg = c
        self.u = np.ascontiguousarray(p["fields"].copy())
        self.felas = np.zeros((max(p["nac"], 1), n, n, n))
        self.fstate = np.zeros((n, n, n))

    def set_energy_tensors(self, elam: np.ndarray, form: int) -> None:
        for i, v in enumerate(np.asarray(elam, dtype=np.float64).reshape(-1)):
            self.cfg.elam[i] = v
        self.cfg.energy_form = form

    def step(self, k: int = 1) -> None:
        for _ in range(k):
            self.lib.orc_step(ctypes.byref(self.cfg), _ptr(self.u), _ptr(self.felas), _ptr(self.fstate))

    def rhs(self) -> np.ndarray:
        """Fill + elastic + right-hand sides on the current state (modifies
        ghosts and elastic scratch like the reference's first half-pass)."""
        for m in range(self.F):
            self.lib.orc_ghost_fill(ctypes.c_int(self.n), _ptr(self.u[m]))
        if self.p["elastic"]:
            self.lib.orc_elastic(ctypes.byref(self.cfg), _ptr(self.u), _ptr(self.felas), _ptr(self.fstate))
        out = np.zeros_like(self.u)
        self.lib.orc_rhs(ctypes.byref(self.cfg), _ptr(self.u), _ptr(self.felas), _ptr(out))
        return out

    def check_soln(self) -> np.ndarray:
        out = np.zeros(self.F * 4)
        self.lib.orc_check_soln(ctypes.byref(self.cfg), _ptr(self.u), _ptr(out))
        return out.reshape(self.F, 4)

    def mode_product(self, mat_colmajor: np.ndarray, a: np.ndarray) -> np.ndarray:
        out = np.zeros_like(a)
        self.lib.orc_mode_product(ctypes.c_int(self.n), _ptr(np.ascontiguousarray(mat_colmajor)),
                                  _ptr(np.ascontiguousarray(a)), _ptr(out))
        return out

    def threads(self) -> int:
        return self.lib.orc_threads()


# ---- the alpha driver's output formats (restated; its HIP code cannot run here) ----

def chk_file_bytes(irun: int, block: np.ndarray) -> bytes:
    """write_chk (source_beta_to_alpha/src/vars.c:966-989): the step counter
    as a native int, then every cell of the block as native doubles."""
    return np.array([irun], dtype=np.int32).tobytes() + np.ascontiguousarray(block, dtype=np.float64).tobytes()


def field2b_codes(kind: int, block: np.ndarray) -> np.ndarray:
    """Dtype2B_E / Dtype2B_CI (source_beta_to_alpha/src/anisotropic_hip.c:
    3920-3944): (eta + 0.1) * 30000 for order parameters (kind 0), c * 50000
    for concentrations (kind 1), truncated toward zero to unsigned short.
    Defined by the reference only inside [0, 65535]; callers keep to that."""
    v = (block + 0.1) * 30000.0 if kind == 0 else block * 50000.0
    return np.trunc(v).astype(np.uint16)


def vtk_text(istep: int, blocks: np.ndarray) -> str:
    """The VTK layout of visualisation/write_vtk.py:57-101, restated: legacy ASCII
    structured grid of the whole block, points with x fastest written as
    (z, y, x) with 14-wide six-digit exponent format, then one float scalar
    block per field named eta0, eta1, ..."""
    nf, n = blocks.shape[0], blocks.shape[1]
    cells = n ** 3
    out = ["# vtk DataFile Version 2.0", f"time_{istep:d}.vtk", "ASCII", "DATASET STRUCTURED_GRID",
           f"DIMENSIONS {n:>5d}  {n:>5d}  {n:>5d}", f"POINTS {cells:>7d} float"]
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    for a, b, c in zip(z.ravel(), y.ravel(), x.ravel()):
        out.append(f"{float(a):>14.6e}   {float(b):>14.6e}   {float(c):>14.6e}")
    out.append(f"POINT_DATA {cells:>5d}")
    for m in range(nf):
        out.append(f"SCALARS eta{m}  float  1")
        out.append("LOOKUP_TABLE default")
        out.extend(f"{v:>14.6e}" for v in blocks[m].ravel())
    return "\n".join(out) + "\n"


def soln_log_rows(iter_: int, nac: int, nch: int, d: np.ndarray, couple=None) -> Dict[str, str]:
    """The lines check_soln_new (source_beta_to_omega/src/field.c:419-455, 524,
    591, 647) adds to its log files for one call, restated: file name -> text.
    d holds (max, min, vol, eng) per field, AC fields first; iter 0 starts each
    file with its header line."""
    out = {}

    def row(name, header, vals):
        text = (header + "\n") if iter_ == 0 else ""
        out[name] = text + str(iter_) + "".join(f",{v:+.15f}" for v in vals) + "\n"

    if couple is not None and nac > 0 and nch > 0:
        row("phi_couple.csv", "iter,eng", [couple])
    for m in range(nac + nch):
        if m < nac:
            row(f"phi_ac_{m}.csv", "iter,maxphiE,minphiE,volE,engE", d[m])
        else:
            row(f"phi_ch_{m - nac}.csv", "iter,maxphiCI,minphiCI,volCI,engCI", d[m])
    return out
