"""Host side of the learned coarse-step corrector (sclet_net_* and
sclet_learned_step of include/sclet_gb300.h): training pairs generated by the
solver itself, the training loop, and coarse stepping judged by the plain-ETD
checks.  Device arrays are torch CUDA tensors (device memory only; every
computation runs in libsclet_gb300.so).

Training pair of a run at fine step t (ratio = coarse dt / fine dt), with
D = coarse(u_t) - u_t the coarse increment and the scale
s = RMS(D) + FLOOR RMS(u_t) (RMS over all cells and fields; the floor keeps s
away from zero where the state has stopped moving):
  input  = [u_t, D / s]                      owned cells, FP32, 8 channels
  target = (fine^ratio(u_t) - coarse(u_t)) / s   4 channels
where coarse is one ETD step of the mixed-precision form with the coarse dt
(the step the corrector is deployed on) and fine^ratio is ratio ETD steps of
the fine dt.  The learned step (sclet_learned_step) forms the same input and
applies s times the output.
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile
from typing import Iterable, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import sclet_gb300 as sg  # noqa: E402

NET_IN, NET_OUT = 8, 4
FLOOR = 1e-3  # SCLET_NET_FLOOR


def pair(u0: np.ndarray, c1: np.ndarray, f1: np.ndarray):
    """(input, target, scale) of one training pair from the start state, the
    coarse step's result and the fine steps' result (owned cells)."""
    d = c1 - u0
    s = float(np.sqrt(np.mean(d * d)) + FLOOR * np.sqrt(np.mean(u0 * u0))) or 1.0
    return np.concatenate([u0, d / s]).astype(np.float32), ((f1 - c1) / s).astype(np.float32), s


def _ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


class Net:
    """One corrector network (a sclet_net)."""

    def __init__(self, device: int = 0, seed: int = 1, out_scale: float = 1.0):
        self.L = sg.lib()
        h = ctypes.c_void_p()
        rc = self.L.sclet_net_create(device, seed, out_scale, ctypes.byref(h))
        if rc != 0:
            msg = self.L.sclet_net_last_error(h).decode() if h else ""
            if h:
                self.L.sclet_net_destroy(h)
            raise sg.ScletError(f"sclet_net_create failed ({rc}): {msg}")
        self.h = h
        self.out_scale = out_scale
        self.nparam = int(self.L.sclet_net_param_count())

    def _ck(self, rc: int, what: str):
        if rc != 0:
            raise sg.ScletError(f"{what} failed ({rc}): {self.L.sclet_net_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.L.sclet_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparam, dtype=np.float32)
        self._ck(self.L.sclet_net_get_params(self.h, out.ctypes.data_as(ctypes.c_void_p)), "get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparam
        self._ck(self.L.sclet_net_set_params(self.h, p.ctypes.data_as(ctypes.c_void_p)), "set_params")

    def forward(self, inp, out):
        """inp [B][8][N,N,N] and out [B][4][N,N,N]: CUDA float32 tensors."""
        import torch
        torch.cuda.synchronize()
        B, N = inp.shape[0], inp.shape[-1]
        self._ck(self.L.sclet_net_forward(self.h, N, B, _ptr(inp), _ptr(out)), "forward")
        self._ck(self.L.sclet_net_sync(self.h), "sync")

    def gradient(self, inp, target):
        import torch
        torch.cuda.synchronize()
        B, N = inp.shape[0], inp.shape[-1]
        loss = ctypes.c_double()
        g = np.zeros(self.nparam, dtype=np.float32)
        self._ck(self.L.sclet_net_gradient(self.h, N, B, _ptr(inp), _ptr(target), ctypes.byref(loss),
                                           g.ctypes.data_as(ctypes.c_void_p)), "gradient")
        return loss.value, g

    def train_step(self, inp, target, lr: float) -> float:
        B, N = inp.shape[0], inp.shape[-1]
        loss = ctypes.c_double()
        self._ck(self.L.sclet_net_train_step(self.h, N, B, _ptr(inp), _ptr(target), lr, ctypes.byref(loss)),
                 "train_step")
        return loss.value


def owned(u: np.ndarray) -> np.ndarray:
    return u[:, 2:-2, 2:-2, 2:-2]


def case_params(case, dt: Optional[float] = None):
    """sclet_params of an oracle case (cases.Case), with dt replaced."""
    import cases
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        p = sg.read_case(td, case.suffix)
    if dt is not None:
        p.dt = dt
    return p


def block_fields(case) -> np.ndarray:
    n = case.n
    out = np.zeros((case.nac + case.nch, n, n, n))
    for f, (_, _, vals) in enumerate(case.initial_fields()):
        out[f, 2:-2, 2:-2, 2:-2] = vals
    return out


def make_pairs(make_case, seeds: Iterable[int], sample_steps: Sequence[int], ratio: int, fine_precision=sg.FP64,
               device: int = 0):
    """Training pairs from the solver.  make_case(seed) gives the run
    (cases.Case with the fine dt); the fine solver advances from the seeded
    state, and at each fine step count of sample_steps one pair is taken.
    Returns torch CUDA tensors X [P][8][N,N,N], Y [P][4][N,N,N] (float32)."""
    import torch
    xs: List[np.ndarray] = []
    ys: List[np.ndarray] = []
    fine = coarse = None
    for seed in seeds:
        case = make_case(seed)
        pf = case_params(case)
        pc = case_params(case, dt=case.dt * ratio)
        if fine is None:
            fine = sg.Solver(pf, fine_precision, device=device)
            coarse = sg.Solver(pc, sg.MIXED, device=device)
        fine.set_fields(block_fields(case))
        t = 0
        for ts in sorted(sample_steps):
            if ts > t:
                fine.step(ts - t)
                t = ts
            u = fine.get_fields()
            coarse.set_fields(u)
            coarse.step(1)
            uc = coarse.get_fields()
            fine.step(ratio)
            t += ratio
            uf = fine.get_fields()
            x, y, _ = pair(owned(u), owned(uc), owned(uf))
            xs.append(x)
            ys.append(y)
    fine.close()
    coarse.close()
    X = torch.from_numpy(np.stack(xs)).to(f"cuda:{device}")
    Y = torch.from_numpy(np.stack(ys)).to(f"cuda:{device}")
    return X, Y


def train(net: Net, X, Y, iters: int, batch: int, lr: float, seed: int = 0, lr_final: Optional[float] = None):
    """Adam on random mini-batches of the pairs; cosine decay of the rate to
    lr_final.  Returns the loss of every iteration."""
    import math

    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    P = X.shape[0]
    lr_final = lr * 0.05 if lr_final is None else lr_final
    losses = []
    torch.cuda.synchronize()
    for it in range(iters):
        idx = torch.randperm(P, generator=g)[:batch].to(X.device)
        xb = X.index_select(0, idx).contiguous()
        yb = Y.index_select(0, idx).contiguous()
        torch.cuda.synchronize()
        rate = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / max(iters - 1, 1)))
        losses.append(net.train_step(xb, yb, rate))
    return np.array(losses)


def relative_errors(net: Optional[Net], X, Y) -> np.ndarray:
    """Per pair: ||coarse + correction - fine|| / ||fine - coarse|| over all
    fields (net None: the coarse step alone, which gives 1; the pair's scale
    cancels)."""
    import torch
    out = []
    for i in range(X.shape[0]):
        y = Y[i:i + 1]
        if net is None:
            out.append(1.0)
            continue
        pred = torch.empty_like(y)
        net.forward(X[i:i + 1].contiguous(), pred)
        out.append(float(torch.linalg.vector_norm(pred - y) / torch.linalg.vector_norm(y)))
    return np.array(out)


def aggregate_error(net: Optional[Net], X, Y, S) -> float:
    """Over all pairs, in the fields' own units (each pair's error times its
    scale S[i]): sqrt(sum |s (correction - y)|^2 / sum |s y|^2), i.e. the
    error left by the corrected coarse step relative to that of the coarse
    step alone (1 without a corrector)."""
    import torch
    num = den = 0.0
    for i in range(X.shape[0]):
        y = Y[i:i + 1]
        e = y if net is None else None
        if net is not None:
            pred = torch.empty_like(y)
            net.forward(X[i:i + 1].contiguous(), pred)
            e = pred - y
        num += float(S[i]) ** 2 * float(torch.sum(e * e))
        den += float(S[i]) ** 2 * float(torch.sum(y * y))
    return (num / den) ** 0.5 if den > 0 else 0.0


def learned_steps(coarse: "sg.Solver", fine: "sg.Solver", net: Optional[Net], ratio: int, nsteps: int,
                  check_every: int = 50, deviation_bound: float = 1e-2, energy_tol: float = 1e-9) -> dict:
    """nsteps coarse steps judged by the plain-ETD checks (sclet_learned_step)."""
    st = sg.LearnedStats()
    rc = sg.lib().sclet_learned_step(coarse.h, fine.h, net.h if net is not None else None, ratio, nsteps,
                                     check_every, deviation_bound, energy_tol, ctypes.byref(st))
    coarse._ck(rc, "learned_step")
    return st.as_dict()
