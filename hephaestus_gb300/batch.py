"""Batches of uneven frequency-domain (eddy-current) solves on one GPU.

Each problem is curl(nu curl A) + i omega sigma A = J on a cube hex mesh with
its own size, Nedelec order, frequency and per-element sigma/nu fields, the
operator of ComplexMaxwellOperator::Solve
(src/formulations/ComplexMaxwell/complex_maxwell_formulation.cpp:171-222) with
permittivity 0.  Every problem keeps its mesh factors, preconditioner
hierarchy and Krylov vectors on the device, owns a CUDA stream, and is solved
by a graph-driven COCG (hc_solve_complex_graph); hc_solve_complex_batch
enqueues all graphs before collecting any, so the solves overlap on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import meshes
from .operator import GpuComplexCOCGSolver, HCurlOperator, solve_complex_batch


@dataclass
class Problem:
    n: int
    p: int
    omega: float
    seed: int

    @property
    def ndof(self):
        a = self.n * self.p
        return 3 * a * (a + 1) ** 2


def make_batch(count=64, seed=0, n_range=(8, 40), orders=(1, 2, 3), omega_range=(1e1, 1e5)):
    """Seeded problem list: n uniform in n_range, order uniform in orders,
    omega log-uniform in omega_range."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        p = int(rng.choice(orders))
        om = float(np.exp(rng.uniform(np.log(omega_range[0]), np.log(omega_range[1]))))
        out.append(Problem(n, p, om, int(rng.integers(1 << 31))))
    return out


class DeviceBatch:
    """Resident operators, right-hand sides and solutions of a problem list.
    autotune: time the launch configurations of each order-1/2 problem's FP32
    complex apply once (hc_autotune) before anything is solved."""

    def __init__(self, problems, params, autotune=False):
        import torch

        self.problems = problems
        self.ops, self.solvers, self.rhs, self.sols, self.streams = [], [], [], [], []
        self.tuning = []
        for pb in problems:
            rng = np.random.default_rng(pb.seed)
            ne = pb.n ** 3
            nu = meshes.loguniform(ne, 1.0, 1e3, rng)
            sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
            st = torch.cuda.Stream()
            op = HCurlOperator(pb.n, pb.n, pb.n, pb.p, nu, sigma, dt=1.0, ess_attr_bits=0x3F, stream=st)
            b = torch.zeros(op.ndof, dtype=torch.float64, device="cuda")
            op.LoadCoilDevice(b, I0=float(rng.uniform(0.5, 2.0)))
            b.mul_(torch.tensor(op.ess_mask() == 0, device="cuda"))
            if autotune and pb.p <= 2:
                self.tuning.append(dict(op.Autotune("complex"), n=pb.n, p=pb.p))
            self.ops.append(op)
            self.streams.append(st)
            self.solvers.append(GpuComplexCOCGSolver(dict(params), op, pb.omega))
            self.rhs.append((b, torch.zeros_like(b)))
            self.sols.append((torch.zeros_like(b), torch.zeros_like(b)))
        torch.cuda.synchronize()

    def set_params(self, params):
        for s in self.solvers:
            om = s.omega
            s.__init__(dict(params), s.op, om)

    def zero(self):
        for xr, xi in self.sols:
            xr.zero_()
            xi.zero_()

    def solve(self):
        """All solves at once; returns the per-problem result dicts."""
        return solve_complex_batch(self.solvers, self.rhs, self.sols)

    def solutions(self):
        return [(xr.clone(), xi.clone()) for xr, xi in self.sols]

    def close(self):
        for op in self.ops:
            op.close()
        self.ops = []
