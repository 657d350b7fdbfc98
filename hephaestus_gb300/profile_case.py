"""Small, self-contained operator-apply case for profiling (ncu) runs.

    python -m hephaestus_gb300.profile_case N P [mult|add|fp64|solve|complex|tets]

Builds an N^3-hex, order-P operator with nu = 10^U(0,3), sigma = 10^U(-2,6),
dt = 0.01 (the benchmark's coefficient distributions) and applies it:
  mult  - y = J x in FP32 (masked init + apply), 5 times
  add   - y += P K P x in FP32 (the accumulate-form apply kernel alone), 5 times
  fp64  - y = J x in FP64, 3 times
  solve - one mixed-precision PCG solve (auxiliary-space preconditioner) of
          the coil load, capped at 8 inner iterations and 1 refinement step
  complex - y = (C + i omega M) x in FP32 (fused complex kernel), 5 times
  tets  - Kuhn N^3 tet mesh (jitter 0.15 h), order P: 16-RHS FP32 apply, 3 times
  tetsolve - the same tet mesh: one mixed-precision 16-RHS block solve of coil
          loads (auxiliary-space preconditioner), capped at 8 inner iterations
          and 1 refinement step
"""
import sys

import numpy as np


def main(argv):
    import torch

    from hephaestus_gb300 import HCurlOperator, meshes

    n = int(argv[0]) if argv else 96
    p = int(argv[1]) if len(argv) > 1 else 2
    mode = argv[2] if len(argv) > 2 else "mult"
    rng = np.random.default_rng(0)
    if mode in ("tets", "tetsolve"):
        v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.15, seed=0)
        ne = len(t)
        op = HCurlOperator.from_tets(v, t, p, meshes.loguniform(ne, 1, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng),
                                     dt=0.01, btris=bt, battr=ba, ess_attr_bits=0x3F)
        if mode == "tetsolve":
            from hephaestus_gb300 import GpuHCurlPCGSolver

            B = torch.empty(op.ndof, 16, dtype=torch.float64, device="cuda")
            col = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
            free = torch.tensor(op.ess_mask() == 0, device="cuda")
            for k in range(16):
                op.LoadCoilDevice(col, I0=0.5 + 0.1 * k, xc=0.45 + 0.01 * k, q=4)
                B[:, k] = col * free
            X = torch.zeros_like(B)
            s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 8, "MaxOuter": 1, "Precision": "mixed",
                                   "Preconditioner": "aux"}, op)
            s.MultMultiDevice(B, X)
            torch.cuda.synchronize()
            print("ok", mode, op.ndof, op.AuxLevels())
            return
        X = torch.randn(op.ndof, 16, device="cuda")
        Y = torch.empty_like(X)
        for _ in range(3):
            op.MultMultiDevice(X, Y)
        torch.cuda.synchronize()
        print("ok", mode, op.ndof)
        return
    nu = meshes.loguniform(n ** 3, 1, 1e3, rng)
    sg = meshes.loguniform(n ** 3, 1e-2, 1e6, rng)
    op = HCurlOperator(n, n, n, p, nu, sg, dt=0.01)
    if mode == "solve":
        from hephaestus_gb300 import GpuHCurlPCGSolver

        b = torch.tensor(np.where(op.ess_mask() != 0, 0.0, op.LoadCoil()), device="cuda")
        x = torch.zeros_like(b)
        s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 8, "MaxOuter": 1, "Precision": "mixed",
                               "Preconditioner": "aux"}, op)
        s.MultDevice(b, x)
    elif mode == "complex":
        xr = torch.randn(op.ndof, device="cuda")
        xi = torch.randn_like(xr)
        yr, yi = torch.empty_like(xr), torch.empty_like(xr)
        for _ in range(5):
            op.MultComplexDevice(1e3, xr, xi, yr, yi)
    elif mode == "fp64":
        x = torch.randn(op.ndof, device="cuda", dtype=torch.float64)
        y = torch.empty_like(x)
        for _ in range(3):
            op.MultDevice(x, y)
    else:
        x = torch.randn(op.ndof, device="cuda")
        y = torch.zeros_like(x)
        for _ in range(5):
            (op.AddMultDevice if mode == "add" else op.MultDevice)(x, y)
    torch.cuda.synchronize()
    print("ok", mode, op.ndof)


if __name__ == "__main__":
    main(sys.argv[1:])
