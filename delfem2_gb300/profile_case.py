"""One static-elasticity solve on a voxel block, for profiler captures.

  python -m delfem2_gb300.profile_case [--nx 64 --ny 64 --nz 64] [--fp64] [--solves 1] [--method reliable]
                                       [--poisson] [--sweep-mode M] [--precond K]
  python -m delfem2_gb300.profile_case --cloth NDIV [--solves K]

Sets the problem up (mesh, pattern, level sets, assembly, ILU(0)) and runs
`--solves` solves of K u = b to 1e-10 (FP32-inner/FP64-refinement by default,
with reliable updates or restarted refinement; plain FP64 Solve_PCG with
--fp64), printing the device time of each. --poisson solves the scalar
Poisson problem (1x1 blocks) on the same mesh instead: alpha = 1, source = 1,
the z = 0 face at 0 and the top face at 1. --sweep-mode selects the triangular-sweep
schedule (a dfm2g_sweep value); --precond K replaces the solves by K FP32
SolvePrecond calls (forward + backward sweep) on a seeded vector.
--cloth NDIV runs `--solves` backward-Euler steps of the implicit cloth
(StepTime_InternalDynamicsILU) on an NDIV x NDIV-cell sheet instead: E = 1e3,
nu = 0.3, bending 1e-3, two corners pinned, dt = 0.01, FP64 ILU(0)-PCG to 1e-8
capped at 100 iterations per step.
"""
from __future__ import annotations

import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=64)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--nz", type=int, default=64)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--levels", action="store_true", help="level-by-level sweep schedule")
    ap.add_argument("--method", choices=["reliable", "restart"], default="reliable")
    ap.add_argument("--poisson", action="store_true", help="scalar Poisson (1x1 blocks) on the same mesh")
    ap.add_argument("--sweep-mode", type=int, default=None, help="triangular-sweep schedule (dfm2g_sweep value)")
    ap.add_argument("--precond", type=int, default=0, help="K FP32 SolvePrecond calls instead of solves")
    ap.add_argument("--cloth", type=int, default=0, help="cloth sheet of NDIV x NDIV cells instead of the tets")
    args = ap.parse_args()

    import torch
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N

    if args.cloth:
        cloth_steps(args.cloth, args.solves)
        return

    a = D.voxel_problem_arrays(args.nx, args.ny, args.nz, 1.0 / args.nx, seed=3)
    if args.poisson:
        import numpy as np
        K = D.CMatrixSparse()
        K.Initialize(a["np"], 1, True)
        K.SetPattern(a["psup_ind"], a["psup"])
        ilu = D.CPreconditionerILU()
        ilu.SetPattern0(K)
        z = a["xyz"].reshape(-1, 3)[:, 2]
        top = z > z.max() - 1e-12
        bc = torch.tensor(((z < 1e-12) | top).astype(np.int32), device="cuda")
        b = torch.zeros(a["np"], dtype=torch.float64, device="cuda")
        D.TetMesh(K, a["xyz"], a["tet"]).assemble_poisson(1.0, 1.0, b, torch.tensor(np.where(top, 1.0, 0.0),
                                                                                     device="cuda"))
        K.SetFixedBC(bc)
        D.setRHS_Zero(b, bc)
        ilu.CopyValue(K)
        assert ilu.Decompose()
    else:
        P = D.StaticElasticProblem(a)
        K, ilu = P.K, P.ilu
        b = P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
        assert P.factor()
    if args.levels:
        ilu.set_sweep_mode(N.SWEEP_LEVELS)
    if args.sweep_mode is not None:
        ilu.set_sweep_mode(args.sweep_mode)
    torch.cuda.synchronize()
    if args.precond:
        gen = torch.Generator(device="cuda").manual_seed(0)
        v = torch.randn(b.numel(), dtype=torch.float32, device="cuda", generator=gen)
        for k in range(args.precond):
            u = v.clone()
            t = time.perf_counter()
            ilu.SolvePrecond(u)
            torch.cuda.synchronize()
            print(f"precond {k}: {1e3 * (time.perf_counter() - t):.3f} ms, |z| = {float(u.norm()):.6e}")
        return
    for k in range(args.solves):
        t = time.perf_counter()
        if args.fp64:
            r, x = b.clone(), torch.zeros_like(b)
            hist = D.Solve_PCG(r, x, 1e-10, 20000, K, ilu)
            torch.cuda.synchronize()
            print(f"solve {k}: fp64 {len(hist) - 1} iterations, {1e3 * (time.perf_counter() - t):.1f} ms")
        else:
            x = torch.zeros_like(b)
            st = D.Solve_PCG_Mixed(b, x, 1e-10, K, ilu, method=args.method)
            torch.cuda.synchronize()
            print(f"solve {k}: mixed {st.iterations} inner / {st.outer} outer, rel {st.rel_residual:.2e}, "
                  f"{1e3 * (time.perf_counter() - t):.1f} ms")


def cloth_steps(ndiv: int, nsteps: int):
    import torch
    from delfem2_gb300 import cloth as DC
    xyz0, _, tri, quad = DC.SetClothShape_Square(ndiv, 1.0)
    cl = DC.Cloth(xyz0, tri, quad)
    bc = torch.tensor(DC.pin_two_corners(ndiv), device="cuda")
    E = torch.full((cl.ntri,), 1e3, dtype=torch.float64, device="cuda")
    x = torch.tensor(xyz0, device="cuda")
    v = torch.zeros_like(x)
    for k in range(nsteps):
        t = time.perf_counter()
        st = cl.StepTime_InternalDynamicsILU(x, v, bc, E, 0.3, 1e-3, (0.0, 0.0, -10.0), 1.0 / cl.np, 0.01, 1e-8, 100)
        torch.cuda.synchronize()
        print(f"cloth step {k}: {st.iterations} PCG iterations, rel {st.rel_residual:.2e}, "
              f"{1e3 * (time.perf_counter() - t):.1f} ms")


if __name__ == "__main__":
    main()
