"""One static-elasticity solve on a voxel block, for profiler captures.

  python -m delfem2_gb300.profile_case [--nx 64 --ny 64 --nz 64] [--fp64] [--solves 1] [--method reliable]

Sets the problem up (mesh, pattern, level sets, assembly, ILU(0)) and runs
`--solves` solves of K u = b to 1e-10 (FP32-inner/FP64-refinement by default,
with reliable updates or restarted refinement; plain FP64 Solve_PCG with
--fp64), printing the device time of each.
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
    args = ap.parse_args()

    import torch
    import delfem2_gb300 as D
    from delfem2_gb300 import _native as N

    a = D.voxel_problem_arrays(args.nx, args.ny, args.nz, 1.0 / args.nx, seed=3)
    P = D.StaticElasticProblem(a)
    if args.levels:
        P.ilu.set_sweep_mode(N.SWEEP_LEVELS)
    b = P.assemble(b=torch.zeros(a["np"] * 3, dtype=torch.float64, device="cuda"))
    assert P.factor()
    torch.cuda.synchronize()
    for k in range(args.solves):
        t = time.perf_counter()
        if args.fp64:
            r, x = b.clone(), torch.zeros_like(b)
            hist = D.Solve_PCG(r, x, 1e-10, 20000, P.K, P.ilu)
            torch.cuda.synchronize()
            print(f"solve {k}: fp64 {len(hist) - 1} iterations, {1e3 * (time.perf_counter() - t):.1f} ms")
        else:
            x = torch.zeros_like(b)
            st = D.Solve_PCG_Mixed(b, x, 1e-10, P.K, P.ilu, method=args.method)
            torch.cuda.synchronize()
            print(f"solve {k}: mixed {st.iterations} inner / {st.outer} outer, rel {st.rel_residual:.2e}, "
                  f"{1e3 * (time.perf_counter() - t):.1f} ms")


if __name__ == "__main__":
    main()
