"""Finite-difference check of the adjoint gradients on the 48^3 voxel block.

  python -m delfem2_gb300.check_adjoint [--n 48] [--tets 64] [--dofs 64] [--h 1e-6]

Problem: per-tet E log-uniform in [0.5, 2] (seed 4), target u* = the solve at
a second E field (seed 40), load f ~ N(0, 1e-3^2) per DOF (seed 41),
L = 1/2 |u - u*|^2. Gradients dL/dE (per tet) and dL/df by the adjoint
(FP32+FP64-refinement solves) and by the FP64 adjoint, against FP64 central
finite differences with step h on random tets / DOFs. Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time


def setup(n: int, device="cuda"):
    import torch
    import delfem2_gb300 as D
    from .problem import young_log_uniform
    a = D.voxel_problem_arrays(n, n, n, 1.0 / n, seed=4, e_range=(0.5, 2.0))
    P = D.StaticElasticProblem(a)
    E = torch.from_numpy(a["young"]).to(device)
    E_target = torch.from_numpy(young_log_uniform(a["ntet"], 0.5, 2.0, 40)).to(device)
    g = torch.Generator(device="cpu").manual_seed(41)
    f = (torch.randn(a["np"] * 3, generator=g, dtype=torch.float64) * 1e-3).to(device)
    return a, P, E, E_target, f


def loss_and_grads(P, E, f, u_star, precision, tol=1e-10):
    import torch
    from .autograd import linear_elastic_solve
    Er = E.clone().requires_grad_(True)
    fr = f.clone().requires_grad_(True)
    u = linear_elastic_solve(Er, fr, P, precision, tol)
    L = 0.5 * torch.sum((u - u_star) ** 2)
    L.backward()
    return float(L.detach()), Er.grad.detach(), fr.grad.detach()


def fd_loss(P, E, f, u_star, tol=1e-14):
    import torch
    from .autograd import linear_elastic_solve
    with torch.no_grad():
        u = linear_elastic_solve(E, f, P, "fp64", tol)
        return float(0.5 * torch.sum((u - u_star) ** 2))


def fd_loss_change(P, E, f, u0, u_star, tol=1e-12):
    """L(E, f) - L(E0, f0) for the solve u = K(E)^-1 P f, in residual form.

    u = u0 + d with K(E) d = P f - K(E) u0 (FP64 SpMV and FP64 Solve_PCG), so
    L - L0 = d.(u0 - u*) + |d|^2 / 2 without subtracting two O(1) losses."""
    import torch
    from .ls import Solve_PCG
    with torch.no_grad():
        P.assemble_stiffness(E.contiguous())
        P.factor()
        r = (f * P.free_mask(f)).contiguous()
        P.K.MatVec(r, -1.0, u0.contiguous(), 1.0)
        d = torch.zeros_like(r)
        Solve_PCG(r.clone(), d, tol, 100000, P.K, P.ilu)
        return float(torch.dot(d, u0 - u_star) + 0.5 * torch.dot(d, d))


def fd_rows(P, E, f, u0, u_star, tets, dofs, h, gE, gf, gE_mixed, gf_mixed):
    """Central differences of L on the sampled tets and DOFs, next to the
    FP64 and mixed adjoint gradients: two lists of (fd, g_fp64, g_mixed)."""
    rowsE, rowsf = [], []
    for e in tets:
        Ep, Em = E.clone(), E.clone()
        Ep[e] += h
        Em[e] -= h
        fd = (fd_loss_change(P, Ep, f, u0, u_star) - fd_loss_change(P, Em, f, u0, u_star)) / (2 * h)
        rowsE.append((fd, float(gE[e]), float(gE_mixed[e])))
    for i in dofs:
        fp, fm = f.clone(), f.clone()
        fp[i] += h
        fm[i] -= h
        fd = (fd_loss_change(P, E, fp, u0, u_star) - fd_loss_change(P, E, fm, u0, u_star)) / (2 * h)
        rowsf.append((fd, float(gf[i]), float(gf_mixed[i])))
    return rowsE, rowsf


def fd_errors(rows, scale):
    """(vector, entry) relative errors of the FP64 and mixed adjoints against
    the differences: vector = max|g - fd| / max|g| (scale) over the samples;
    entry = max|g - fd| / |fd| over the samples with |fd| >= 1e-2 scale
    (smaller entries sit at the FP64 solves' accuracy floor). Also returns
    the number of such significant samples."""
    import numpy as np
    r = np.array(rows)
    sig = np.abs(r[:, 0]) >= 1e-2 * scale
    out = {}
    for col, tag in ((1, "fp64"), (2, "mixed")):
        out[tag] = (float(np.abs(r[:, col] - r[:, 0]).max() / scale),
                    float((np.abs(r[sig, col] - r[sig, 0]) / np.abs(r[sig, 0])).max()) if sig.any() else 0.0)
    return out, int(sig.sum())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--tets", type=int, default=64)
    ap.add_argument("--dofs", type=int, default=64)
    ap.add_argument("--h", type=float, default=1e-6)
    ap.add_argument("--tol", type=float, default=1e-10, help="tolerance of the mixed-precision solves")
    args = ap.parse_args()
    import numpy as np
    import torch
    from .autograd import linear_elastic_solve

    a, P, E, E_t, f = setup(args.n)
    with torch.no_grad():
        u_star = linear_elastic_solve(E_t, f, P, "fp64", 1e-14)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L, gE_mixed, gf_mixed = loss_and_grads(P, E, f, u_star, "mixed", args.tol)
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t0
    L64, gE, gf = loss_and_grads(P, E, f, u_star, "fp64", 1e-14)
    with torch.no_grad():
        u0 = linear_elastic_solve(E, f, P, "fp64", 1e-14)
    rng = np.random.default_rng(7)
    tets = rng.choice(a["ntet"], size=args.tets, replace=False)
    free = np.nonzero(a["bc"] == 0)[0]
    dofs = rng.choice(free, size=args.dofs, replace=False)
    h = args.h
    rowsE, rowsf = fd_rows(P, E, f, u0, u_star, tets, dofs, h, gE, gf, gE_mixed, gf_mixed)
    out = {"n": args.n, "dof": a["np"] * 3, "tets": a["ntet"], "L": L, "L_fp64": L64, "h": h,
           "n_tet_samples": len(tets), "n_dof_samples": len(dofs),
           "mixed_vs_fp64_adjoint_dLdE_max_rel": float((gE_mixed - gE).abs().max() / gE.abs().max()),
           "mixed_forward_plus_backward_s": t_mixed, "mixed_tol": args.tol,
           "fd": "central differences of L with u(E+-h) = u0 + d, K(E+-h) d = P f - K(E+-h) u0 (FP64)",
           "errors": ("vector: max|g - fd| / max|g| over the samples; entry: max |g - fd| / |fd| over samples "
                      "with |fd| >= 1e-2 max|g| (smaller entries sit at the FP64 solves' accuracy floor)")}
    for name, rows, scale in (("dLdE", rowsE, float(gE.abs().max())), ("dLdf", rowsf, float(gf.abs().max()))):
        errs, nsig = fd_errors(rows, scale)
        for tag, (vec, ent) in errs.items():
            out[f"{name}_{tag}_vs_fd_vector_rel"] = vec
            out[f"{name}_{tag}_vs_fd_entry_rel"] = ent
        out[f"{name}_significant_samples"] = nsig
    print(json.dumps(out))


if __name__ == "__main__":
    main()
