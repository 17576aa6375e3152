"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs oracle/_ref/libdfm2ref.so (the unmodified DelFEM2 headers compiled by
oracle/Makefile), so it only works where the reference source tree exists.
The outputs are small .npz files committed next to this script; the tests
read them on machines without the reference.

  python tests/golden/make_golden.py [tiny cfg1 cfg1e cfg2 cfg3 cfg4 cloth iluk bicgstab nd dynamic deform]
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build, reference  # noqa: E402

NU, RHO, G = 0.3, 1.0, np.array([0.0, 0.0, -1e-3])


def young_log_uniform(ntet, lo, hi, seed):
    # identical to delfem2_gb300.problem.young_log_uniform (kept separate so that
    # this script does not load the CUDA library)
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), ntet))


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def system(R, nx, ny, nz, h, young):
    xyz, tet = R.voxel_tet_mesh(nx, ny, nz, h)
    np_ = xyz.size // 3
    ind, psup = R.psup(tet, 4, np_)
    vc = np.zeros(psup.size * 9)
    vd = np.zeros(np_ * 9)
    b = np.zeros(np_ * 3)
    if np.isscalar(young):
        young = np.full(tet.size // 4, float(young))
    assert R.assemble_tet_linear(ind, psup, vc, vd, b, xyz, tet, young, NU, RHO, G) == 0
    bc = np.zeros(np_ * 3, np.int32)
    bc[np.repeat(xyz[2::3] == 0.0, 3)] = 1
    R.set_fixed_bc(ind, psup, vc, vd, bc)
    R.rhs_zero(b, bc)
    col, dia = R.ilu_pattern0(ind, psup)
    ivc, ivd = R.ilu_copy_value(ind, col, psup, vc, vd)
    st, _ = R.ilu_decompose(ind, col, dia, ivc, ivd)
    assert st == 0
    return dict(xyz=xyz, tet=tet, ind=ind, psup=psup, vc=vc, vd=vd, b=b, bc=bc, col=col, dia=dia, ivc=ivc,
                ivd=ivd, young=young)


def solve(R, s, tol, maxit=100000):
    t = time.time()
    x, r, hist = R.solve_pcg(s["ind"], s["psup"], s["vc"], s["vd"], s["col"], s["dia"], s["ivc"], s["ivd"],
                             s["b"], tol, maxit)
    return x, hist, time.time() - t


def sample_idx(n, k=2000, seed=123):
    return np.sort(np.random.default_rng(seed).choice(n, size=min(k, n), replace=False)).astype(np.int64)


def make_tiny(R):
    s = system(R, 3, 2, 2, 1.0 / 3, young_log_uniform(3 * 2 * 2 * 6, 0.1, 10.0, 7))
    x, hist, _ = solve(R, s, 1e-10)
    vec = np.random.default_rng(11).standard_normal(s["b"].size)
    fwd = R.ilu_forward(s["ind"], s["col"], s["dia"], s["ivc"], s["ivd"], vec)
    both = R.ilu_backward(s["ind"], s["col"], s["dia"], s["ivc"], fwd)
    mv = R.matvec(s["ind"], s["psup"], s["vc"], s["vd"], np.zeros_like(vec), 1.0, vec, 0.0)
    np.savez_compressed(os.path.join(HERE, "tiny.npz"), x=x, hist=np.array(hist), vec=vec, fwd=fwd,
                        precond=both, matvec=mv, **{k: v for k, v in s.items()})


def make_cfg(R, name, nx, ny, nz, h, young, tol, full_x):
    s = system(R, nx, ny, nz, h, young)
    x, hist, dt = solve(R, s, tol)
    idx = sample_idx(x.size)
    out = dict(nx=nx, ny=ny, nz=nz, h=h, tol=tol, n_iter=len(hist) - 1, hist=np.array(hist),
               pattern_sha=sha(s["ind"], s["psup"]), dia_sha=sha(s["dia"]),
               young_sha=sha(s["young"]), b=s["b"] if full_x else s["b"][idx],
               x_norm=np.linalg.norm(x), x_sum=x.sum(), b_norm=np.linalg.norm(s["b"]),
               K_abs_sum=np.abs(s["vc"]).sum() + np.abs(s["vd"]).sum(), idx=idx, x_sample=x[idx],
               ilu_dia_sample=s["ivd"][idx % s["ivd"].size], seconds=dt)
    if full_x:
        out["x"] = x
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: ndof={x.size} iterations={len(hist) - 1} final={hist[-1]:.3e} "
          f"rel={hist[-1] / hist[0]:.3e} time={dt:.1f}s")


def make_cloth(R):
    """Cloth element functions on seeded inputs and short backward-Euler runs on
    a 16x16-cell sheet (289 vertices): StepTime_InternalDynamicsILU itself
    (uniform E = 1e3, its own 1e-4 / 100) and the same step with per-triangle
    E and PCG to 1e-8 (the cloth workload's settings)."""
    from oracle import cloth as CL
    rng = np.random.default_rng(55)
    out = {}
    Cc = rng.standard_normal((32, 3, 3))
    cc = Cc + 0.3 * rng.standard_normal((32, 3, 3))
    lm = rng.uniform(0.2, 2.0, (32, 2))
    res = [CL.wdwddw_cst(R, Cc[i], cc[i], lm[i, 0], lm[i, 1]) for i in range(32)]
    out.update(cst_C=Cc, cst_c=cc, cst_lm=lm, cst_W=np.array([r[0] for r in res]),
               cst_dW=np.array([r[1] for r in res]), cst_ddW=np.array([r[2] for r in res]))
    Cq = rng.standard_normal((32, 4, 3))
    cq = Cq + 0.2 * rng.standard_normal((32, 4, 3))
    res = [CL.wdwddw_bend(R, Cq[i], cq[i], 1e-3) for i in range(32)]
    out.update(bend_C=Cq, bend_c=cq, bend_W=np.array([r[0] for r in res]),
               bend_dW=np.array([r[1] for r in res]), bend_ddW=np.array([r[2] for r in res]))
    s2 = rng.standard_normal((64, 3))
    out.update(pd_s2=s2, pd_s3=np.array([CL.make_pd_sim22(R, v) for v in s2]))
    ndiv = 16
    xyz0, tri, quad = CL.cloth_square(R, ndiv)
    np_ = xyz0.size // 3
    ind, psup = R.psup(quad, 4, np_)
    bc = np.zeros(np_ * 3, np.int32)
    bc[0:3] = 1
    bc[ndiv * 3:ndiv * 3 + 3] = 1
    g = np.array([0.0, 0.0, -10.0])
    mass = 1.0 / np_
    young_rand = young_log_uniform(tri.size // 3, 5e2, 2e3, 56)
    out.update(xyz0=xyz0, tri=tri, quad=quad, ind=ind, psup=psup, bc=bc, young_rand=young_rand)
    xyz = xyz0 + 0.01 * rng.standard_normal(xyz0.size)
    W, vc, vd, dW = CL.cloth_assemble(R, ind, psup, xyz0, xyz, tri, quad, young_rand, 0.3, 1e-3)
    out.update(asm_xyz=xyz, asm_W=W, asm_vc=vc, asm_vd=vd, asm_dW=dW)
    for tag, young, tol, mi, nstep in (("own", np.full(tri.size // 3, 1e3), 1e-4, 100, 10),
                                       ("rand", young_rand, 1e-8, 1000, 10)):
        x, v = xyz0.copy(), np.zeros_like(xyz0)
        traj, nh = [], []
        for _ in range(nstep):
            x, v, n = CL.cloth_step(R, ind, psup, x, v, xyz0, bc, tri, quad, young, 0.3, 1e-3, g, mass, 0.01, tol,
                                    mi)
            traj.append(x.copy())
            nh.append(n)
        out[f"step_{tag}_x"] = np.array(traj)
        out[f"step_{tag}_v"] = v
        out[f"step_{tag}_nhist"] = np.array(nh)
    np.savez_compressed(os.path.join(HERE, "cloth.npz"), **out)
    print("cloth: rand-E iterations per step", out["step_rand_nhist"] - 1)


def make_iluk(R):
    """Initialize_ILUk patterns (k = 1, 2, 3 and full fill), the ILU(k) factors
    and Solve_PCG with them on an 8^3 voxel block (per-tet E log-uniform
    [0.1, 10], seed 9), from the reference."""
    s = system(R, 8, 8, 8, 1.0 / 8, young_log_uniform(8 ** 3 * 6, 0.1, 10.0, 9))
    out = {"young_seed": 9, "n": 8}
    for k in (1, 2, 3, -1):
        rs, col, dia = R.ilu_pattern_k(s["ind"], s["psup"], k)
        ivc, ivd = R.ilu_copy_value_k(s["ind"], s["psup"], s["vc"], s["vd"], k, rs, col)
        st, _ = R.ilu_decompose(rs, col, dia, ivc, ivd)
        assert st == 0
        x, _, hist = R.solve_pcg_k(s["ind"], s["psup"], s["vc"], s["vd"], rs, col, dia, ivc, ivd, s["b"], 1e-10, 1000)
        tag = "full" if k == -1 else str(k)
        si = sample_idx(ivc.size, 3000, seed=10 + k)
        out.update({f"k{tag}_rs": rs, f"k{tag}_col": col, f"k{tag}_dia": dia, f"k{tag}_ivc_idx": si,
                    f"k{tag}_ivc_sample": ivc[si], f"k{tag}_ivc_abs_sum": np.abs(ivc).sum(),
                    f"k{tag}_ivd_abs_sum": np.abs(ivd).sum(), f"k{tag}_x": x.astype(np.float64),
                    f"k{tag}_hist": np.array(hist)})
        print(f"iluk: k={k} nnz={col.size} iterations={len(hist) - 1}")
    np.savez_compressed(os.path.join(HERE, "iluk.npz"), **out)


def nonsymmetric(s, seed=11):
    """K with each off-diagonal block scaled by a seeded factor in [0.7, 1.3]
    (so block (i,j) is no longer block (j,i)^T), clamped again."""
    rng = np.random.default_rng(seed)
    vc = s["vc"] * (1.0 + 0.3 * rng.uniform(-1.0, 1.0, s["vc"].size // 9).repeat(9))
    return vc, s["vd"].copy()


def make_bicgstab(R):
    """The reference's Solve_PBiCGStab with ILU(0) and ILU(1) on a non-symmetric
    version of the 8^3 block (E seed 5), tol 1e-10 and 1e-6. The system is
    assembled and factorised by the C restatement (pinned to the reference by
    the other fixtures): BiCGStab amplifies 1e-16 differences in K or the
    factors into different iteration counts, so the solver is pinned on
    identical inputs."""
    from oracle import port
    P = port()
    s = system(P, 8, 8, 8, 1.0 / 8, young_log_uniform(8 ** 3 * 6, 0.1, 10.0, 5))
    vc, vd = nonsymmetric(s)
    P.set_fixed_bc(s["ind"], s["psup"], vc, vd, s["bc"])
    out = {}
    for k in (0, 1):
        rs, col, dia = P.ilu_pattern_k(s["ind"], s["psup"], k)
        ivc, ivd = P.ilu_copy_value_k(s["ind"], s["psup"], vc, vd, k, rs, col)
        assert P.ilu_decompose(rs, col, dia, ivc, ivd)[0] == 0
        for tol in (1e-10, 1e-6):
            x, r, hist = R.solve_pbicgstab(s["ind"], s["psup"], vc, vd, rs, col, dia, ivc, ivd, s["b"], tol, 1000)
            tag = f"k{k}_t{int(-np.log10(tol))}"
            out.update({f"{tag}_x": x, f"{tag}_r": r, f"{tag}_hist": np.array(hist)})
            print(f"bicgstab: ILU({k}) tol {tol}: {len(hist)} iterations, last {hist[-1]:.3e}")
    np.savez_compressed(os.path.join(HERE, "bicgstab.npz"), **out)


def make_nd(R):
    """Scalar (ndim 1) and 2x2 (ndim 2) systems of tests/nd_systems.py, all from
    the reference: assembly (MergeLinSys_Poission_MeshTet3D,
    MergeLinSys_Poission_MeshTri2D, MergeLinSys_SolidLinear_Static_MeshTri2D),
    SetFixedBC, MatVec of a seeded vector, ILU(0) / ILU(1) factors, one forward
    and backward sweep, Solve_PCG and Solve_PBiCGStab to 1e-10; plus a Merge of
    an element that repeats a node, for ndim 1, 2 and 3."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import nd_systems as S
    out = {}
    for name, make in S.SYSTEMS.items():
        s = make(R)
        nd, n = s["ndim"], s["b"].size
        out.update({f"{name}_{k}": s[k] for k in ("ind", "psup", "vc", "vd", "b", "bc", "elem")})
        rng = np.random.default_rng(7)
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        out[f"{name}_mv_x"], out[f"{name}_mv_y"] = x, y
        out[f"{name}_mv"] = R.nd_matvec(nd, s["ind"], s["psup"], s["vc"], s["vd"], y, 1.5, x, 0.5)
        for k in (0, 1):
            rs, col, dia, ivc, ivd = S.factor(R, s, k)
            t = f"{name}_k{k}"
            out.update({f"{t}_rs": rs, f"{t}_col": col, f"{t}_dia": dia, f"{t}_vc": ivc, f"{t}_vd": ivd})
            out[f"{t}_fwd"] = R.nd_ilu_forward(nd, rs, col, dia, ivc, ivd, x)
            out[f"{t}_bwd"] = R.nd_ilu_backward(nd, rs, col, dia, ivc, x)
            for solver in ("pcg", "pbicgstab"):
                f = R.nd_solve_pcg if solver == "pcg" else R.nd_solve_pbicgstab
                xs, _, hist = f(nd, s["ind"], s["psup"], s["vc"], s["vd"], rs, col, dia, ivc, ivd, s["b"], 1e-10, 1000)
                out[f"{t}_{solver}_x"], out[f"{t}_{solver}_hist"] = xs, np.array(hist)
                print(f"nd {name} ILU({k}) {solver}: {len(hist)} entries, last {hist[-1]:.3e}")
    # Merge of one element whose nodes 0 and 2 coincide (diagonal rule of the reference)
    for nd in (1, 2, 3):
        ind = np.array([0, 2, 4, 6], np.uint32)
        psup = np.array([1, 2, 0, 2, 0, 1], np.uint32)
        rng = np.random.default_rng(20 + nd)
        vc = rng.standard_normal(6 * nd * nd)
        vd = rng.standard_normal(3 * nd * nd)
        nodes = np.array([0, 1, 0, 2], np.uint32)
        emat = rng.standard_normal(16 * nd * nd)
        out[f"merge{nd}_vc0"], out[f"merge{nd}_vd0"], out[f"merge{nd}_emat"] = vc.copy(), vd.copy(), emat
        st = R.nd_merge(nd, ind, psup, vc, vd, nodes, emat) if nd < 3 else R.merge(ind, psup, vc, vd, nodes, emat)
        assert st == 0
        out[f"merge{nd}_vc"], out[f"merge{nd}_vd"] = vc, vd
    np.savez_compressed(os.path.join(HERE, "nd.npz"), **out)


def make_dynamic(R):
    """The reference's MergeLinSys_SolidLinear_BEuler_MeshTet3D,
    MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D and
    MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D, and the Q1 hex element loop,
    on the inputs of tests/dyn_systems.py (K values and b)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import dyn_systems as DS
    s = DS.inputs(R)
    out = {}
    for kind in DS.KINDS:
        vc, vd, b = DS.assemble(R, s, kind)
        out.update({f"{kind}_vc": vc, f"{kind}_vd": vd, f"{kind}_b": b})
    vc, vd, b = DS.assemble_hex(R, DS.hex_inputs(R))  # the element loop of MergeLinSys_LinearSolid3D_Static_Q1
    out.update({"hexq1_vc": vc, "hexq1_vd": vd, "hexq1_b": b})
    np.savez_compressed(os.path.join(HERE, "dynamic.npz"), **out)


def make_deform(R):
    """The ARAP deformer (Deformer_Arap: per-point elements, ILU(0)-PCG to 1e-7) and the linear Laplacian deformer
    (CDef_LaplacianLinear: dual-Laplacian elements, ILU(20)-PCG to 1e-5) on the cylinder of tests/deform_systems.py,
    each run once by the reference: the element matrices they hand to Merge, the ILU(20) pattern, the results."""
    sys.path.insert(0, os.path.dirname(HERE))
    from deform_systems import cylinder, handles
    xyz0, tri = cylinder()
    bc, xdef = handles(xyz0)
    np_ = xyz0.size // 3
    quat = np.tile(np.array([0.0, 0.0, 0.0, 1.0]), np_)  # identity rotations (x, y, z, w)
    ptr, idx, eM, eR = R.arap_elements(xyz0, tri, xdef, quat)
    x_arap, h_arap = R.arap_deform(xyz0, tri, xdef, quat, bc)
    lap = R.lap_deform(xyz0, tri, bc, xdef)
    out = dict(xyz0=xyz0, tri=tri, bc=bc, xdef=xdef, quat=quat, arap_ptr=ptr, arap_idx=idx, arap_eM=eM, arap_eR=eR,
               arap_x=x_arap, arap_hist=h_arap)
    out.update({"lap_" + k: v for k, v in lap.items()})
    np.savez_compressed(os.path.join(HERE, "deform.npz"), **out)
    print(f"deform: {np_} points, ARAP {len(h_arap) - 1} iterations, Laplacian {len(lap['hist']) - 1} iterations, "
          f"ILU(20) {lap['ilu_col'].size} blocks (matrix {lap['pat_col'].size})")


def main(which):
    build(quiet=True)
    R = reference()
    if "tiny" in which:
        make_tiny(R)
    if "cfg1" in which:  # unit cube 16^3, E = 1
        make_cfg(R, "cfg1", 16, 16, 16, 1 / 16, 1.0, 1e-10, True)
    if "cfg1e" in which:  # 16^3, E log-uniform [0.1, 10], seed 0
        make_cfg(R, "cfg1e", 16, 16, 16, 1 / 16, young_log_uniform(16 ** 3 * 6, 0.1, 10.0, 0), 1e-10, True)
    if "cfg2" in which:  # 64^3, E log-uniform [0.1, 10], seed 2, oracle to 1e-12
        make_cfg(R, "cfg2", 64, 64, 64, 1 / 64, young_log_uniform(64 ** 3 * 6, 0.1, 10.0, 2), 1e-12, False)
    if "cfg3" in which:  # 128x128x64, spacing 1/128, E log-uniform [0.1, 10], seed 3, to 1e-12
        make_cfg(R, "cfg3", 128, 128, 64, 1 / 128, young_log_uniform(128 * 128 * 64 * 6, 0.1, 10.0, 3), 1e-12,
                 False)
    if "cfg4" in which:  # 48^3, E log-uniform [0.5, 2], seed 4, to 1e-12
        make_cfg(R, "cfg4", 48, 48, 48, 1 / 48, young_log_uniform(48 ** 3 * 6, 0.5, 2.0, 4), 1e-12, False)
    if "cloth" in which:
        make_cloth(R)
    if "iluk" in which:
        make_iluk(R)
    if "bicgstab" in which:
        make_bicgstab(R)
    if "nd" in which:
        make_nd(R)
    if "dynamic" in which:
        make_dynamic(R)
    if "deform" in which:
        make_deform(R)


if __name__ == "__main__":
    main(sys.argv[1:] or ["tiny", "cfg1", "cfg1e", "cfg2"])
