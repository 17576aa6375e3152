"""Inputs of the two deformers that solve through the block ILU-PCG path
(the ARAP deformer of defarap.cpp and the linear Laplacian deformer of
deflap.cpp), shared by tests/golden/make_golden.py and the GPU tests: a
closed-side cylinder of triangles (24 points around, 16 rings), its bottom
ring fixed and its top ring lifted and twisted, as the deformer examples
drag handles of a surface mesh."""
import numpy as np

NTH, NZ, RADIUS, HEIGHT = 24, 16, 0.5, 1.5


def cylinder():
    """Points (NTH * NZ, ring-major) and triangles of the cylinder's side."""
    th = 2.0 * np.pi * np.arange(NTH) / NTH
    z = HEIGHT * np.arange(NZ) / (NZ - 1)
    xyz = np.stack([np.tile(RADIUS * np.cos(th), NZ), np.tile(RADIUS * np.sin(th), NZ), np.repeat(z, NTH)], -1)
    tri = []
    for k in range(NZ - 1):
        for i in range(NTH):
            a, b = k * NTH + i, k * NTH + (i + 1) % NTH
            c, d = a + NTH, b + NTH
            tri += [(a, b, d), (a, d, c)]
    return xyz.ravel().astype(np.float64), np.array(tri, np.uint32).ravel()


def handles(xyz, lift=0.3, twist=0.4):
    """Fixed DOFs (bottom and top rings) and the deformed starting positions:
    the top ring lifted by `lift` and turned by `twist` radians about z."""
    p = xyz.reshape(-1, 3)
    np_ = p.shape[0]
    bottom = np.arange(NTH)
    top = np.arange((NZ - 1) * NTH, NZ * NTH)
    bc = np.zeros(np_ * 3, np.int32)
    for r in (bottom, top):
        bc[(3 * r[:, None] + np.arange(3)).ravel()] = 1
    q = p.copy()
    c, s = np.cos(twist), np.sin(twist)
    q[top, 0], q[top, 1] = c * p[top, 0] - s * p[top, 1], s * p[top, 0] + c * p[top, 1]
    q[top, 2] += lift
    return bc, q.ravel()


def extend_pattern(ind, psup, np_):
    """The 1-ring pattern extended to the 2-ring (neighbours of neighbours,
    self excluded), rows sorted: the matrix pattern both deformers build."""
    rows = []
    for i in range(np_):
        s = set()
        for j in psup[ind[i]:ind[i + 1]]:
            s.add(int(j))
            s.update(int(k) for k in psup[ind[j]:ind[j + 1]])
        s.discard(i)
        rows.append(sorted(s))
    out_ind = np.zeros(np_ + 1, np.uint32)
    out_ind[1:] = np.cumsum([len(r) for r in rows])
    return out_ind, np.array([j for r in rows for j in r], np.uint32)
