"""Why the cloth workload's PCG cannot converge at its configured size: the
natural-order ILU(0) of the first backward-Euler matrix of the square sheet
(M/dt^2 + K(x0); E = 1e3, nu = 0.3, bending 1e-3, dt = 0.01, mass 1/np per
vertex, two corners pinned) amplifies a vector by a factor that explodes
between 48 and 64 cells per side.

Growth |M^-1 r| / |r| for r seeded unit-normal (numpy PCG64, seed 0), with the
matrix assembled and factored by the reference's own compiled code
(oracle/_ref, where the reference tree is available) and by the C
restatement: below 1 at 48 cells, above 1e15 at 64 and above 1e100 at 255
(the 256 x 256-vertex workload), in both. CPU only."""
import numpy as np
import pytest

from oracle import HAVE_REFERENCE_BUILD
from oracle.cloth import step_matrix

E, NU, BEND, DT = 1e3, 0.3, 1e-3, 0.01


def _growth(O, ndiv):
    from delfem2_gb300.cloth import SetClothShape_Square, pin_two_corners
    from oracle import port
    xyz0, _, tri, quad = SetClothShape_Square(ndiv, 1.0)
    n = xyz0.size // 3
    ind, psup = port().psup(quad, 4, n)
    young = np.full(tri.size // 3, E)
    _, _, icol, dia, ivc, ivd = step_matrix(O, ind, psup, xyz0, xyz0.copy(), pin_two_corners(ndiv), tri, quad, young,
                                            NU, BEND, 1.0 / n, DT)
    r = np.random.default_rng(0).standard_normal(3 * n)
    z = O.ilu_backward(ind, icol, dia, ivc, O.ilu_forward(ind, icol, dia, ivc, ivd, r))
    return float(np.linalg.norm(z) / np.linalg.norm(r))


def _oracles():
    from oracle import port, reference
    out = [("restatement", port())]
    if HAVE_REFERENCE_BUILD():
        out.append(("reference", reference()))
    return out


@pytest.mark.parametrize("ndiv,lo,hi", [(48, 0.0, 1.0), (64, 1e15, np.inf), (255, 1e100, np.inf)])
def test_cloth_ilu0_growth(ndiv, lo, hi):
    for name, O in _oracles():
        g = _growth(O, ndiv)
        assert lo < g < hi or (hi == np.inf and not np.isfinite(g)), (name, ndiv, g)
