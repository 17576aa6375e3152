"""Dynamic linear-tet assembly in the CPU oracle (backward Euler,
stiffness-warped backward Euler, Newmark-beta: fem_solidlinear.h:331-530),
pinned against the reference: the fixture tests/golden/dynamic.npz and
directly where the reference is built. The element matrix is summed in one
expression instead of the reference's two, so values agree to 1e-14
relative, not bit for bit."""
import numpy as np
import pytest

import dyn_systems as DS
from conftest import golden, rel_err
from oracle import HAVE_REFERENCE_BUILD


@pytest.mark.parametrize("kind", DS.KINDS)
def test_port_matches_golden(port, kind):
    G = golden("dynamic")
    s = DS.inputs(port)
    vc, vd, b = DS.assemble(port, s, kind)
    assert rel_err(vc, G[f"{kind}_vc"]) < 1e-14
    assert rel_err(vd, G[f"{kind}_vd"]) < 1e-14
    assert rel_err(b, G[f"{kind}_b"]) < 1e-14


def test_warp_with_identity_rotations_is_beuler(port):
    """R = I for every node: P + u + dt v - R P = u + dt v and R K R^T = K."""
    s = DS.inputs(port)
    s["rot"] = np.tile(np.eye(3).ravel(), s["xyz"].size // 3)
    a, b = DS.assemble(port, s, "warp"), DS.assemble(port, s, "beuler")
    for x, y in zip(a, b):
        assert rel_err(x, y) < 1e-14


@pytest.mark.skipif(not HAVE_REFERENCE_BUILD(), reason="reference driver not built")
@pytest.mark.parametrize("kind", DS.KINDS)
def test_port_equals_reference_directly(port, kind):
    from oracle import reference
    R = reference()
    s = DS.inputs(port)
    for x, y in zip(DS.assemble(port, s, kind), DS.assemble(R, s, kind)):
        assert rel_err(x, y) < 1e-14


def test_hex_q1_matches_golden_bit_for_bit(port):
    """The Q1 element follows the reference's arithmetic exactly (three-point
    Gauss rule from the reference's table, same summation order)."""
    G = golden("dynamic")
    vc, vd, b = DS.assemble_hex(port, DS.hex_inputs(port))
    assert np.array_equal(vc, G["hexq1_vc"]) and np.array_equal(vd, G["hexq1_vd"])
    assert np.array_equal(b, G["hexq1_b"])


def test_hex_q1_element_is_symmetric_and_annihilates_translations(port):
    """The unit-cube element matrix is symmetric and maps rigid translations to zero."""
    from oracle.oracle import hex_grid
    xyz, hexa = hex_grid(1, 1, 1, 1.0)
    emat, _ = port.emat_hex_q1(xyz.reshape(-1, 3)[hexa], 1.0, 2.0, 1.0, np.zeros(3), np.zeros((8, 3)))
    K = emat.transpose(0, 2, 1, 3).reshape(24, 24)
    assert np.abs(K - K.T).max() < 1e-14
    for d in range(3):
        t = np.zeros((8, 3))
        t[:, d] = 1.0
        assert np.abs(K @ t.ravel()).max() < 1e-14
