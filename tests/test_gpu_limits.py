"""Capacity limits of the row kernels: a node may be shared by at most 64
elements (the warp's incidence list holds two words per lane).  A fan of
tetrahedra around one centre node at exactly 64 incidences assembles and
matches the oracle; one more is rejected at creation with FEDD_ERR_CAPACITY,
not assembled wrongly."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300 as F
    return F


def fan(n_top, n_bottom):
    """Centre node 0, poles 1 (top) and 2 (bottom), ring nodes after them;
    tets (centre, ring i, ring i+1, top) and (centre, ring i+1, ring i,
    bottom), all positively oriented.  The centre has n_top + n_bottom
    incidences."""
    n = max(n_top, n_bottom)
    ang = 2.0 * np.pi * np.arange(n) / n
    ring = np.stack([np.cos(ang), np.sin(ang), np.zeros(n)], axis=1)
    xyz = np.vstack([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, -1.0], ring])
    el = []
    for i in range(n_top):
        el.append([0, 3 + i, 3 + (i + 1) % n, 1])
    for i in range(n_bottom):
        el.append([0, 3 + (i + 1) % n, 3 + i, 2])
    return np.ascontiguousarray(xyz), np.ascontiguousarray(el, dtype=np.int32)


def test_fan_is_positively_oriented():
    xyz, el = fan(32, 32)
    p = xyz[el]
    det = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    assert (det > 0).all()


def test_node_with_64_incidences_assembles(F):
    xyz, el = fan(32, 32)
    a = F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0)
    (v,), b, _ = a.assemble()
    orp, oci, ov = O.assemble_laplace(1, 1, xyz, el)
    rp, ci, _ = a.pattern(0)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert np.linalg.norm(v - ov) <= 1e-12 * np.linalg.norm(ov)
    assert np.linalg.norm(b - O.assemble_rhs(1, 1, xyz, el, 1.0)) <= 1e-12 * np.linalg.norm(b)


def test_node_with_65_incidences_is_rejected(F):
    xyz, el = fan(33, 32)
    with pytest.raises(F.FeddError) as ei:
        F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0)
    assert ei.value.code == 9  # FEDD_ERR_CAPACITY
