"""Mesh front end on the host side: medit files as FEDDLib reads them
(MeshFileReader.cpp / MeshFileReader.hpp, one-based ids) and the oracle's
P2-of-P1 restatement (buildP2ofP1MeshEdge), pinned against the structured P2
generator (buildMesh3D): P2-of-P1 of the structured P1 mesh must reproduce the
structured P2 mesh element by element.  No GPU needed."""
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def F():
    import feddlib_gb300
    return feddlib_gb300


def test_medit_fixture(F):
    m = F.medit_read(os.path.join(HERE, "golden", "two_tets.mesh"))
    np.testing.assert_array_equal(m["coords"], [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]])
    np.testing.assert_array_equal(m["node_flags"], [1, 2, 2, 3, 0])
    np.testing.assert_array_equal(m["tets"], [[0, 1, 2, 3], [1, 2, 3, 4]])
    np.testing.assert_array_equal(m["tet_flags"], [5, 6])
    np.testing.assert_array_equal(m["tris"], [[0, 1, 2], [1, 2, 4]])
    np.testing.assert_array_equal(m["tri_flags"], [11, 12])


def test_medit_round_trip_is_exact(F, tmp_path):
    xyz, el = F.structured_mesh(4, 1, seed=3)
    flags = (np.arange(xyz.shape[0]) % 7).astype(np.int32)
    path = tmp_path / "cube.mesh"
    F.medit_write(path, xyz, el, node_flags=flags, tet_flags=np.full(el.shape[0], 10),
                  tris=el[:5, :3], tri_flags=np.arange(5))
    m = F.medit_read(path)
    assert np.array_equal(m["coords"].view(np.uint64), xyz.view(np.uint64))
    np.testing.assert_array_equal(m["tets"], el)
    np.testing.assert_array_equal(m["node_flags"], flags)
    np.testing.assert_array_equal(m["tris"], el[:5, :3])
    np.testing.assert_array_equal(m["tri_flags"], np.arange(5))


@pytest.mark.parametrize("text,code", [
    ("Dimension 3\nVertices\n2\n0 0 0 0\n1 0 0 0\nTetrahedra\n1\n1 2 3 4 0\nEnd\n", 3),   # node id > nv
    ("Dimension 2\nVertices\n1\n0 0 0\nEnd\n", 8),                                      # 2D: unsupported
    ("Dimension 3\nVertices\n2\n0 0 0 0\n1 0 zero 0\n", 3),                              # not a number
])
def test_medit_rejects(F, tmp_path, text, code):
    path = tmp_path / "bad.mesh"
    path.write_text(text)
    with pytest.raises(F.FeddError) as ei:
        F.medit_read(path)
    assert ei.value.code == code


def test_medit_missing_file(F, tmp_path):
    with pytest.raises(F.FeddError) as ei:
        F.medit_read(tmp_path / "none.mesh")
    assert ei.value.code == 1  # FEDD_ERR_ARG


@pytest.mark.parametrize("M,seed", [(1, 0), (3, 2), (6, 9)])
def test_oracle_p2_of_p1_reproduces_structured_p2(M, seed):
    x1, c1, _ = O.mesh(M, 1, seed=seed)
    x2, c2, _ = O.mesh(M, 2, seed=seed)
    y2, d2 = O.p2_of_p1(x1, c1)
    assert y2.shape == x2.shape and d2.shape == c2.shape
    # same elements, vertices and edge midpoints, bit for bit (numbering differs)
    assert np.array_equal(y2[d2].view(np.uint64), x2[c2].view(np.uint64))
    # the reference numbering: P1 nodes first, edge nodes by sorted (min, max) pair
    assert np.array_equal(y2[:x1.shape[0]], x1)
    pairs = np.sort(np.stack([d2[:, [0, 1, 0, 0, 1, 2]], d2[:, [1, 2, 2, 3, 3, 3]]], -1), axis=-1)
    ids = d2[:, 4:]
    order = np.lexsort((pairs[..., 1].ravel(), pairs[..., 0].ravel()))
    assert np.all(np.diff(ids.ravel()[order]) >= 0)
