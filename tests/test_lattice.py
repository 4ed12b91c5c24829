"""Stencil tables derived by the library from the BCC geometry, pinned against
the reference's own outputs (tests/golden, generated by running the
reference's getLaplacian/getPositions and its Mesh library)."""
import itertools
import math

import numpy as np
import pytest

from conftest import golden
from vaikkari_gb300.gpe import Lattice, lattice_info


def _neigh_vectors(info):
    """Per slot: list of (displacement in block_scale units, weight)."""
    W = info["block_width"]
    pos = info["position"]
    out = []
    for s in range(info["slots"]):
        row = []
        for dx, dy, dz, sl, c in info["entry"][s]:
            d = np.array([dx, dy, dz]) * W + pos[sl] - pos[s]
            row.append((d, info["class_weight"][c]))
        out.append(row)
    return out


def test_tetra12_table_equals_reference_getLaplacian():
    """Same neighbours and the same summation order as the reference's table."""
    ref = golden("ref_tables.json")
    ours = lattice_info(Lattice.TETRA12)
    assert ours["slots"] == 12 and ours["neighbours"] == 4 and ours["classes"] == 1
    nb = np.array(ref["neighbours"]).reshape(12, 4, 4)
    for s in range(12):
        want = [tuple(int(v) for v in e) for e in nb[s]]
        got = [tuple(int(v) for v in e[:4]) for e in ours["entry"][s]]
        assert got == want, f"slot {s}"


def test_tetra12_positions_weight_volume_equal_reference():
    ref = golden("ref_tables.json")
    ours = lattice_info(Lattice.TETRA12)
    np.testing.assert_allclose(ours["position"], np.array(ref["positions"]), rtol=0, atol=1e-14)
    assert ours["class_weight"][0] == pytest.approx(ref["hodge"], rel=1e-13)
    assert ours["block_width"] == pytest.approx(ref["block_width"], rel=1e-15)
    assert ours["cell_volume"] == pytest.approx(ref["volume"], rel=1e-13)


def test_bcc2_weights_equal_mesh_library():
    """getEdgeHodge/getNodeHodge of DelaunayMesh::createBccGrid with h = 1."""
    mesh = golden("ref_mesh_hodge.json")
    ours = lattice_info(Lattice.BCC2)
    assert ours["slots"] == 2 and ours["neighbours"] == 14 and ours["classes"] == 2
    vec = _neigh_vectors(ours)
    for node in mesh["nodes"]:
        assert ours["cell_volume"] == pytest.approx(node["node_hodge"], rel=1e-12)
        want = sorted((tuple(np.round(e[:3], 9)), round(e[3], 9)) for e in node["edges"])
        for s in range(2):
            got = sorted((tuple(np.round(d, 9)), round(w, 9)) for d, w in vec[s])
            assert got == want, f"slot {s}"


def test_tetra12_weights_equal_mesh_library():
    """getBodyHodge/getFaceHodge around interior tetrahedra, in units of the cube edge."""
    mesh = golden("ref_mesh_hodge.json")
    ours = lattice_info(Lattice.TETRA12)
    W = ours["block_width"]
    vec = _neigh_vectors(ours)
    slot_sets = [sorted((tuple(np.round(d / W, 9)), round(w * W * W, 9)) for d, w in row) for row in vec]
    assert len(mesh["bodies"]) == 12
    for body in mesh["bodies"]:
        # 1/|tet| in cube-edge units equals 1/(cell_volume / W^3)
        assert body["body_hodge"] == pytest.approx(W ** 3 / ours["cell_volume"], rel=1e-12)
        got = sorted((tuple(np.round(f[:3], 9)), round(f[3], 9)) for f in body["faces"])
        assert got in slot_sets


def test_quadratic_exactness_bcc2():
    """Primal-node stencil: sum_k w_k d_k d_k^T = 2 I and sum_k w_k d_k = 0 at
    every value, so Lap(x^2) = 2 exactly."""
    info = lattice_info(Lattice.BCC2)
    for row in _neigh_vectors(info):
        M = sum(w * np.outer(d, d) for d, w in row)
        v = sum(w * d for d, w in row)
        np.testing.assert_allclose(M, 2 * np.eye(3), atol=1e-12)
        np.testing.assert_allclose(v, 0, atol=1e-12)


def test_quadratic_exactness_tetra12():
    """Dual-node (circumcentre) stencil of the reference: exact on r^2 at every
    value (trace = 6), but each tetrahedron is anisotropic (diag 3, 1.5, 1.5);
    only the average over the 12 orientations is 2 I."""
    info = lattice_info(Lattice.TETRA12)
    Ms = []
    for row in _neigh_vectors(info):
        M = sum(w * np.outer(d, d) for d, w in row)
        assert np.trace(M) == pytest.approx(6.0, abs=1e-12)
        assert sorted(np.round(np.linalg.eigvalsh(M), 9)) == [1.5, 1.5, 3.0]
        Ms.append(M)
    np.testing.assert_allclose(np.mean(Ms, axis=0), 2 * np.eye(3), atol=1e-12)


@pytest.mark.parametrize("lattice", [Lattice.TETRA12, Lattice.BCC2])
def test_table_symmetric(lattice):
    info = lattice_info(lattice)
    edges = set()
    for s in range(info["slots"]):
        for dx, dy, dz, sl, c in info["entry"][s]:
            edges.add((s, int(sl), int(dx), int(dy), int(dz), int(c)))
    for (s, sl, dx, dy, dz, c) in edges:
        assert (sl, s, -dx, -dy, -dz, c) in edges


def test_tetra12_summation_order_is_class_then_offset():
    info = lattice_info(Lattice.BCC2)
    for s in range(2):
        keys = [(int(e[4]), int(e[2]), int(e[1]), int(e[0]), int(e[3])) for e in info["entry"][s]]
        assert keys == sorted(keys)


def test_vortex_fixture_header_consistent():
    """The binary header of state.dat decodes to the fields VortexState::load
    reads (VortexState.cpp:49-72) and the diagnostics main() prints."""
    h = golden("ref_state_header.json")
    v = golden("ref_vortex_state.json")
    assert (h["kappa"], h["g"], h["mu"]) == (v["kappa"], v["g"], v["mu"])
    assert h["file_bytes"] == 52 + 8 * h["rsize"] * h["zsize"]
    assert v["block_scale"] == pytest.approx(0.0699674, abs=5e-8)
    assert v["maxr"] == pytest.approx(8.53991, abs=5e-6)
    assert v["maxz"] == pytest.approx(29.79, abs=1e-12)


@pytest.mark.parametrize("lattice", [Lattice.TETRA12, Lattice.BCC2])
def test_library_tables_equal_the_oracles(lattice):
    """The oracle builds its grids from its own copy of the reference's tables
    (oracle/lattice.py, from tests/golden), not from the library.  The library's
    tables must equal those: the same neighbours in the same summation order, the
    same weight doubles and the same value positions bit for bit (the trap
    potential is formed from them).  The TETRA12 tetrahedron volume is derived
    from the geometry and agrees with the reference's sqrt(32/9) to 2 ulp; it only
    scales the observables."""
    from oracle.lattice import tables
    ours, ref = lattice_info(lattice), tables(lattice)
    assert (ours["slots"], ours["neighbours"], ours["classes"]) == (ref["slots"], ref["neighbours"], ref["classes"])
    np.testing.assert_array_equal(np.asarray(ours["entry"]), ref["entry"])
    assert list(ours["class_weight"]) == list(ref["class_weight"])
    assert ours["block_width"] == ref["block_width"]
    np.testing.assert_array_equal(np.asarray(ours["position"]), ref["position"])
    assert ours["cell_volume"] == pytest.approx(ref["cell_volume"], rel=1e-15, abs=0)
