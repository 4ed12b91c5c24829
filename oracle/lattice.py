"""Stencil tables of the two lattices, taken from the reference's own outputs.

TEST INFRASTRUCTURE ONLY (used by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py).  The oracle's grids take their neighbour tables, weights,
volumes and value positions from here, not from the library under test, so
that a fault in the library's lattice construction cannot reach both sides of
a parity check.  tests/test_lattice.py checks that the library's tables equal
these.

Sources (fixtures under tests/golden/, written by tests/golden/make_golden.py
from the reference's code built here):

* TETRA12 - ref_tables.json: the reference's getLaplacian and getPositions
  (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:69-142), run.  Each value's
  four neighbours (block offset, slot) in the order the reference lists them
  (its kernel sums them in that order), the Hodge weight 1.5, the block edge
  sqrt(8), the tetrahedron volume sqrt(32/9) and the 12 circumcentres, all in
  units of block_scale.
* BCC2 - ref_mesh_hodge.json: DelaunayMesh::createBccGrid of the reference's
  Mesh library with unit cube edge (jukan_koodit/Mesh/DelaunayMesh.cpp:178-219,
  Mesh.cpp:1479-1512): the 14 edges of a lattice node (displacement, Hodge
  weight |dual face|/|edge|) and its dual volume.  Two conventions of this
  project are added, since the reference has no primal-node kernel: the
  corner node sits at 1/4 and the centre node at 3/4 of the block along each
  axis, and a value's neighbours are summed by weight class (largest weight
  first), then by (dz, dy, dx, slot).
"""
from __future__ import annotations

import json
import os
from functools import lru_cache

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden")

TETRA12, BCC2 = 0, 1


def _golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@lru_cache(maxsize=None)
def _tetra12():
    ref = _golden("ref_tables.json")
    nb = np.asarray(ref["neighbours"], dtype=np.int32).reshape(12, 4, 4)
    entry = np.zeros((12, 4, 5), dtype=np.int32)
    entry[:, :, :4] = nb  # (dx, dy, dz, slot), weight class 0
    return {"lattice": TETRA12, "slots": 12, "neighbours": 4, "classes": 1,
            "block_width": float(ref["block_width"]), "cell_volume": float(ref["volume"]),
            "class_weight": [float(ref["hodge"])], "position": np.asarray(ref["positions"], dtype=np.float64),
            "entry": entry}


@lru_cache(maxsize=None)
def _bcc2():
    mesh = _golden("ref_mesh_hodge.json")
    pos = np.array([[0.25] * 3, [0.75] * 3])
    # the node at the origin of the mesh's lattice: every BCC node has the same star
    node = next(n for n in mesh["nodes"] if all(abs(c) < 1e-12 for c in n["position"]))
    weights = sorted({round(float(e[3]), 12) for e in node["edges"]}, reverse=True)
    entry = []
    for s in range(2):
        row = []
        for e in node["edges"]:
            d = np.asarray(e[:3], dtype=np.float64)
            tgt = pos[s] + d
            blk = np.floor(tgt).astype(int)
            frac = tgt - blk
            sl = 0 if np.allclose(frac, 0.25) else 1
            assert np.allclose(frac, pos[sl]), "edge does not end on a lattice node"
            cls = weights.index(round(float(e[3]), 12))
            row.append((cls, int(blk[2]), int(blk[1]), int(blk[0]), sl))
        row.sort()
        entry.append([(dx, dy, dz, sl, cls) for cls, dz, dy, dx, sl in row])
    return {"lattice": BCC2, "slots": 2, "neighbours": len(node["edges"]), "classes": len(weights),
            "block_width": 1.0, "cell_volume": float(node["node_hodge"]), "class_weight": weights,
            "position": pos, "entry": np.asarray(entry, dtype=np.int32)}


def tables(lattice) -> dict:
    """The stencil of lattice 0 (TETRA12) or 1 (BCC2), in the layout of the
    library's gpe_lattice_info (positions and weights in block_scale units)."""
    return _tetra12() if int(lattice) == TETRA12 else _bcc2()


def value_positions(nx, ny, nz, block_scale, origin, lattice) -> np.ndarray:
    """Position of every value, shape (nz, ny, nx, slots, 3), in the reference's
    block order (GPUGrossPitaevskii_BCC.cu:258): origin + bs*(i*width + pos)."""
    t = tables(lattice)
    bw, pos = t["block_width"], t["position"]
    i = np.arange(nx)[None, None, :, None]
    j = np.arange(ny)[None, :, None, None]
    k = np.arange(nz)[:, None, None, None]
    out = np.empty((nz, ny, nx, t["slots"], 3))
    out[..., 0] = origin[0] + block_scale * (i * bw + pos[None, None, None, :, 0])
    out[..., 1] = origin[1] + block_scale * (j * bw + pos[None, None, None, :, 1])
    out[..., 2] = origin[2] + block_scale * (k * bw + pos[None, None, None, :, 2])
    return out


def harmonic(pos: np.ndarray, trap) -> np.ndarray:
    """0.5 * sum_a trap[a] * x_a^2 at each position."""
    return 0.5 * (trap[0] * pos[..., 0] ** 2 + trap[1] * pos[..., 1] ** 2 + trap[2] * pos[..., 2] ** 2)
