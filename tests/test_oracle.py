"""The CPU oracle on its own: agreement between its summation orders, with the
reference's own neighbour table, and the scheme's known properties.  No GPU."""
import math

import numpy as np
import pytest

import oracle.oracle as orc
from conftest import golden
from helpers import interleave, random_state, rel_l2
from oracle.lattice import tables
from vaikkari_gb300.gpe import Instance, Lattice, value_positions
from vaikkari_gb300 import workloads


def _grid(lattice, dims, bs=0.3, dt=1e-3, g=50.0, entry=None):
    info = tables(lattice)
    nx, ny, nz = dims
    return orc.Grid(nx, ny, nz, info["entry"] if entry is None else entry, info["class_weight"], bs, dt, g)


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 5, 7), (13, 7, 9)])
def test_bcc2_box_order_agrees_with_table_order(dims):
    """The fused kernel's summation order (box sums reused across planes) and the
    generic table order compute the same stencil up to rounding."""
    g = _grid(Lattice.BCC2, dims)
    shp = (dims[2], dims[1], dims[0], 2)
    e = interleave(random_state(shp, 1, 0.3), np.float64)
    o = interleave(random_state(shp, 2, 0.3), np.float64)
    v = np.ascontiguousarray(np.random.default_rng(0).uniform(0, 0.01, shp))
    e1, o1, e2, o2 = e.copy(), o.copy(), e.copy(), o.copy()
    g.leapfrog(e1, o1, v, 5)
    g.leapfrog_bcc2(e2, o2, v, 5)
    assert np.abs(e1 - e2).max() <= 1e-14 * np.abs(e1).max()


def test_tetra12_reference_table_order_agrees():
    """Leapfrog with the reference's own 48-entry table (its order) and with the
    geometry-derived table (its order) agree to rounding."""
    ref = golden("ref_tables.json")
    nb = np.array(ref["neighbours"]).reshape(12, 4, 4)
    entry_ref = np.concatenate([nb, np.zeros((12, 4, 1), np.int64)], axis=2).astype(np.int32)
    dims = (4, 3, 5)
    shp = (dims[2], dims[1], dims[0], 12)
    ga = _grid(Lattice.TETRA12, dims, bs=0.2)
    gb = _grid(Lattice.TETRA12, dims, bs=0.2, entry=entry_ref)
    e = interleave(random_state(shp, 3, 0.3), np.float64)
    o = interleave(random_state(shp, 4, 0.3), np.float64)
    v = np.ascontiguousarray(np.random.default_rng(1).uniform(0, 0.01, shp))
    e1, o1, e2, o2 = e.copy(), o.copy(), e.copy(), o.copy()
    ga.leapfrog(e1, o1, v, 4)
    gb.leapfrog(e2, o2, v, 4)
    assert np.abs(e1 - e2).max() <= 1e-14 * np.abs(e1).max()


def test_fp32_scheme_accuracy_small():
    """FP32 against FP64 of the same scheme on a Gaussian condensate (16^3 cells,
    300 steps): relative L2 well under 1e-5."""
    c = workloads.config1(n=16)
    info = tables(Lattice.BCC2)
    inst = c.inst
    g = _grid(Lattice.BCC2, (16, 16, 16), bs=inst.block_scale, dt=inst.dt, g=inst.g)
    vdt64 = np.ascontiguousarray(c.V * inst.dt)
    vdt32 = np.ascontiguousarray((c.V.astype(np.float32).astype(np.float64) * inst.dt).astype(np.float32))
    vol = info["cell_volume"] * inst.block_scale ** 3
    e64 = interleave(c.psi, np.float64)
    mu = g.observables(e64, vdt64, vol)["mu"]
    odd = workloads.odd_from_even(c.psi, mu, inst.dt)
    o64 = interleave(odd, np.float64)
    e32, o32 = e64.astype(np.float32), o64.astype(np.float32)
    g.leapfrog_bcc2(e64, o64, vdt64, 300)
    g.leapfrog_bcc2(e32, o32, vdt32, 300)
    assert rel_l2(e32, e64) < 1e-5
    n64 = g.observables(e64, vdt64, vol)["norm"]
    n32 = g.observables(e32, vdt32, vol)["norm"]
    assert abs(n32 - n64) / n64 < 1e-6


def test_imaginary_time_harmonic_ground_state():
    """g = 0, isotropic trap: the normalised Euler iteration converges to
    mu ~ 3/2 (discretisation error O(a^2))."""
    n, L = 16, 5.0
    a = 2 * L / n
    info = tables(Lattice.BCC2)
    inst = Instance(n, n, n, a, 5e-3, 0.0, origin=(-L, -L, -L))
    g = _grid(Lattice.BCC2, (n, n, n), bs=a, dt=5e-3, g=0.0)
    rng = np.random.default_rng(3)
    psi = interleave((1.0 + 0.1 * rng.standard_normal((n, n, n, 2))).astype(np.complex128), np.float64)
    vdt = np.ascontiguousarray(workloads.harmonic(value_positions(inst, info), (1, 1, 1)) * inst.dt)
    vol = info["cell_volume"] * a ** 3
    conv, mu = g.imaginary(psi, vdt, vol, 4000, 1e-10)
    assert conv > 0
    assert mu[conv] == pytest.approx(1.5, rel=0.05)
    assert g.observables(psi, vdt, vol)["norm"] == pytest.approx(1.0, rel=1e-12)


def test_leapfrog_conserves_norm_approximately():
    """The staggered leapfrog conserves the norm up to O(dt) oscillations."""
    c = workloads.config1(n=12)
    inst = c.inst
    info = tables(Lattice.BCC2)
    g = _grid(Lattice.BCC2, (12, 12, 12), bs=inst.block_scale, dt=inst.dt, g=inst.g)
    vdt = np.ascontiguousarray(c.V * inst.dt)
    vol = info["cell_volume"] * inst.block_scale ** 3
    e = interleave(c.psi, np.float64)
    mu = g.observables(e, vdt, vol)["mu"]
    o = interleave(workloads.odd_from_even(c.psi, mu, inst.dt), np.float64)
    n0 = g.observables(e, vdt, vol)["norm"]
    g.leapfrog(e, o, vdt, 200)
    assert abs(g.observables(e, vdt, vol)["norm"] - n0) / n0 < 1e-3


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 3, 4), (9, 7, 11)])
def test_bcc2_fast_path_bit_identical(dims):
    """The timed CPU baseline (direct interior indexing) equals the checked path."""
    g = _grid(Lattice.BCC2, dims)
    shp = (dims[2], dims[1], dims[0], 2)
    e = interleave(random_state(shp, 5, 0.3), np.float64)
    o = interleave(random_state(shp, 6, 0.3), np.float64)
    v = np.ascontiguousarray(np.random.default_rng(2).uniform(0, 0.01, shp))
    e1, o1, e2, o2 = e.copy(), o.copy(), e.copy(), o.copy()
    g.leapfrog_bcc2(e1, o1, v, 3)
    g.leapfrog_bcc2_fast(e2, o2, v, 3)
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(o1, o2)


def test_workloads_same_with_oracle_geometry():
    """The CPU baseline builds the seeded batch with the oracle's stencil tables
    (so it never loads the library); the condensates must be the very ones the
    GPU path builds with the library's tables."""
    from vaikkari_gb300.gpe import lattice_info
    a = workloads.config4(geometry=tables(Lattice.BCC2), count=6)
    b = workloads.config4(geometry=lattice_info(Lattice.BCC2), count=6)
    for x, y in zip(a, b):
        assert x.inst == y.inst
        np.testing.assert_array_equal(x.psi, y.psi)
    c1 = workloads.config1(Lattice.TETRA12, geometry=tables(Lattice.TETRA12), n=6)
    c2 = workloads.config1(Lattice.TETRA12, n=6)
    np.testing.assert_array_equal(c1.V, c2.V)
    np.testing.assert_allclose(c1.psi, c2.psi, rtol=1e-14, atol=0)
