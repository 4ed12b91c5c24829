"""Parity against the reference itself: its own update kernel (compiled
unmodified for sm_103a) and this library's TETRA12 path, on the same inputs,
bit for bit.

The factors are computed as the reference computes them, the neighbours are
summed in the reference's table order, and the single-class update rounds as
the reference's kernel does (fma(L, S, c*psi)), so the library, the oracle and
the reference's kernel agree exactly.  Skipped where the cubin was not built
(it needs the reference source tree at build time).
"""
import numpy as np
import pytest

import refkernel
from helpers import grid_for, interleave, random_state
from conftest import golden
from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refkernel.available(), reason="oracle/_ref/ref_bcc.cubin not built here")]


@pytest.mark.parametrize("dims", [(5, 4, 3), (17, 9, 6), (1, 1, 1)])
def test_reference_update_kernel_matches_tetra12_fp64(dims):
    X, Y, Z = dims
    bs, dt, g, steps = 0.35, 1e-3, 80.0, 4
    bw = 8 ** 0.5
    inst = Instance(X, Y, Z, bs, dt, g, origin=tuple(-0.5 * n * bs * bw for n in dims))
    shp = (Z, Y, X, 12)
    even = random_state(shp, 11, 0.3)
    odd = random_state(shp, 12, 0.3)
    V = np.random.default_rng(13).uniform(0.0, 10.0, size=shp)

    ref = refkernel.ReferenceUpdate(X, Y, Z)
    ref.upload(interleave(even, np.float64), interleave(odd, np.float64), V * dt)
    ref.step(steps, bs, dt, g)
    re, ro = ref.download()

    st = Stepper([inst], lattice=Lattice.TETRA12, precision=Precision.FP64, kernel=Kernel.PLAIN,
                 potential=Potential.ARRAY)
    st.upload(0, even, odd, V)
    st.step(steps)
    oe, oo = st.download(0)

    # the CPU oracle with the reference's own table order
    tab = golden("ref_tables.json")
    nb = np.array(tab["neighbours"]).reshape(12, 4, 4)
    entry = np.concatenate([nb, np.zeros((12, 4, 1), np.int64)], axis=2).astype(np.int32)
    import oracle.oracle as orc
    go = orc.Grid(X, Y, Z, entry, [tab["hodge"]], bs, dt, g)
    ce, co = interleave(even, np.float64), interleave(odd, np.float64)
    go.leapfrog(ce, co, np.ascontiguousarray(V * dt), steps)
    st.close()

    np.testing.assert_array_equal(oe, re)
    np.testing.assert_array_equal(oo, ro)
    np.testing.assert_array_equal(ce, re)
    np.testing.assert_array_equal(co, ro)
