"""The persistent kernel variants (gpe_variant_kind 2).

One cooperative launch advances every instance of a batch by all the steps of
a gpe_step call; each work item starts a half-step as soon as the items it
reads from (its neighbours within one tile and one z-chunk) have published
the previous one.  The arithmetic is the one-launch-per-half-step kernel's, so
the fields must equal the CPU oracle bit for bit, across calls (the epoch words
carry over), with several items per CTA (the ring continues across items), in
FP64, FP32 and compensated FP32.  A withheld copy must end the whole launch in
GPE_ERR_TIMEOUT within a few seconds, and the handle must work again after it.
"""
import time

import numpy as np
import pytest

import oracle.oracle as orc
from helpers import grid_for, interleave, random_state, vdt_for
from vaikkari_gb300.gpe import (GpeError, Instance, Kernel, Lattice, Mode, Potential, Precision, Status, Stepper,
                                variants)

pytestmark = pytest.mark.gpu


def _tiles():
    return [v["tile"] for v in variants() if v["persistent"]]


def _insts(dims_list):
    out = []
    for k, (nx, ny, nz) in enumerate(dims_list):
        bs = 0.3 + 0.05 * k
        origin = tuple(-0.5 * n * bs + 0.1 * k for n in (nx, ny, nz))
        out.append(Instance(nx, ny, nz, block_scale=bs, dt=1e-3 * (1 + 0.2 * k), g=50.0 + 10 * k, origin=origin,
                            trap=(1.0, 1.5 + 0.1 * k, 0.7)))
    return out


def _check(prec, potential, dims_list, calls, tile, zchunk=0, seed=0):
    """Steps a batch with `calls` gpe_step calls (step counts) and compares every
    field with the oracle run for the total."""
    insts = _insts(dims_list)
    st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=potential, tile=tile,
                 zchunk=zchunk)
    rng = np.random.default_rng(seed)
    want = []
    for i in range(len(insts)):
        shp = st.shape(i)
        even = random_state(shp, seed + 10 * i, 0.3)
        odd = random_state(shp, seed + 10 * i + 1, 0.3)
        V = rng.uniform(0.0, 10.0, size=shp)
        st.upload(i, even, odd, V if potential == Potential.ARRAY else None)
        g, vdt = grid_for(st, i), vdt_for(st, i, V)
        if prec == Precision.FP32C:
            eh, el = orc.split_comp(interleave(even, np.float64))
            oh, ol = orc.split_comp(interleave(odd, np.float64))
            g.leapfrog_bcc2_comp(eh, oh, el, ol, vdt, sum(calls))
            want.append((orc.join_comp(eh, el), orc.join_comp(oh, ol)))
        else:
            T = np.float64 if prec == Precision.FP64 else np.float32
            e, o = interleave(even, T), interleave(odd, T)
            g.leapfrog_bcc2(e, o, vdt, sum(calls))
            want.append((e, o))
    n0 = st.launch_count()
    for c in calls:
        st.step(c)
    launches = st.launch_count() - n0
    for i in range(len(insts)):
        ge, go = st.download(i)
        np.testing.assert_array_equal(ge, want[i][0], err_msg=f"tile {tile} even, instance {i}")
        np.testing.assert_array_equal(go, want[i][1], err_msg=f"tile {tile} odd, instance {i}")
    st.close()
    return launches


SIZES = [(1, 1, 1), (3, 5, 7), (13, 7, 9), (40, 9, 20), (33, 17, 5)]


def test_there_are_persistent_variants():
    vs = [v for v in variants() if v["persistent"]]
    assert len(vs) >= 1 and all(v["half_steps"] == 1 and v["kind"] == 2 for v in vs)


@pytest.mark.parametrize("potential", [Potential.TRAP, Potential.ARRAY])
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32, Precision.FP32C])
def test_persistent_variants_bit_exact(prec, potential):
    """Every persistent variant on a batch of ragged sizes, in two calls of odd
    length (3 + 4 steps): one launch per call."""
    for tile in _tiles():
        assert _check(prec, potential, SIZES, [3, 4], tile) == 2


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32C])
def test_persistent_many_items_per_cta(prec):
    """One-plane z-chunks give several thousand work items, far more than the
    resident CTAs, so every CTA runs many items per half-step and its ring
    continues across items and half-steps; a single one-step call, then ten."""
    dims = [(64, 64, 64), (48, 40, 36), (5, 3, 9)]
    for tile in _tiles()[:2]:
        assert _check(prec, Potential.TRAP, dims, [1, 10], tile, zchunk=1, seed=3) == 2


def test_persistent_equals_the_half_step_kernel():
    """The same batch through the default one-launch-per-half-step variant and
    through a persistent one: identical fields after 25 steps."""
    insts = _insts(SIZES)
    out = []
    for tile in (0, _tiles()[0]):
        st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED,
                     potential=Potential.TRAP, tile=tile)
        for i in range(len(insts)):
            shp = st.shape(i)
            st.upload(i, random_state(shp, 50 + i, 0.3), random_state(shp, 60 + i, 0.3))
        st.step(25)
        out.append([st.download(i) for i in range(len(insts))])
        st.close()
    for (a_e, a_o), (b_e, b_o) in zip(*out):
        np.testing.assert_array_equal(a_e, b_e)
        np.testing.assert_array_equal(a_o, b_o)


def test_persistent_timeout_ends_the_launch_and_the_handle_recovers():
    """The test hook withholds one copy of item 0's first half-step: that CTA's
    consumers time out, set the error word, and every other CTA's waits see it
    and stop, so the launch of 50 steps ends within a few seconds instead of
    hanging; GPE_ERR_TIMEOUT is reported, and after it the epoch words are reset
    and a clean run equals the oracle."""
    tile = _tiles()[0]
    insts = _insts([(40, 24, 30), (16, 16, 16)])
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED,
                 potential=Potential.TRAP, tile=tile, zchunk=2)
    fields = []
    for i in range(len(insts)):
        shp = st.shape(i)
        fields.append((random_state(shp, 70 + i, 0.3), random_state(shp, 80 + i, 0.3)))
        st.upload(i, *fields[i])
    st.debug_inject(3)
    t0 = time.perf_counter()
    st.step(50)
    with pytest.raises(GpeError) as err:
        st.synchronize()
    assert err.value.status == Status.TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    st.debug_inject(-1)
    want = []
    for i in range(len(insts)):
        st.upload(i, *fields[i])
        e, o = interleave(fields[i][0], np.float32), interleave(fields[i][1], np.float32)
        grid_for(st, i).leapfrog_bcc2(e, o, vdt_for(st, i), 6)
        want.append((e, o))
    st.step(6)
    for i in range(len(insts)):
        ge, go = st.download(i)
        np.testing.assert_array_equal(ge, want[i][0])
        np.testing.assert_array_equal(go, want[i][1])
    st.close()


def test_persistent_refuses_imaginary_time_and_slabs():
    tile = _tiles()[0]
    insts = _insts([(8, 8, 8), (8, 8, 8)])
    with pytest.raises(GpeError) as err:
        Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED, mode=Mode.IMAGINARY,
                potential=Potential.TRAP, tile=tile)
    assert err.value.status == Status.UNSUPPORTED
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED,
                 potential=Potential.TRAP, tile=tile)
    with pytest.raises(GpeError) as err:
        st.link_z(0, 1)
    assert err.value.status == Status.UNSUPPORTED
    st.close()
