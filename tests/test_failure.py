"""Failure detection without faulting the GPU.

A bounded device wait that runs out (forced with the test hook that withholds
one TMA copy) turns into GPE_ERR_TIMEOUT on the host and leaves the context
usable; NaN in a field trips the observables watchdog; bad calls return codes.
"""
import numpy as np
import pytest

from helpers import grid_for, interleave, random_state, vdt_for
from vaikkari_gb300.gpe import GpeError, Instance, Kernel, Lattice, Potential, Precision, Status, Stepper

pytestmark = pytest.mark.gpu


def _stepper(kernel=Kernel.FUSED, tile=0, precision=Precision.FP32):
    inst = Instance(8, 8, 8, 0.4, 1e-3, 50.0, origin=(-1.6, -1.6, -1.6))
    return Stepper([inst], lattice=Lattice.BCC2, precision=precision, kernel=kernel, potential=Potential.TRAP,
                   graph_steps=-1, tile=tile)


def _tiles():
    """The default variant and the first and last whole-step variants (double
    buffered sets; their consumers agree on a timeout at the per-plane barrier)."""
    from vaikkari_gb300.gpe import variants
    two = [v["tile"] for v in variants() if v["half_steps"] == 2]
    return [0, two[0], two[-1]]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_bounded_wait_timeout_is_reported_and_context_survives(which):
    st = _stepper(tile=_tiles()[which])
    shp = st.shape(0)
    e, o = random_state(shp, 1, 0.3), random_state(shp, 2, 0.3)
    st.upload(0, e, o)
    st.debug_inject(3)
    st.step(1)
    with pytest.raises(GpeError) as err:
        st.synchronize()
    assert err.value.status == Status.TIMEOUT
    # the error word was cleared and the context still works: a clean run
    # afterwards is bit-exact with the oracle
    st.debug_inject(-1)
    st.upload(0, e, o)
    st.step(3)
    ge, go = st.download(0)
    g = grid_for(st, 0)
    we, wo = interleave(e, np.float32), interleave(o, np.float32)
    g.leapfrog_bcc2(we, wo, vdt_for(st, 0), 3)
    st.close()
    np.testing.assert_array_equal(ge, we)
    np.testing.assert_array_equal(go, wo)


def test_bounded_wait_timeout_with_compensated_storage():
    """The compensated kernel's stages also carry the residual tile; a withheld
    copy still ends in GPE_ERR_TIMEOUT, and a clean run afterwards equals the
    oracle bit for bit."""
    import oracle.oracle as orc
    st = _stepper(precision=Precision.FP32C)
    shp = st.shape(0)
    e, o = random_state(shp, 1, 0.3), random_state(shp, 2, 0.3)
    st.upload(0, e, o)
    st.debug_inject(3)
    st.step(1)
    with pytest.raises(GpeError) as err:
        st.synchronize()
    assert err.value.status == Status.TIMEOUT
    st.debug_inject(-1)
    st.upload(0, e, o)
    st.step(3)
    ge, go = st.download(0)
    eh, el = orc.split_comp(interleave(e, np.float64))
    oh, ol = orc.split_comp(interleave(o, np.float64))
    grid_for(st, 0).leapfrog_bcc2_comp(eh, oh, el, ol, vdt_for(st, 0), 3)
    st.close()
    np.testing.assert_array_equal(ge, orc.join_comp(eh, el))
    np.testing.assert_array_equal(go, orc.join_comp(oh, ol))


def test_nan_in_field_trips_the_watchdog():
    st = _stepper()
    shp = st.shape(0)
    e = random_state(shp, 3, 0.3)
    e[2, 3, 4, 1] = complex(np.nan, 0.0)
    st.upload(0, e, e)
    with pytest.raises(GpeError) as err:
        st.observables(0)
    assert err.value.status == Status.NOT_FINITE
    st.close()


def test_debug_inject_needs_the_fused_kernel():
    st = _stepper(Kernel.PLAIN)
    with pytest.raises(GpeError) as err:
        st.debug_inject(1)
    assert err.value.status == Status.UNSUPPORTED
    st.close()
