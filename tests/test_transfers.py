"""Batched transfers (gpe_upload_many / gpe_download_many) against the
per-instance calls: the same fields on the device and back, bit for bit, for
every precision and both potential forms; bad calls return error codes."""
import numpy as np
import pytest

from helpers import random_state
from vaikkari_gb300.gpe import GpeError, Instance, Kernel, Lattice, Potential, Precision, Stepper

pytestmark = pytest.mark.gpu

DIMS = [(1, 1, 1), (5, 3, 7), (17, 9, 4), (33, 12, 6)]


def _insts():
    return [Instance(nx, ny, nz, 0.3 + 0.05 * k, 1e-3, 20.0 + k, origin=(-0.15 * nx, -0.15 * ny, -0.15 * nz))
            for k, (nx, ny, nz) in enumerate(DIMS)]


@pytest.mark.parametrize("prec,potential", [(Precision.FP32, Potential.ARRAY), (Precision.FP64, Potential.TRAP),
                                            (Precision.FP32C, Potential.TRAP), (Precision.FP32C, Potential.ARRAY)])
def test_batched_transfers_equal_single_calls(prec, potential):
    insts = _insts()
    kw = dict(lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=potential)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    rng = np.random.default_rng(3)
    items = []
    for i in range(len(insts)):
        shp = a.shape(i)
        V = rng.uniform(0, 5, shp) if potential == Potential.ARRAY else None
        items.append((i, random_state(shp, 10 + i, 0.3), random_state(shp, 20 + i, 0.3), V))
    for i, e, o, V in items:
        a.upload(i, e, o, V)
    b.upload_many(items[::-1])            # any order
    a.step(5)
    b.step(5)
    want = [a.download(i) for i in range(len(insts))]
    got = b.download_many(range(len(insts)))
    a.close()
    b.close()
    for (we, wo), (ge, go) in zip(want, got):
        assert ge.dtype == we.dtype
        np.testing.assert_array_equal(ge, we)
        np.testing.assert_array_equal(go, wo)


def test_download_many_into_given_buffers_and_partial():
    insts = _insts()
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED, potential=Potential.TRAP)
    fields = [(i, random_state(st.shape(i), i, 0.3), random_state(st.shape(i), 50 + i, 0.3), None)
              for i in range(len(insts))]
    st.upload_many(fields)
    outs = [(np.empty(st.shape(i) + (2,), np.float32), None) for i in (2, 0)]
    st.download_many([2, 0], outs=outs)    # even fields only, two of the instances
    for (e, _), i in zip(outs, (2, 0)):
        np.testing.assert_array_equal(e, st.download(i, odd=False)[0])
    st.close()


def test_batched_transfers_reject_bad_calls():
    insts = _insts()
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED, potential=Potential.ARRAY)
    shp = st.shape(0)
    e = random_state(shp, 1, 0.3)
    with pytest.raises(GpeError):
        st.upload_many([(0, e, e, None)])                 # array potential missing
    with pytest.raises(GpeError):
        st.upload_many([(0, e, None, np.zeros(shp))])     # odd field missing in real time
    with pytest.raises(IndexError):
        st.upload_many([(7, e, e, np.zeros(shp))])        # no such instance
    with pytest.raises(ValueError):
        st.download_many([0], outs=[(np.empty(shp + (2,), np.float64), None)])   # wrong element type
    st.close()
