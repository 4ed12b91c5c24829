"""gpe_round_trip: upload, steps, observables and download of every instance in
one call, with the copies of some instance groups overlapping the steps of
others.  Its fields and observables must equal, bit for bit, those of the same
calls made one after another (gpe_upload_many, gpe_step, gpe_observables_get,
gpe_download_many) in every storage, lattice and kernel form; a launch count
shows where the instances went in groups; output buffers may be the input ones;
a timed-out wait is reported as by the other calls."""
import numpy as np
import pytest

from helpers import random_state
from vaikkari_gb300.gpe import (GpeError, Instance, Kernel, Lattice, Mode, Potential, Precision, Status, Stepper,
                                variants)

pytestmark = pytest.mark.gpu

BW = 8 ** 0.5
DIMS = [(40, 9, 20), (1, 1, 1), (33, 17, 5), (24, 24, 24), (5, 3, 7), (17, 30, 9)]


def _insts(dims, tetra=False):
    out = []
    for k, (nx, ny, nz) in enumerate(dims):
        bs = (0.3 + 0.05 * k) / (BW if tetra else 1.0)
        w = bs * (BW if tetra else 1.0)
        out.append(Instance(nx, ny, nz, bs, 1e-3 * (1 + 0.1 * k), 20.0 + 5 * k,
                            origin=(-0.5 * nx * w, -0.5 * ny * w + 0.05 * k, -0.5 * nz * w),
                            trap=(1.0, 1.0 + 0.1 * k, 0.8)))
    return out


def _pinned(shape, dtype):
    import torch
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    blk = torch.empty(n + 64, dtype=torch.uint8, pin_memory=True)
    return blk.numpy()[:n].view(dtype).reshape(shape), blk


def _fields(st, seed, pinned):
    keep, pairs = [], []
    for i in range(len(st.instances)):
        shp = st.shape(i)
        pair = []
        for f in range(2):
            z = random_state(shp, seed + 10 * i + f, 0.3)
            a = np.stack([z.real, z.imag], -1).astype(st.field_dtype)
            if pinned:
                p, blk = _pinned(a.shape, st.field_dtype)
                p[...] = a
                keep.append(blk)
                a = p
            pair.append(a)
        pairs.append(tuple(pair))
    return pairs, keep


def _potentials(st, seed):
    rng = np.random.default_rng(seed)
    vdt = np.float64 if st.precision == Precision.FP64 else np.float32
    return [rng.uniform(0.0, 5.0, st.shape(i)).astype(vdt) for i in range(len(st.instances))]


def _sequential(st, pairs, steps, V=None):
    n = len(st.instances)
    st.upload_many([(i, pairs[i][0], pairs[i][1], V[i] if V else None) for i in range(n)])
    st.step(steps)
    obs = st.observables(0)
    return st.download_many(range(n)), obs


def _compare(got, want):
    (g_out, g_obs), (w_out, w_obs) = got, want
    for i, ((ge, go), (we, wo)) in enumerate(zip(g_out, w_out)):
        np.testing.assert_array_equal(ge, we, err_msg=f"even field, instance {i}")
        np.testing.assert_array_equal(go, wo, err_msg=f"odd field, instance {i}")
    for i, (a, b) in enumerate(zip(g_obs, w_obs)):
        for k in ("norm", "energy", "mu", "kinetic", "potential", "interaction"):
            assert a[k] == b[k], (i, k)


def _step_launches(lattice, kernel, tile, groups, steps):
    """(fewest, most) step launches of one round trip; None where not fixed
    (plain kernels).  Groups that step at the same time share launches: at
    least steps + groups - 1 rounds of two half-step launches, at most one
    group per round."""
    if kernel != Kernel.FUSED:
        return None
    kind = variants()[tile]["kind"] if lattice == Lattice.BCC2 else 0
    if kind == 2:      # persistent: one launch per call
        return 1, 1
    if kind == 1:      # two-step: one launch per step
        return steps, steps
    return 2 * (steps + groups - 1), 2 * steps * groups


# (lattice, precision, host precision, potential, kernel, tile, groups expected)
CASES = [
    (Lattice.BCC2, Precision.FP32, None, Potential.TRAP, Kernel.FUSED, 0, 4),
    (Lattice.BCC2, Precision.FP32C, Precision.FP32, Potential.ARRAY, Kernel.FUSED, 3, 4),
    (Lattice.BCC2, Precision.FP32C, None, Potential.TRAP, Kernel.FUSED, 0, 4),
    (Lattice.BCC2, Precision.FP64, None, Potential.ARRAY, Kernel.FUSED, 0, 4),
    (Lattice.TETRA12, Precision.FP32, None, Potential.ARRAY, Kernel.FUSED, 0, 4),
    (Lattice.BCC2, Precision.FP64, None, Potential.TRAP, Kernel.PLAIN, 0, 1),
    (Lattice.BCC2, Precision.FP32, None, Potential.TRAP, Kernel.FUSED, 13, 1),   # a two-step variant
    (Lattice.BCC2, Precision.FP32C, None, Potential.TRAP, Kernel.FUSED, 20, 1),  # a persistent variant
    (Lattice.TETRA12, Precision.FP64, None, Potential.TRAP, Kernel.PLAIN, 0, 1),
]


@pytest.mark.parametrize("lattice,prec,host,potential,kernel,tile,groups", CASES)
def test_round_trip_equals_calls_in_sequence(lattice, prec, host, potential, kernel, tile, groups):
    tetra = lattice == Lattice.TETRA12
    insts = _insts(DIMS, tetra)
    kw = dict(lattice=lattice, precision=prec, potential=potential, kernel=kernel, tile=tile, graph_steps=-1)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    if host is not None:
        a.set_host_precision(host)
        b.set_host_precision(host)
    pairs, keep = _fields(a, 3, pinned=True)
    V = _potentials(a, 9) if potential == Potential.ARRAY else None
    steps = 5
    want = _sequential(a, pairs, steps, V)
    if V:  # the potential stays resident; the round trip moves fields only
        b.upload_many([(i, pairs[i][0], pairs[i][1], V[i]) for i in range(len(insts))])
    n0 = b.launch_count()
    got = b.round_trip(pairs, steps)
    bounds = _step_launches(lattice, kernel, tile, groups, steps)
    if bounds is not None:
        # one conversion launch per group each way, 2 observables launches, the step launches
        stepping = b.launch_count() - n0 - 2 * groups - 2
        assert bounds[0] <= stepping <= bounds[1], (stepping, bounds)
    _compare(got, want)
    a.close()
    b.close()


def test_round_trip_with_graphs_in_place_and_after():
    """Per-group graphs (steps above graph_steps, with a remainder), outputs
    written into the input buffers, a second round trip reusing the graphs, and a
    plain gpe_step afterwards covering every instance again."""
    insts = _insts(DIMS)
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32C, potential=Potential.TRAP, kernel=Kernel.FUSED,
              graph_steps=7)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    a.set_host_precision(Precision.FP32)
    b.set_host_precision(Precision.FP32)
    pairs, keep = _fields(a, 11, pinned=True)
    copies = [(e.copy(), o.copy()) for e, o in pairs]
    want = _sequential(a, copies, 17)
    got = b.round_trip(pairs, 17, outs=pairs)
    _compare(got, want)
    want2 = _sequential(a, [(e.copy(), o.copy()) for e, o in want[0]], 9)
    got2 = b.round_trip(pairs, 9, outs=pairs)
    _compare(got2, want2)
    a.step(3)
    b.step(3)
    for i in range(len(insts)):
        ae, ao = a.download(i)
        be, bo = b.download(i)
        np.testing.assert_array_equal(be, ae)
        np.testing.assert_array_equal(bo, ao)
    a.close()
    b.close()


def test_round_trip_pageable_buffers_and_partial_outputs():
    """Pageable host arrays give the same fields; output entries left out are
    not downloaded; without observables none are returned."""
    insts = _insts(DIMS[:3])
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32, potential=Potential.TRAP, kernel=Kernel.FUSED,
              graph_steps=-1)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    pairs, _ = _fields(a, 21, pinned=False)
    (w_out, _) = _sequential(a, pairs, 4)
    outs = [(np.full(a.shape(i) + (2,), 7.0, np.float32), None if i == 1 else np.empty(a.shape(i) + (2,), np.float32))
            for i in range(len(insts))]
    outs[2] = (None, outs[2][1])
    got, obs = b.round_trip(pairs, 4, outs=outs, observables=False)
    assert obs is None
    np.testing.assert_array_equal(got[0][0], w_out[0][0])
    np.testing.assert_array_equal(got[0][1], w_out[0][1])
    np.testing.assert_array_equal(got[1][0], w_out[1][0])
    np.testing.assert_array_equal(got[2][1], w_out[2][1])
    a.close()
    b.close()


def test_round_trip_imaginary_time_equals_calls_in_sequence():
    insts = _insts(DIMS[:4])
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32, potential=Potential.TRAP, kernel=Kernel.FUSED,
              mode=Mode.IMAGINARY, graph_steps=10)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    pairs, keep = _fields(a, 31, pinned=True)
    psis = [(e, None) for e, _ in pairs]
    n = len(insts)
    a.upload_many([(i, psis[i][0], None, None) for i in range(n)])
    a.step(25)
    w_obs = a.observables(0)
    w_out = a.download_many(range(n), odd=False)
    outs = [(np.empty(a.shape(i) + (2,), np.float32), None) for i in range(n)]
    got, obs = b.round_trip(psis, 25, outs=outs)
    _compare((got, obs), ([(e, None) for e, _ in w_out], w_obs))
    a.close()
    b.close()


def test_round_trip_reports_a_timeout_and_the_handle_recovers():
    insts = _insts(DIMS[2:4])
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32, potential=Potential.TRAP, kernel=Kernel.FUSED,
              graph_steps=-1)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    pairs, keep = _fields(a, 41, pinned=True)
    b.debug_inject(3)
    with pytest.raises(GpeError) as err:
        b.round_trip(pairs, 1)
    assert err.value.status == Status.TIMEOUT
    b.debug_inject(-1)
    want = _sequential(a, pairs, 2)
    _compare(b.round_trip(pairs, 2), want)
    a.close()
    b.close()


def test_round_trip_argument_checks():
    insts = _insts(DIMS[:2])
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32, potential=Potential.TRAP,
                 kernel=Kernel.FUSED)
    pairs, _ = _fields(st, 1, pinned=False)
    with pytest.raises(GpeError) as err:
        st.round_trip(pairs, -1)
    assert err.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as err:
        st.round_trip([(pairs[0][0], None), pairs[1]], 1)  # real time needs the odd field
    assert err.value.status == Status.INVALID_ARGUMENT
    st.close()
