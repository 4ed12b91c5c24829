"""The face (Hodge) form of the update, as the reference's multi-GPU program
computes it (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi.cu:329-397):
sum_f h_f (psi_f - psi) over each value's four faces, in that kernel's face
order, with one Hodge weight per face from its own table
(tests/golden/ref_multi_tables.json, printed by its getLaplacian).

CPU: the table checks of gpe_create, and the oracle's face form against the
lattice form it equals algebraically.  GPU: bit for bit against the reference's
own kernel (built from its source) and against the oracle, FP64 and FP32, array
and trap potentials, batches; imaginary time and observables."""
import numpy as np
import pytest

import oracle.oracle as orc
from oracle.lattice import tables
from conftest import golden
from helpers import random_state, rel_l2, vdt_for
from vaikkari_gb300.gpe import (GpeError, Instance, Kernel, Lattice, Mode, Potential, Precision, Stepper,
                                default_face_table, lattice_info)

TABLE = [tuple(r) for r in golden("ref_multi_tables.json")["faces"]]


def _insts(dims, bs=0.4, dt=2e-3, g=40.0):
    return [Instance(nx, ny, nz, bs + 0.03 * k, dt, g + 5 * k, origin=(-1.0, -0.8, -0.6), trap=(1.0, 1.3, 0.7))
            for k, (nx, ny, nz) in enumerate(dims)]


def _fields(shape, seed, dtype):
    e = random_state(shape, seed, 0.3)
    o = random_state(shape, seed + 100, 0.3)
    cast = lambda a: np.ascontiguousarray(np.stack([a.real, a.imag], -1).astype(dtype))
    return cast(e), cast(o)


def test_reference_table_is_the_tetra12_graph():
    """Every slot's four faces in the reference's table are the library's four
    TETRA12 neighbours; the weights are the Mesh library's 1.5 to rounding."""
    info = lattice_info(Lattice.TETRA12)
    for s in range(12):
        ours = sorted(tuple(int(v) for v in info["entry"][s][k][:4]) for k in range(4))
        ref = sorted(tuple(int(v) for v in r[:4]) for r in TABLE[4 * s:4 * s + 4])
        assert ours == ref, s
    assert all(abs(r[4] - 1.5) < 1e-14 for r in TABLE)


def test_create_rejects_bad_face_tables():
    """gpe_create checks the table before touching the GPU."""
    insts = _insts([(4, 3, 2)])
    bad = list(TABLE)
    bad[5] = (1, 1, 1, 5, 1.5)                                        # not a neighbour of slot 1
    with pytest.raises(GpeError):
        Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP64, faces=bad)
    dup = list(TABLE)
    dup[1] = dup[0]                                                   # one neighbour twice
    with pytest.raises(GpeError):
        Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP64, faces=dup)
    nan = list(TABLE)
    nan[7] = (*nan[7][:4], float("nan"))
    with pytest.raises(GpeError):
        Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP64, faces=nan)
    with pytest.raises(GpeError):                                     # BCC2 has no face form
        Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP64, faces=TABLE)
    with pytest.raises(ValueError):
        Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP64, faces=TABLE[:47])


def test_face_oracle_equals_lattice_form_to_rounding():
    """With every weight 1.5 the face form is the lattice form of
    GPUGrossPitaevskii_BCC.cu:213 rearranged: after 20 steps the two oracles
    agree to rounding."""
    info = tables(Lattice.TETRA12)
    nx, ny, nz, bs, dt, g = 6, 5, 4, 0.35, 1e-3, 60.0
    e, o = _fields((nz, ny, nx, 12), 3, np.float64)
    V = np.random.default_rng(4).uniform(0, 2, (nz, ny, nx, 12))
    vdt = np.ascontiguousarray(V * dt)
    fo = orc.Faces(nx, ny, nz, default_face_table(), bs, dt, g)
    gl = orc.Grid(nx, ny, nz, info["entry"], info["class_weight"], bs, dt, g)
    e1, o1, e2, o2 = e.copy(), o.copy(), e.copy(), o.copy()
    fo.leapfrog(e1, o1, vdt, 20)
    gl.leapfrog(e2, o2, vdt, 20)
    assert rel_l2(e1, e2) < 1e-13 and rel_l2(o1, o2) < 1e-13
    assert not np.array_equal(e1, e2)   # a different order of operations


def _run_faces(prec, potential, dims, steps, table=TABLE, kernel=Kernel.PLAIN, tile=0):
    T = np.float64 if prec == Precision.FP64 else np.float32
    insts = _insts(dims)
    st = Stepper(insts, lattice=Lattice.TETRA12, precision=prec, kernel=kernel, potential=potential,
                 faces=table, tile=tile)
    want = []
    for i in range(len(insts)):
        shp = st.shape(i)
        e, o = _fields(shp, 10 + i, T)
        V = np.random.default_rng(20 + i).uniform(0, 3, shp) if potential == Potential.ARRAY else None
        st.upload(i, e, o, V)
        fo = orc.Faces(insts[i].nx, insts[i].ny, insts[i].nz, table, insts[i].block_scale, insts[i].dt, insts[i].g)
        vdt = vdt_for(st, i, V)
        fo.leapfrog(e, o, vdt, steps)
        want.append((e, o))
    st.step(steps)
    got = [st.download(i) for i in range(len(insts))]
    st.close()
    return got, want


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
@pytest.mark.parametrize("potential", [Potential.ARRAY, Potential.TRAP])
def test_faces_bit_exact_oracle(prec, potential):
    """A ragged batch (one launch per half-step) equals the oracle's face form
    bit for bit."""
    got, want = _run_faces(prec, potential, [(1, 1, 1), (7, 5, 3), (33, 9, 6)], 5)
    for i, ((ge, go), (we, wo)) in enumerate(zip(got, want)):
        np.testing.assert_array_equal(ge, we, err_msg=f"even, instance {i}")
        np.testing.assert_array_equal(go, wo, err_msg=f"odd, instance {i}")


@pytest.mark.gpu
@pytest.mark.parametrize("potential", [Potential.ARRAY, Potential.TRAP])
@pytest.mark.parametrize("tile", [0, 3])
def test_fused_face_form_bit_exact_oracle(tile, potential):
    """FP32: the fused TETRA12 kernel in the face form (faces and weights from the
    handle, one fma per face) equals the oracle's face form bit for bit."""
    got, want = _run_faces(Precision.FP32, potential, [(1, 1, 1), (7, 5, 3), (33, 9, 6), (40, 4, 9)], 5,
                           kernel=Kernel.FUSED, tile=tile)
    for i, ((ge, go), (we, wo)) in enumerate(zip(got, want)):
        np.testing.assert_array_equal(ge, we, err_msg=f"even, instance {i}")
        np.testing.assert_array_equal(go, wo, err_msg=f"odd, instance {i}")


@pytest.mark.gpu
def test_fused_face_form_imaginary_time_follows_plain():
    """FP32 imaginary time in the face form: the fused kernel (sums fused into the
    step) and the plain kernel end within FP32 rounding of each other."""
    insts = [Instance(10, 10, 10, 0.5, 2e-3, 30.0, origin=(-7.1, -7.1, -7.1), trap=(1.0, 1.0, 1.0))]
    rng = np.random.default_rng(19)
    psi0 = np.exp(1j * rng.uniform(0, 2 * np.pi, size=(10, 10, 10, 12)))
    out = []
    for kern in (Kernel.FUSED, Kernel.PLAIN):
        st = Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP32, kernel=kern, mode=Mode.IMAGINARY,
                     potential=Potential.TRAP, faces=TABLE, graph_steps=20)
        st.upload(0, psi0)
        steps, conv, mu = st.imaginary_time(120, 0.0)
        out.append((mu[0], st.download(0, odd=False)[0]))
        st.close()
    assert out[0][0] == pytest.approx(out[1][0], rel=1e-6)
    assert rel_l2(out[0][1], out[1][1]) < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(21, 6, 5), (16, 3, 4), (40, 7, 3)])
def test_faces_equal_reference_multi_kernel(dims):
    """FP64, the reference's own table: the library's face form, the reference's
    multi-GPU update kernel (built from its source for sm_103a) and the oracle
    agree bit for bit after 6 leapfrog steps."""
    import refkernel
    if not refkernel.multi_available():
        pytest.skip("oracle/_ref/ref_multi.cubin is built where the reference source is present")
    X, Y, Z = dims
    bs, dt, g = 0.45, 1.5e-3, 80.0
    st = Stepper([Instance(X, Y, Z, bs, dt, g)], lattice=Lattice.TETRA12, precision=Precision.FP64,
                 kernel=Kernel.PLAIN, potential=Potential.ARRAY, faces=TABLE)
    shp = st.shape(0)
    e, o = _fields(shp, 5, np.float64)
    V = np.random.default_rng(6).uniform(0, 4, shp)
    st.upload(0, e, o, V)
    st.step(6)
    ge, go = st.download(0)
    st.close()
    rk = refkernel.ReferenceHodgeUpdate(X, Y, Z)
    rk.upload(e, o, V * dt)
    rk.step_faces(6, TABLE, bs, dt, g)
    re, ro = rk.download()
    np.testing.assert_array_equal(ge, re)
    np.testing.assert_array_equal(go, ro)
    fo = orc.Faces(X, Y, Z, TABLE, bs, dt, g)
    fo.leapfrog(e, o, np.ascontiguousarray(V * dt), 6)
    np.testing.assert_array_equal(ge, e)
    np.testing.assert_array_equal(go, o)


@pytest.mark.gpu
def test_faces_observables_and_imaginary_time():
    """The observables of a face-form handle use its face weights: with every
    weight 1.5 they equal the lattice form's to rounding.  Imaginary time in the
    face form follows the lattice form's to rounding."""
    insts = [Instance(10, 10, 10, 0.5, 2e-3, 30.0, origin=(-7.1, -7.1, -7.1), trap=(1.0, 1.0, 1.0))]
    kw = dict(lattice=Lattice.TETRA12, precision=Precision.FP64, kernel=Kernel.PLAIN, potential=Potential.TRAP)
    a = Stepper(insts, faces=default_face_table(), **kw)
    b = Stepper(insts, **kw)
    e, o = _fields(a.shape(0), 8, np.float64)
    for st in (a, b):
        st.upload(0, e, o, None)
    oa, ob = a.observables()[0], b.observables()[0]
    for k in ("norm", "kinetic", "potential", "interaction", "energy", "mu"):
        assert abs(oa[k] - ob[k]) <= 1e-12 * abs(ob[k]), k
    a.close()
    b.close()
    rng = np.random.default_rng(9)
    psi0 = np.exp(1j * rng.uniform(0, 2 * np.pi, size=a.shape(0)))
    out = []
    for faces in (default_face_table(), None):
        st = Stepper(insts, mode=Mode.IMAGINARY, faces=faces, graph_steps=20, **kw)
        st.upload(0, psi0)
        steps, conv, mu = st.imaginary_time(200, 0.0)
        out.append((mu[0], st.download(0, odd=False)[0]))
        st.close()
    assert abs(out[0][0] - out[1][0]) <= 1e-11 * abs(out[1][0])
    assert rel_l2(out[0][1], out[1][1]) < 1e-11


@pytest.mark.gpu
def test_faces_slabs_equal_undivided_grid():
    """The multi-GPU program splits one grid into z-slabs; the face form over 3
    linked slabs of one batch equals the undivided grid bit for bit."""
    from vaikkari_gb300.slabs import SlabStepper
    dims = (12, 10, 11)
    inst = Instance(*dims, 0.25, 1e-3, 40.0, origin=(-5.0, -3.0, -3.5))
    kw = dict(lattice=Lattice.TETRA12, precision=Precision.FP64, kernel=Kernel.PLAIN, potential=Potential.ARRAY,
              faces=TABLE)
    shp = (dims[2], dims[1], dims[0], 12)
    e, o = _fields(shp, 31, np.float64)
    V = np.random.default_rng(32).uniform(0, 3, shp)
    whole = Stepper([inst], **kw)
    whole.upload(0, e, o, V)
    whole.step(130)
    we, wo = whole.download(0)
    whole.close()
    sl = SlabStepper(inst, 3, **kw)
    sl.upload(e, o, V)
    sl.step(130)
    se, so = sl.download()
    sl.close()
    assert np.abs(we).max() > 0.05
    np.testing.assert_array_equal(se, we)
    np.testing.assert_array_equal(so, wo)


@pytest.mark.gpu
def test_face_form_fp64_rate_against_the_reference_kernel():
    """FP64 on the production grid (87 x 87 x 302 blocks, 27.4 M values): the
    library's face form and the reference's own multi-GPU update kernel (built
    from its source for sm_103a) timed in the same process, best of three runs
    of 30 leapfrog steps each.  Both are bound by the FP64 pipe; the library
    must keep up with the reference kernel (measured 1.22e10 against 1.19e10
    value-updates/s; the 3% margin absorbs timing noise)."""
    import time
    import refkernel
    if not refkernel.multi_available():
        pytest.skip("oracle/_ref/ref_multi.cubin is built where the reference source is present")
    X, Y, Z, steps = 87, 87, 302, 30
    bs, dt, g = 0.06997, 1e-4, 100.0
    rng = np.random.default_rng(5)
    shp = (Z, Y, X, 12)
    e = np.ascontiguousarray(np.stack([rng.standard_normal(shp), rng.standard_normal(shp)], -1) * 0.3)
    o = np.ascontiguousarray(np.stack([rng.standard_normal(shp), rng.standard_normal(shp)], -1) * 0.3)
    V = rng.uniform(0.0, 10.0, shp)
    values = X * Y * Z * 12
    st = Stepper([Instance(X, Y, Z, bs, dt, g)], lattice=Lattice.TETRA12, precision=Precision.FP64,
                 kernel=Kernel.PLAIN, potential=Potential.ARRAY, graph_steps=-1, faces=TABLE)
    st.upload(0, e, o, V)
    st.step(2)
    st.synchronize()
    ours = values * steps / (min(st.time_steps(steps) for _ in range(3)) * 1e-3)
    st.close()
    rk = refkernel.ReferenceHodgeUpdate(X, Y, Z)
    rk.upload(e, o, V * dt)
    rk.step_faces(2, TABLE, bs, dt, g)
    best = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        rk.step_faces(steps, TABLE, bs, dt, g)   # launches, then synchronises the context
        best = min(best, time.perf_counter() - t0)
    ref = values * steps / best
    print(f"face form FP64: library {ours:.4g}, reference kernel {ref:.4g} value-updates/s ({ours / ref:.3f}x)")
    assert ours >= 0.97 * ref, (ours, ref)
