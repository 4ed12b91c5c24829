"""The fused TETRA12 half-step (FP32): in real time bit for bit the plain kernel
and the oracle (the reference's update and neighbour order), for every variant,
both potential forms, ragged sizes, batches, graphs with remainders and short
z-chunks; in imaginary time (sums fused into the step) within FP32 rounding of
the FP64 oracle and of the plain kernel; a withheld copy ends in GPE_ERR_TIMEOUT
with the context intact; the forms it does not cover are refused."""
import numpy as np
import pytest

from helpers import grid_for, interleave, random_state, rel_l2, vdt_for, vol_for
from vaikkari_gb300.gpe import GpeError, Instance, Kernel, Lattice, Mode, Potential, Precision, Status, Stepper

pytestmark = pytest.mark.gpu

SIZES = [(1, 1, 1), (3, 5, 7), (33, 17, 5), (40, 9, 20), (70, 3, 4)]
BW = 8 ** 0.5


def _insts(dims_list):
    out = []
    for k, (nx, ny, nz) in enumerate(dims_list):
        bs = (0.3 + 0.05 * k) / BW
        origin = tuple(-0.5 * n * bs * BW + 0.1 * k for n in (nx, ny, nz))
        out.append(Instance(nx, ny, nz, block_scale=bs, dt=1e-3 * (1 + 0.2 * k), g=50.0 + 10 * k, origin=origin,
                            trap=(1.0, 1.5 + 0.1 * k, 0.7)))
    return out


def _fields(st, insts, seed, potential):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(len(insts)):
        shp = st.shape(i)
        e, o = random_state(shp, seed + 10 * i, 0.3), random_state(shp, seed + 10 * i + 1, 0.3)
        V = rng.uniform(0.0, 10.0, size=shp) if potential == Potential.ARRAY else None
        out.append((e, o, V))
    return out


@pytest.mark.parametrize("potential", [Potential.TRAP, Potential.ARRAY])
@pytest.mark.parametrize("tile", [0, 1, 2, 3, 4, 5])
def test_t12_fused_equals_oracle_and_plain(tile, potential):
    insts = _insts(SIZES)
    kw = dict(lattice=Lattice.TETRA12, precision=Precision.FP32, potential=potential, graph_steps=-1)
    fu = Stepper(insts, kernel=Kernel.FUSED, tile=tile, **kw)
    pl = Stepper(insts, kernel=Kernel.PLAIN, **kw)
    fields = _fields(fu, insts, 7, potential)
    steps = 4
    for i, (e, o, V) in enumerate(fields):
        fu.upload(i, e, o, V)
        pl.upload(i, e, o, V)
    fu.step(steps)
    pl.step(steps)
    for i, (e, o, V) in enumerate(fields):
        g = grid_for(fu, i)
        we, wo = interleave(e, np.float32), interleave(o, np.float32)
        g.leapfrog(we, wo, vdt_for(fu, i, V), steps)
        ge, go = fu.download(i)
        pe, po = pl.download(i)
        np.testing.assert_array_equal(ge, we, err_msg=f"even vs oracle, instance {i}")
        np.testing.assert_array_equal(go, wo, err_msg=f"odd vs oracle, instance {i}")
        np.testing.assert_array_equal(ge, pe)
        np.testing.assert_array_equal(go, po)
    fu.close()
    pl.close()


def test_t12_fused_graphs_and_short_chunks_equal_plain():
    """Graphs of 7 steps with a remainder, and z-chunks of 3 planes (items whose
    halo planes are their neighbours' outputs)."""
    insts = _insts([(33, 17, 11), (9, 40, 7)])
    kw = dict(lattice=Lattice.TETRA12, precision=Precision.FP32, potential=Potential.TRAP)
    fu = Stepper(insts, kernel=Kernel.FUSED, graph_steps=7, zchunk=3, **kw)
    pl = Stepper(insts, kernel=Kernel.PLAIN, graph_steps=-1, **kw)
    for i, (e, o, _) in enumerate(_fields(fu, insts, 3, Potential.TRAP)):
        fu.upload(i, e, o)
        pl.upload(i, e, o)
    fu.step(17)
    pl.step(17)
    for i in range(len(insts)):
        ge, go = fu.download(i)
        pe, po = pl.download(i)
        np.testing.assert_array_equal(ge, pe)
        np.testing.assert_array_equal(go, po)
    fu.close()
    pl.close()


def test_t12_fused_timeout_is_reported_and_context_survives():
    insts = _insts([(8, 8, 8)])
    st = Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP32, kernel=Kernel.FUSED,
                 potential=Potential.TRAP, graph_steps=-1)
    (e, o, _), = _fields(st, insts, 1, Potential.TRAP)
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
    g = grid_for(st, 0)
    we, wo = interleave(e, np.float32), interleave(o, np.float32)
    g.leapfrog(we, wo, vdt_for(st, 0), 3)
    st.close()
    np.testing.assert_array_equal(ge, we)
    np.testing.assert_array_equal(go, wo)


@pytest.mark.parametrize("potential", [Potential.TRAP, Potential.ARRAY])
@pytest.mark.parametrize("tile", [0, 3])
def test_t12_fused_imaginary_time_matches_oracle_and_plain(tile, potential):
    """80 normalised imaginary-time steps of two condensates in one batch: the
    fields within 2e-6 (relative L2) of the FP64 oracle, and the reported mu (the
    FP64 observables of the final normalised field, for FP32 handles) within 1e-6
    of the oracle's observables of its own final field; the plain kernel's FP32 run
    within the same distances."""
    insts = [Instance(10, 9, 8, 0.45 / BW, 2e-3, 40.0, origin=(-2.25, -2.0, -1.8), trap=(1.0, 1.0, 4.0)),
             Instance(35, 6, 13, 0.4 / BW, 1e-3, 10.0, origin=(-7.0, -1.2, -2.6))]
    rng = np.random.default_rng(11)
    psis = [np.exp(1j * rng.uniform(0, 2 * np.pi, size=(i.nz, i.ny, i.nx, 12))) for i in insts]
    Vs = [rng.uniform(0.0, 5.0, size=(i.nz, i.ny, i.nx, 12)) for i in insts]
    runs = {}
    for kern in (Kernel.FUSED, Kernel.PLAIN):
        st = Stepper(insts, lattice=Lattice.TETRA12, precision=Precision.FP32, mode=Mode.IMAGINARY, kernel=kern,
                     potential=potential, graph_steps=20, tile=tile if kern == Kernel.FUSED else 0, zchunk=4)
        for i, p in enumerate(psis):
            st.upload(i, p, None, Vs[i] if potential == Potential.ARRAY else None)
        steps, conv, mu = st.imaginary_time(80, 0.0)
        assert steps == 80 and not conv
        runs[kern] = ([st.download(i, odd=False)[0] for i in range(len(insts))], mu,
                      [(grid_for(st, i), vdt_for(st, i, Vs[i] if potential == Potential.ARRAY else None),
                        vol_for(st, i)) for i in range(len(insts))])
        st.close()
    fused, mu_f, geo = runs[Kernel.FUSED]
    plain, mu_p, _ = runs[Kernel.PLAIN]
    for i, p in enumerate(psis):
        g, vdt, vol = geo[i]
        psi = interleave(p, np.float64)
        v64 = vdt.astype(np.float64)
        g.imaginary(psi, v64, vol, 80, 0.0)
        mu_ref = g.observables(psi, v64, vol)["mu"]
        assert rel_l2(fused[i], psi) < 2e-6
        assert rel_l2(plain[i], psi) < 2e-6
        assert mu_f[i] == pytest.approx(mu_ref, rel=1e-6)
        assert mu_p[i] == pytest.approx(mu_ref, rel=1e-6)


@pytest.mark.parametrize("prec,mode", [(Precision.FP64, Mode.REAL), (Precision.FP64, Mode.IMAGINARY)])
def test_t12_fused_refuses_what_it_does_not_cover(prec, mode):
    with pytest.raises(GpeError) as err:
        Stepper(_insts([(4, 4, 4)]), lattice=Lattice.TETRA12, precision=prec, kernel=Kernel.FUSED, mode=mode,
                potential=Potential.TRAP)
    assert err.value.status == Status.UNSUPPORTED
