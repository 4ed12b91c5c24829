"""Compensated FP32 storage (Precision.FP32C): FP32 fields and arithmetic, with an
int8 residual per component, in units of ulp(value)/256, carried from step to
step, so the leapfrog's accumulation of the stored values keeps about 8 bits
more than FP32 at 16 bits per value.

CPU: the residual code against a candidate-by-candidate reference (nearest
multiple of the unit, ties to even, clipped to +-127), the float64 <-> (FP32,
int8) split and join, and the oracle's compensated leapfrog against FP64 of the
same scheme (much closer than plain FP32).  GPU: the fused kernel's compensated
mode equals the oracle bit for bit (values and residuals, through the float64
download), refuses the set-ups it does not cover, and keeps a strongly
interacting condensate of the 64-instance batch within 1e-5 of FP64 after 1000
steps where plain FP32 is above 1e-4; the whole batch, run twice, gives
identical results in FP32 and FP32C."""
import numpy as np
import pytest

import oracle.oracle as orc
from helpers import grid_for, interleave, random_state, rel_l2, vdt_for
from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Mode, Potential, Precision, Stepper


def _unit_reference(hi):
    """ulp(hi)/256 from frexp, with the floor 2^-126 for tiny values."""
    m, e = np.frexp(np.asarray(hi, np.float32).astype(np.float64))   # |hi| = m 2^e, m in [0.5, 1)
    unit = np.ldexp(1.0, (e - 1) - 23 - 8)
    return np.where((hi == 0) | (unit < 2.0 ** -126), 2.0 ** -126, unit)


def _encode_reference(r, hi):
    """The nearest multiple of the unit, candidate by candidate: floor and
    floor + 1, the nearer (ties to the even one), clipped to +-127."""
    u = _unit_reference(hi)
    x = np.asarray(r, np.float32).astype(np.float64) / u
    f = np.floor(x)
    d0, d1 = x - f, f + 1 - x
    pick = (d1 < d0) | ((d1 == d0) & (np.mod(f, 2) == 1))
    return np.clip(np.where(pick, f + 1, f), -127, 127).astype(np.int8)


def test_residual_code_matches_nearest_even_multiple_of_the_unit():
    rng = np.random.default_rng(0)
    hi = (rng.standard_normal(200000) * 10.0 ** rng.uniform(-40, 30, 200000)).astype(np.float32)
    hi[:50] = 0.0
    # residuals up to half an ulp of hi, as a two-sum leaves them, plus exact ties
    r = (rng.uniform(-0.5, 0.5, hi.size) * _unit_reference(hi) * 256).astype(np.float32)
    np.testing.assert_array_equal(orc.comp_encode(r, hi), _encode_reference(r, hi))
    ones = np.ones(4, np.float32)
    u = float(orc.comp_unit(ones)[0])
    assert u == 2.0 ** -31                                                        # ulp(1) / 256
    ties = np.array([0.5, 1.5, 2.5, -2.5], np.float32) * np.float32(u)
    np.testing.assert_array_equal(orc.comp_encode(ties, ones), [0, 2, 2, -2])     # ties to even
    np.testing.assert_array_equal(orc.comp_encode(np.float32(128 * u) * ones[:1], ones[:1]), [127])  # clipped
    assert orc.comp_unit(np.float32(1e-35)) == np.float32(2.0 ** -126)           # the floor


def test_split_join_keeps_32_bits():
    rng = np.random.default_rng(1)
    x = rng.standard_normal(100000) * 10.0 ** rng.uniform(-20, 20, 100000)
    hi, lo = orc.split_comp(x)
    assert hi.dtype == np.float32 and lo.dtype == np.int8
    back = orc.join_comp(hi, lo)
    # half a unit (2^-32 relative) but where a residual of half an ulp is
    # clipped from 128 to 127 units: one unit, 2^-31
    assert np.all(np.abs(back - x) <= 2.0 ** -31 * np.abs(x))
    assert np.mean(np.abs(back - x) <= 2.0 ** -32 * np.abs(x)) > 0.99
    assert np.all(np.abs(hi.astype(np.float64) - x) <= 2.0 ** -24 * np.abs(x))
    np.testing.assert_array_equal(orc.join_comp(*orc.split_comp(back)), back)   # idempotent


def _gaussian_case(n=16, g=2000.0, dt=1e-4):
    from vaikkari_gb300 import workloads
    from oracle.lattice import tables
    from vaikkari_gb300.gpe import value_positions
    info = tables(Lattice.BCC2)
    inst = workloads.bcc2_instance(n, dt, g, trap=(1.0, 2.0, 0.7))
    rng = np.random.default_rng(4)
    psi = workloads.gaussian_state(inst, info, rng, 1e-3)
    V = workloads.harmonic(value_positions(inst, info), inst.trap)
    grid = orc.Grid(n, n, n, info["entry"], info["class_weight"], inst.block_scale, dt, g)
    vol = info["cell_volume"] * inst.block_scale ** 3
    vdt64 = np.ascontiguousarray(V * dt)
    mu = grid.observables(interleave(psi, np.float64), vdt64, vol)["mu"]
    odd = workloads.odd_from_even(psi, mu, dt)
    return inst, grid, psi, odd, V, vdt64


def test_compensated_oracle_closer_to_fp64():
    """Same scheme, 300 steps on a strongly interacting 16^3 condensate: the
    compensated FP32 run is several times closer to FP64 than plain FP32."""
    inst, grid, psi, odd, V, vdt64 = _gaussian_case()
    e64, o64 = interleave(psi, np.float64), interleave(odd, np.float64)
    vdt32 = vdt64.astype(np.float32)
    e32, o32 = e64.astype(np.float32), o64.astype(np.float32)
    eh, el = orc.split_comp(e64)
    oh, ol = orc.split_comp(o64)
    grid.leapfrog_bcc2(e64, o64, vdt64, 300)
    grid.leapfrog_bcc2(e32, o32, vdt32, 300)
    grid.leapfrog_bcc2_comp(eh, oh, el, ol, vdt32, 300)
    err32 = rel_l2(e32.astype(np.float64), e64)
    errc = rel_l2(orc.join_comp(eh, el), e64)
    assert errc < 1e-6 and errc * 4 < err32, (errc, err32)


# ---------------------------------------------------------------- GPU ---------

SIZES = [(1, 1, 1), (3, 5, 7), (13, 7, 9), (40, 9, 20), (33, 17, 5)]


def _run_comp(potential, dims_list, steps, tile=0, graph_steps=-1, seed=0, zchunk=0):
    rng = np.random.default_rng(seed)
    insts = []
    for k, (nx, ny, nz) in enumerate(dims_list):
        bs = 0.3 + 0.05 * k
        origin = tuple(-0.5 * n * bs + 0.1 * k for n in (nx, ny, nz))
        insts.append(Instance(nx, ny, nz, block_scale=bs, dt=1e-3 * (1 + 0.2 * k), g=50.0 + 10 * k,
                              origin=origin, trap=(1.0, 1.5 + 0.1 * k, 0.7)))
    st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32C, kernel=Kernel.FUSED,
                 potential=potential, tile=tile, graph_steps=graph_steps, zchunk=zchunk)
    want = []
    for i, inst in enumerate(insts):
        shp = st.shape(i)
        even = random_state(shp, seed + 10 * i, 0.3)
        odd = random_state(shp, seed + 10 * i + 1, 0.3)
        V = rng.uniform(0.0, 10.0, size=shp)
        st.upload(i, even, odd, V if potential == Potential.ARRAY else None)
        g = grid_for(st, i)
        vdt = vdt_for(st, i, V)
        eh, el = orc.split_comp(interleave(even, np.float64))
        oh, ol = orc.split_comp(interleave(odd, np.float64))
        g.leapfrog_bcc2_comp(eh, oh, el, ol, vdt, steps)
        want.append((orc.join_comp(eh, el), orc.join_comp(oh, ol)))
    st.step(steps)
    for i in range(len(insts)):
        ge, go = st.download(i)
        assert ge.dtype == np.float64
        np.testing.assert_array_equal(ge, want[i][0], err_msg=f"even, instance {i}")
        np.testing.assert_array_equal(go, want[i][1], err_msg=f"odd, instance {i}")
    st.close()


@pytest.mark.gpu
@pytest.mark.parametrize("potential", [Potential.TRAP, Potential.ARRAY])
@pytest.mark.parametrize("tile", [0, 5, 6, 7])
def test_fp32c_bit_exact(potential, tile):
    _run_comp(potential, SIZES, steps=4, tile=tile)


@pytest.mark.gpu
def test_fp32c_graphs_and_chunks_bit_exact():
    """CUDA graphs of 7 steps over 23 steps (a remainder), short z-chunks."""
    _run_comp(Potential.TRAP, SIZES, steps=23, graph_steps=7, seed=3, zchunk=3)


@pytest.mark.gpu
def test_fp32c_round_trip_without_steps():
    """Upload then download returns join(split(x)) exactly (no step run)."""
    inst = Instance(9, 6, 5, 0.3, 1e-3, 10.0)
    st = Stepper([inst], lattice=Lattice.BCC2, precision=Precision.FP32C, kernel=Kernel.FUSED,
                 potential=Potential.TRAP)
    shp = st.shape(0)
    e = random_state(shp, 7, 0.3)
    o = random_state(shp, 8, 0.3)
    st.upload(0, e, o)
    ge, go = st.download(0)
    st.close()
    np.testing.assert_array_equal(ge, orc.join_comp(*orc.split_comp(interleave(e, np.float64))))
    np.testing.assert_array_equal(go, orc.join_comp(*orc.split_comp(interleave(o, np.float64))))


@pytest.mark.gpu
def test_fp32c_refuses_what_it_does_not_cover():
    from vaikkari_gb300.gpe import GpeError, variants
    inst = Instance(8, 8, 8, 0.3, 1e-3, 10.0)
    two = [v["tile"] for v in variants() if v["half_steps"] == 2][0]
    for kw in (dict(mode=Mode.IMAGINARY), dict(kernel=Kernel.PLAIN), dict(tile=two),
               dict(lattice=Lattice.TETRA12, kernel=Kernel.AUTO)):
        args = dict(lattice=Lattice.BCC2, precision=Precision.FP32C, kernel=Kernel.FUSED) | kw
        with pytest.raises(GpeError):
            Stepper([inst], **args)


@pytest.mark.gpu
def test_fp32c_strongly_interacting_condensate_within_1e5():
    """Condensate 58 of the 64-instance batch (48^3 cells, g = 4658): after 1000
    steps plain FP32 is about 1.3e-4 from FP64 (its storage rounding grows with
    the dynamics), the compensated mode below 1e-5.  Norm drift vs FP64 <= 1e-6."""
    from vaikkari_gb300 import workloads
    c = workloads.config4()[58]
    assert c.inst.nx == 48 and c.inst.g > 4600
    out = {}
    for prec in (Precision.FP64, Precision.FP32, Precision.FP32C):
        st = Stepper([c.inst], lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED,
                     potential=Potential.TRAP, graph_steps=100)
        st.upload(0, c.psi, c.psi)
        mu = st.observables(0)[0]["mu"]
        odd = workloads.odd_from_even(c.psi, mu, c.inst.dt)
        st.upload(0, c.psi, odd)
        st.step(1000)
        e, _ = st.download(0, odd=False)
        out[prec] = (e.astype(np.float64), st.observables(0)[0]["norm"])
        st.close()
    ref, n64 = out[Precision.FP64]
    err32 = rel_l2(out[Precision.FP32][0], ref)
    errc = rel_l2(out[Precision.FP32C][0], ref)
    assert errc < 1e-5 < err32, (errc, err32)
    assert abs(out[Precision.FP32C][1] - n64) / n64 <= 1e-6


@pytest.mark.gpu
def test_batch_runs_are_identical():
    """The 64-instance batch, 120 steps (a graph of 100 plus 20 launches), run twice:
    identical fields in FP32 and FP32C.  Consecutive launches overlap on the SMs
    under programmatic dependent launch; data a launch reads that an earlier launch
    wrote must not come from a stale L1 line (an earlier form of the residual loads
    failed exactly this)."""
    from vaikkari_gb300 import workloads
    conds = workloads.config4()
    insts = [c.inst for c in conds]

    def run(prec):
        st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=Potential.TRAP,
                     graph_steps=100)
        for k, c in enumerate(conds):
            st.upload(k, c.psi, c.psi)
        st.step(120)
        out = [st.download(k) for k in range(len(insts))]
        st.close()
        return out

    for prec in (Precision.FP32, Precision.FP32C):
        a, b = run(prec), run(prec)
        diff = [i for i in range(len(insts)) if not (np.array_equal(a[i][0], b[i][0]) and
                                                     np.array_equal(a[i][1], b[i][1]))]
        assert not diff, (prec.name, diff)


@pytest.mark.gpu
def test_fp32_host_format_of_compensated_storage():
    """gpe_set_host_precision(GPE_FP32) on a GPE_FP32C handle: float fields in
    (residual zero), float fields out (value + residual rounded once), through
    the single and the batched transfers; equal to the oracle's compensated run
    from the same float start, bit for bit."""
    import oracle.oracle as orc
    from helpers import grid_for, interleave, random_state, vdt_for
    from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper
    insts = [Instance(9, 7, 11, 0.35, 1e-3, 80.0, origin=(-1.5, -1.2, -1.9)),
             Instance(16, 5, 6, 0.3, 1.5e-3, 40.0, origin=(-2.4, -0.8, -0.9))]
    for batched in (False, True):
        st = Stepper(insts, lattice=Lattice.BCC2, precision=Precision.FP32C, kernel=Kernel.FUSED,
                     potential=Potential.TRAP)
        st.set_host_precision(Precision.FP32)
        fields, want = [], []
        for i in range(len(insts)):
            shp = st.shape(i)
            e = interleave(random_state(shp, 90 + i, 0.3), np.float32)
            o = interleave(random_state(shp, 95 + i, 0.3), np.float32)
            fields.append((e, o))
            eh, oh = e.copy(), o.copy()
            el, ol = np.zeros(e.shape, np.int8), np.zeros(o.shape, np.int8)
            grid_for(st, i).leapfrog_bcc2_comp(eh, oh, el, ol, vdt_for(st, i), 5)
            want.append((orc.join_comp(eh, el).astype(np.float32), orc.join_comp(oh, ol).astype(np.float32)))
        if batched:
            st.upload_many([(i, e, o, None) for i, (e, o) in enumerate(fields)])
        else:
            for i, (e, o) in enumerate(fields):
                st.upload(i, e, o)
        st.step(5)
        got = st.download_many(range(len(insts))) if batched else [st.download(i) for i in range(len(insts))]
        st.close()
        for (ge, go), (we, wo) in zip(got, want):
            assert ge.dtype == np.float32
            np.testing.assert_array_equal(ge, we)
            np.testing.assert_array_equal(go, wo)
