"""GPU parity: every kernel path against the CPU oracle on the same seeded
inputs, through the C ABI.

Real-time stepping is bit-exact (the kernels and the oracle perform the same
rounded operations in the same order).  Reductions and imaginary time sum in a
different order and are compared with the tolerances written in each test.
"""
import numpy as np
import pytest

from helpers import grid_for, interleave, random_state, rel_l2, vdt_for, vol_for
from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Mode, Potential, Precision, Stepper

pytestmark = pytest.mark.gpu

SIZES = [(1, 1, 1), (3, 5, 7), (13, 7, 9), (40, 9, 20), (33, 17, 5)]


def _dtype(prec):
    return np.float64 if prec == Precision.FP64 else np.float32


def _run_real(lattice, prec, kernel, potential, dims_list, steps=3, tile=0, graph_steps=-1, seed=0):
    T = _dtype(prec)
    rng = np.random.default_rng(seed)
    insts = []
    bw = 8 ** 0.5 if lattice == Lattice.TETRA12 else 1.0
    for k, (nx, ny, nz) in enumerate(dims_list):
        bs = (0.3 + 0.05 * k) / bw
        # centred grid, moderate trap: dt * (largest eigenvalue of H) stays ~0.1,
        # inside the leapfrog's stability bound
        origin = tuple(-0.5 * n * bs * bw + 0.1 * k for n in (nx, ny, nz))
        insts.append(Instance(nx, ny, nz, block_scale=bs, dt=1e-3 * (1 + 0.2 * k), g=50.0 + 10 * k,
                              origin=origin, trap=(1.0, 1.5 + 0.1 * k, 0.7)))
    st = Stepper(insts, lattice=lattice, precision=prec, kernel=kernel, potential=potential, tile=tile,
                 graph_steps=graph_steps)
    want = []
    for i, inst in enumerate(insts):
        shp = st.shape(i)
        even = random_state(shp, seed + 10 * i, 0.3)
        odd = random_state(shp, seed + 10 * i + 1, 0.3)
        V = rng.uniform(0.0, 10.0, size=shp)
        st.upload(i, even, odd, V if potential == Potential.ARRAY else None)
        g = grid_for(st, i)
        vdt = vdt_for(st, i, V)
        e, o = interleave(even, T), interleave(odd, T)
        if lattice == Lattice.BCC2 and kernel != Kernel.PLAIN:
            g.leapfrog_bcc2(e, o, vdt, steps)   # the fused kernel's summation order
        else:
            g.leapfrog(e, o, vdt, steps)
        want.append((e, o))
    st.step(steps)
    for i in range(len(insts)):
        ge, go = st.download(i)
        we, wo = want[i]
        assert ge.dtype == T
        np.testing.assert_array_equal(ge, we, err_msg=f"even, instance {i}")
        np.testing.assert_array_equal(go, wo, err_msg=f"odd, instance {i}")
    n = st.launch_count()
    st.close()
    return n


@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
@pytest.mark.parametrize("dims", SIZES)
def test_plain_tetra12_bit_exact(prec, dims):
    _run_real(Lattice.TETRA12, prec, Kernel.PLAIN, Potential.ARRAY, [dims])


@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
@pytest.mark.parametrize("kernel", [Kernel.PLAIN, Kernel.FUSED])
@pytest.mark.parametrize("dims", SIZES)
def test_bcc2_bit_exact(prec, kernel, dims):
    _run_real(Lattice.BCC2, prec, kernel, Potential.ARRAY, [dims])


@pytest.mark.parametrize("tile", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
def test_fused_tiles_batch_trap_bit_exact(tile, prec):
    _run_real(Lattice.BCC2, prec, Kernel.FUSED, Potential.TRAP, SIZES, steps=4, tile=tile)


def _two_step_tiles():
    from vaikkari_gb300.gpe import variants
    return [v["tile"] for v in variants() if v["half_steps"] == 2]


@pytest.mark.parametrize("potential", [Potential.TRAP, Potential.ARRAY])
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
def test_two_step_variants_bit_exact(prec, potential):
    """The variants that do both half-steps per launch (a second set of fields,
    O' and E' from one pass) equal the one-half-step kernel's order bit for
    bit: a batch of ragged sizes, odd and even step counts, and CUDA graphs of
    an odd number of steps (the sets alternate inside a graph)."""
    tiles = _two_step_tiles()
    assert len(tiles) >= 1
    for tile in tiles:
        n = _run_real(Lattice.BCC2, prec, Kernel.FUSED, potential, SIZES, steps=3, tile=tile)
        # one launch per step; per instance two field packs and two unpacks, and
        # for an array potential its pack and the L0 + V*dt copy
        transfers = len(SIZES) * (4 + (2 if potential == Potential.ARRAY else 0))
        assert n <= 3 + transfers
        _run_real(Lattice.BCC2, prec, Kernel.FUSED, potential, SIZES, steps=4, tile=tile, seed=5)
    _run_real(Lattice.BCC2, prec, Kernel.FUSED, potential, SIZES, steps=23, tile=tiles[0], graph_steps=7, seed=9)


def test_two_step_variant_refuses_imaginary_time_and_slabs():
    from vaikkari_gb300.gpe import GpeError
    tile = _two_step_tiles()[0]
    inst = Instance(8, 8, 8, 0.3, 1e-3, 10.0)
    with pytest.raises(GpeError):
        Stepper([inst], lattice=Lattice.BCC2, kernel=Kernel.FUSED, mode=Mode.IMAGINARY, tile=tile)
    st = Stepper([inst, inst], lattice=Lattice.BCC2, kernel=Kernel.FUSED, tile=tile)
    with pytest.raises(GpeError):
        st.link_z(0, 1)
    st.close()


@pytest.mark.parametrize("lattice", [Lattice.TETRA12, Lattice.BCC2])
def test_trap_potential_plain_bit_exact(lattice):
    _run_real(lattice, Precision.FP32, Kernel.PLAIN, Potential.TRAP, SIZES[:3], steps=2)


def test_graph_replay_equals_direct_launches():
    """A CUDA graph of 4 steps replayed, plus a remainder, equals 10 direct steps."""
    n_graph = _run_real(Lattice.BCC2, Precision.FP32, Kernel.FUSED, Potential.TRAP, SIZES, steps=10, graph_steps=4)
    n_direct = _run_real(Lattice.BCC2, Precision.FP32, Kernel.FUSED, Potential.TRAP, SIZES, steps=10, graph_steps=-1)
    assert n_graph == n_direct


@pytest.mark.parametrize("lattice,kernel", [(Lattice.TETRA12, Kernel.PLAIN), (Lattice.BCC2, Kernel.FUSED)])
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
def test_observables_match_oracle(lattice, kernel, prec):
    T = _dtype(prec)
    insts = [Instance(12, 10, 8, 0.4, 1e-3, 300.0, origin=(-2.4, -2.0, -1.6)),
             Instance(5, 7, 9, 0.5, 2e-3, 20.0, origin=(-1.0, -2.0, -2.0))]
    st = Stepper(insts, lattice=lattice, precision=prec, kernel=kernel, potential=Potential.ARRAY)
    rng = np.random.default_rng(5)
    wants = []
    for i in range(2):
        shp = st.shape(i)
        psi = random_state(shp, 40 + i, 0.1)
        V = rng.uniform(0, 5, size=shp)
        st.upload(i, psi, psi, V)
        g = grid_for(st, i)
        wants.append(g.observables(interleave(psi, T), vdt_for(st, i, V), vol_for(st, i)))
    got = st.observables(0)
    st.close()
    for w, o in zip(wants, got):
        for k in ("norm", "kinetic", "potential", "interaction", "energy", "mu"):
            assert o[k] == pytest.approx(w[k], rel=1e-12, abs=1e-14), k


@pytest.mark.parametrize("lattice,kernel", [(Lattice.TETRA12, Kernel.PLAIN), (Lattice.BCC2, Kernel.PLAIN),
                                            (Lattice.BCC2, Kernel.FUSED)])
def test_imaginary_time_fp64_matches_oracle(lattice, kernel):
    """FP64 imaginary time: psi and mu after 60 normalised Euler steps within 1e-11."""
    inst = Instance(10, 9, 8, 0.45, 2e-3, 40.0, origin=(-2.25, -2.0, -1.8), trap=(1.0, 1.0, 4.0))
    st = Stepper([inst], lattice=lattice, precision=Precision.FP64, mode=Mode.IMAGINARY, kernel=kernel,
                 potential=Potential.TRAP, graph_steps=20)
    shp = st.shape(0)
    rng = np.random.default_rng(7)
    psi0 = np.exp(1j * rng.uniform(0, 2 * np.pi, size=shp))
    st.upload(0, psi0)
    steps, conv, mu = st.imaginary_time(60, 0.0)
    got, _ = st.download(0, odd=False)
    st.close()
    g = grid_for(st, 0)
    psi = interleave(psi0, np.float64)
    vdt = vdt_for(st, 0)
    _, mu_hist = g.imaginary(psi, vdt, vol_for(st, 0), 60, 0.0)
    assert steps == 60 and not conv
    assert rel_l2(got, psi) < 1e-11
    assert mu[0] == pytest.approx(mu_hist[-1], rel=1e-11)


@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
def test_imaginary_time_batch_equals_single_runs(prec):
    """Three different condensates in one fused imaginary-time batch: each ends
    bit-identical to its own single-instance run (same variant and z-chunk, so
    the same work items; each instance's rows fold in a fixed order), including
    mu and the step count at convergence."""
    insts = [Instance(10, 9, 8, 0.45, 2e-3, 40.0, origin=(-2.25, -2.0, -1.8), trap=(1.0, 1.0, 4.0)),
             Instance(17, 6, 13, 0.4, 1e-3, 10.0, origin=(-3.4, -1.2, -2.6)),
             Instance(33, 12, 5, 0.3, 3e-3, 80.0, origin=(-4.95, -1.8, -0.75), trap=(2.0, 0.5, 1.0))]
    rng = np.random.default_rng(8)
    psis = [np.exp(1j * rng.uniform(0, 2 * np.pi, size=(i.nz, i.ny, i.nx, 2))) for i in insts]
    kw = dict(lattice=Lattice.BCC2, precision=prec, mode=Mode.IMAGINARY, kernel=Kernel.FUSED,
              potential=Potential.TRAP, graph_steps=20, tile=2, zchunk=4)
    st = Stepper(insts, **kw)
    for i, p in enumerate(psis):
        st.upload(i, p)
    steps, conv, mu = st.imaginary_time(150, 1e-6)
    batch = [st.download(i, odd=False)[0] for i in range(len(insts))]
    st.close()
    for i, p in enumerate(psis):
        one = Stepper([insts[i]], **kw)
        one.upload(0, p)
        s1, c1, mu1 = one.imaginary_time(steps, 0.0)
        got = one.download(0, odd=False)[0]
        one.close()
        np.testing.assert_array_equal(batch[i], got)
        assert mu[i] == mu1[0]


def test_imaginary_time_many_instances_equal_single_runs():
    """40 small condensates (more than the CTA's warps, so the fold takes the
    instances in several rounds): each equals its own single run bit for bit."""
    rng = np.random.default_rng(12)
    insts, psis = [], []
    for k in range(40):
        nx, ny, nz = (int(v) for v in rng.integers(1, 7, size=3))
        insts.append(Instance(nx, ny, nz, 0.4 + 0.01 * k, 1e-3, 5.0 + k, origin=(-0.2 * nx, -0.2 * ny, -0.2 * nz)))
        psis.append(np.exp(1j * rng.uniform(0, 2 * np.pi, size=(nz, ny, nx, 2))))
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP64, mode=Mode.IMAGINARY, kernel=Kernel.FUSED,
              potential=Potential.TRAP, graph_steps=10, tile=0, zchunk=2)
    st = Stepper(insts, **kw)
    for i, p in enumerate(psis):
        st.upload(i, p)
    steps, conv, mu = st.imaginary_time(25, 0.0)
    batch = [st.download(i, odd=False)[0] for i in range(len(insts))]
    st.close()
    for i in range(0, len(insts), 3):
        one = Stepper([insts[i]], **kw)
        one.upload(0, psis[i])
        _, _, mu1 = one.imaginary_time(steps, 0.0)
        got = one.download(0, odd=False)[0]
        one.close()
        np.testing.assert_array_equal(batch[i], got, err_msg=f"instance {i}")
        assert mu[i] == mu1[0]


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP64])
@pytest.mark.parametrize("mode", [Mode.REAL, Mode.IMAGINARY])
def test_plain_batch_equals_single_runs(prec, mode):
    """A batch on the plain kernel runs in one launch per half-step; each
    instance ends bit-identical to its own single run.  Sizes differ, and one
    instance is large enough to march more planes per thread than the others."""
    dims = [(5, 4, 3), (17, 9, 11), (40, 30, 100), (1, 1, 1), (33, 8, 7)]
    rng = np.random.default_rng(21)
    insts = [Instance(nx, ny, nz, 0.2 + 0.02 * k, 1e-3, 10.0 + k, origin=(-0.1 * nx, -0.1 * ny, -0.1 * nz))
             for k, (nx, ny, nz) in enumerate(dims)]
    kw = dict(lattice=Lattice.TETRA12, precision=prec, kernel=Kernel.PLAIN, mode=mode, potential=Potential.ARRAY,
              graph_steps=5)
    fields = []
    for inst in insts:
        shp = (inst.nz, inst.ny, inst.nx, 12)
        fields.append((random_state(shp, int(rng.integers(1000)), 0.3), random_state(shp, int(rng.integers(1000)), 0.3),
                       rng.uniform(0, 5, shp)))

    def run(sel):
        st = Stepper([insts[i] for i in sel], **kw)
        for k, i in enumerate(sel):
            e, o, V = fields[i]
            st.upload(k, e, o if mode == Mode.REAL else None, V)
        if mode == Mode.REAL:
            st.step(7)
        else:
            st.imaginary_time(7, 0.0)
        out = [st.download(k, odd=False)[0] for k in range(len(sel))]
        st.close()
        return out

    batch = run(list(range(len(insts))))
    for i in range(len(insts)):
        np.testing.assert_array_equal(batch[i], run([i])[0], err_msg=f"instance {i}")


def test_fused_batch_of_300_tiny_instances_bit_exact():
    """One fused launch over 300 instances of 1..4 blocks per side."""
    rng = np.random.default_rng(13)
    dims = [tuple(int(v) for v in rng.integers(1, 5, size=3)) for _ in range(300)]
    _run_real(Lattice.BCC2, Precision.FP32, Kernel.FUSED, Potential.TRAP, dims, steps=3, seed=4)


@pytest.mark.parametrize("kernel", [Kernel.PLAIN, Kernel.FUSED])
def test_imaginary_time_converges_to_harmonic_ground_state(kernel):
    """g = 0, isotropic trap: mu -> 3/2 up to the O(a^2) discretisation error."""
    n = 24
    a = 10.0 / n
    inst = Instance(n, n, n, a, 2e-3, 0.0, origin=(-5.0, -5.0, -5.0))
    st = Stepper([inst], lattice=Lattice.BCC2, precision=Precision.FP64, mode=Mode.IMAGINARY, kernel=kernel,
                 potential=Potential.TRAP)
    rng = np.random.default_rng(3)
    st.upload(0, (1.0 + 0.1 * rng.standard_normal(st.shape(0))).astype(np.complex128))
    steps, conv, mu = st.imaginary_time(20000, 1e-10)
    obs = st.observables(0)[0]
    st.close()
    assert conv
    assert mu[0] == pytest.approx(1.5, rel=3e-2)
    assert obs["norm"] == pytest.approx(1.0, rel=1e-12)
    assert obs["mu"] == pytest.approx(mu[0], rel=1e-8)


@pytest.mark.parametrize("lattice,kernel", [(Lattice.TETRA12, Kernel.PLAIN), (Lattice.BCC2, Kernel.FUSED)])
def test_observables_fp32_smooth_field_trap(lattice, kernel):
    """FP32 fields take the float-pair observables: a smooth Gaussian on a fine
    grid makes each value's Laplacian a small difference of large neighbour
    sums (the hardest case for reduced-precision arithmetic); with the trap
    potential, every sum still agrees with the FP64 oracle to 1e-12."""
    bw = 8 ** 0.5 if lattice == Lattice.TETRA12 else 1.0
    n, L = 24, 4.0
    bs = 2 * L / n / bw
    inst = Instance(n, n, n, bs, 1e-3, 700.0, origin=(-L, -L, -L), trap=(1.0, 1.7, 0.6))
    st = Stepper([inst], lattice=lattice, precision=Precision.FP32, kernel=kernel, potential=Potential.TRAP)
    from oracle.lattice import value_positions
    p = value_positions(n, n, n, bs, inst.origin, lattice)
    psi = np.exp(-0.5 * np.sum(p * p, axis=-1)) * np.exp(0.3j * p[..., 0])
    st.upload(0, psi, psi)
    want = grid_for(st, 0).observables(interleave(psi, np.float32), vdt_for(st, 0), vol_for(st, 0))
    got = st.observables(0)[0]
    st.close()
    for k in ("norm", "kinetic", "potential", "interaction", "energy", "mu"):
        assert got[k] == pytest.approx(want[k], rel=1e-12), k


def test_fp32_imaginary_time_stops_on_its_own_criterion():
    """FP32 imaginary time tests convergence on mu from the FP64 observables,
    once per chunk (mean change per step below tol): from a random-phase start
    it converges at tol 1e-9 by itself, in about as many steps as the FP64 run
    (which tests every step), and to the same mu within FP32's resolution."""
    n = 20
    a = 10.0 / n
    inst = Instance(n, n, n, a, 2e-3, 300.0, origin=(-5.0, -5.0, -5.0), trap=(1.0, 1.0, 4.0))
    rng = np.random.default_rng(31)
    psi = np.exp(1j * rng.uniform(0, 2 * np.pi, size=(n, n, n, 2)))
    res = {}
    for prec in (Precision.FP64, Precision.FP32):
        st = Stepper([inst], lattice=Lattice.BCC2, precision=prec, mode=Mode.IMAGINARY, kernel=Kernel.FUSED,
                     potential=Potential.TRAP, graph_steps=100)
        st.upload(0, psi)
        res[prec] = st.imaginary_time(60000, 1e-9)
        st.close()
    s64, c64, mu64 = res[Precision.FP64]
    s32, c32, mu32 = res[Precision.FP32]
    assert c64 and c32
    assert s32 <= 1.5 * s64 + 200
    assert mu32[0] == pytest.approx(mu64[0], rel=1e-6)
