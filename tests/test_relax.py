"""The vortex relaxation (VortexState::iterateSolution, koodit/GrossPitaevskii/
VortexState.cpp:109-185) and the two-stage state construction of main()
(GPUGrossPitaevskii_BCC.cu:509-531).

CPU: the oracle in the reference's summation order reproduces the reference's
own outputs bit for bit (a state its iterateSolution made here, and the shipped
state.dat by digest); the chunked order the GPU uses stays within rounding of it;
the library's host steps (initial profile, resampling, file format) equal the
oracle's.  GPU: gpe_vortex_relax equals the oracle in the chunked order bit for
bit (one state, a batch of different states, rows in several cluster rounds), and
main()'s whole construction on the GPU agrees with state.dat to rounding."""
import hashlib
import os

import numpy as np
import pytest

import oracle.oracle as orc
from conftest import GOLDEN, golden
from vaikkari_gb300.gpe import GpeError, VortexState, relax

SMALL = os.path.join(GOLDEN, "ref_state_small.dat")


def _coarse(step=0.25):
    return orc.Vortex.from_range(20, 5000.0, 0.0, 15.0, 35.0, step, step)


def test_oracle_reproduces_reference_relaxation():
    """setRange(0, 15, 35, 0.25, 0.25) + iterateSolution(potentialRZ, 3000, 1e-29),
    run by the reference's own code into ref_state_small.dat."""
    ref = orc.Vortex.from_file(SMALL)
    v = _coarse()
    assert (v.rsize, v.zsize, v.rstep, v.zstep) == (ref.rsize, ref.zsize, ref.rstep, ref.zstep)
    its, diff = v.iterate(3000)
    assert its < 3000 and diff < 1e-29     # converged and broke out early
    assert v.mu == ref.mu
    np.testing.assert_array_equal(v.f, ref.f)


def test_oracle_reproduces_shipped_state_dat():
    """main()'s construction (coarse 0.2 grid, 10000 iterations; fine 0.03 grid
    resampled from it, 10000 iterations) equals the reference's state.dat: header,
    mu and the SHA-256 of all 233,000 values."""
    ref = golden("ref_state_main.json")
    s0 = _coarse(0.2)
    s0.iterate(10000)
    eps = 1e-5 * s0.function_max()
    s = orc.Vortex.from_range(20, 5000.0, s0.min_r(eps), s0.max_r(eps), s0.max_z(eps), 0.03, 0.03)
    assert (s.rsize, s.zsize, s.rplug, s.rstep, s.zstep) == (ref["rsize"], ref["zsize"], ref["rplug"],
                                                             ref["rstep"], ref["zstep"])
    s.initialize(s0)
    s.iterate(10000)
    assert s.mu == ref["mu"]
    assert hashlib.sha256(s.f.astype("<f8").tobytes()).hexdigest() == ref["values_sha256"]


def test_chunked_order_within_rounding():
    """The GPU's summation order against the reference's on the same relaxation."""
    ref = orc.Vortex.from_file(SMALL)
    v = _coarse()
    v.iterate(3000, order=1)
    assert abs(v.mu - ref.mu) <= 1e-13 * ref.mu
    assert np.abs(v.f - ref.f).max() <= 1e-12 * ref.f.max()


def test_library_host_steps_equal_oracle(tmp_path):
    """Initial profile (setDimensions), resampling (initialize) and save/load."""
    lib = VortexState.create(20, 5000.0, 0.0, 15.0, 35.0, 0.25, 0.25)
    o = _coarse()
    np.testing.assert_array_equal(lib.values().reshape(-1), o.f)
    fine = VortexState.create(20, 5000.0, 1.0, 9.0, 20.0, 0.1, 0.1)
    of = orc.Vortex.from_range(20, 5000.0, 1.0, 9.0, 20.0, 0.1, 0.1)
    src = VortexState(SMALL)
    fine.initialize(src)
    of.initialize(orc.Vortex.from_file(SMALL))
    np.testing.assert_array_equal(fine.values().reshape(-1), of.f)
    assert fine.describe()["mu"] == of.mu
    p = str(tmp_path / "s.dat")
    fine.save(p)
    back = orc.Vortex.from_file(p)
    np.testing.assert_array_equal(back.f, of.f)
    assert src.describe()["min_r"] == orc.Vortex.from_file(SMALL).min_r(1e-5 * src.describe()["function_max"])


# ---------------------------------------------------------------- GPU ---------

def _pair(*args):
    return VortexState.create(*args), orc.Vortex.from_range(*args)


@pytest.mark.gpu
def test_relax_equals_oracle_chunked_order():
    """The coarse relaxation to convergence: same iteration count, mu and values."""
    lib, o = _pair(20, 5000.0, 0.0, 15.0, 35.0, 0.25, 0.25)
    res = lib.relax(3000)
    its, diff = o.iterate(3000, order=1)
    assert res["iterations"] == its and res["diff"] == diff
    assert lib.describe()["mu"] == o.mu
    np.testing.assert_array_equal(lib.values().reshape(-1), o.f)


@pytest.mark.gpu
def test_relax_batch_and_cluster_rounds():
    """Three different states in one call; one has 1099 updated rows (35 bands of
    32 over a cluster of 8 CTAs of 4 bands, so two rounds), one a single z
    column, one odd sizes."""
    args = [(20, 5000.0, 0.0, 15.0, 3.0, 15.0 / 1100, 0.5),    # 1100 x 6
            (4, 100.0, 0.5, 6.0, 1.0, 0.05, 1.0),       # 110 x 1: main()'s 2-D set-up (laplz = 0)
            (8, 800.0, 0.3, 9.7, 13.0, 0.37, 0.29)]     # odd sizes
    libs, ors = zip(*[_pair(*a) for a in args])
    res = relax(list(libs), 40, eps=0.0, graph_iterations=16)
    for lib, o, r in zip(libs, ors, res):
        its, diff = o.iterate(40, eps=0.0, order=1)
        assert r["iterations"] == its == 40 and r["diff"] == diff
        assert lib.describe()["mu"] == o.mu
        np.testing.assert_array_equal(lib.values().reshape(-1), o.f)


@pytest.mark.gpu
def test_relax_edge_cases():
    lib, o = _pair(20, 5000.0, 0.0, 15.0, 35.0, 0.5, 0.5)
    before = lib.values().copy()
    r = lib.relax(0)                       # no iterations: row 0 zeroed, sign rule only
    o.iterate(0, order=1)
    assert r["iterations"] == 0
    np.testing.assert_array_equal(lib.values().reshape(-1), o.f)
    assert np.array_equal(lib.values()[1:], before[1:])
    one = VortexState.create(1, 1.0, 0.0, 0.5, 1.0, 1.0, 0.5)   # a single r row: nothing to relax
    with pytest.raises(GpeError):
        one.relax(10)


def test_degenerate_range_refused():
    """zmax below half a step: the reference's setRange divides by a zero count."""
    with pytest.raises(GpeError):
        VortexState.create(4, 100.0, 0.5, 6.0, 0.4, 0.05, 1.0)
    with pytest.raises(ValueError):
        orc.Vortex.from_range(4, 100.0, 0.5, 6.0, 0.4, 0.05, 1.0)


@pytest.mark.gpu
def test_main_construction_on_gpu_matches_state_dat():
    """main()'s two relaxations on the GPU (library calls only) against the
    reference's shipped state.dat: mu within 1e-12, values within 1e-10 of the
    maximum (the per-iteration sums round differently)."""
    ref = golden("ref_state_main.json")
    s0 = VortexState.create(20, 5000.0, 0.0, 15.0, 35.0, 0.2, 0.2)
    s0.relax(10000)
    d0 = s0.describe(1e-5)
    s = VortexState.create(20, 5000.0, d0["min_r"], d0["max_r"], d0["max_z"], 0.03, 0.03)
    d = s.describe()
    assert (d["rsize"], d["zsize"], d["rplug"], d["rstep"], d["zstep"]) == (
        ref["rsize"], ref["zsize"], ref["rplug"], ref["rstep"], ref["zstep"])
    s.initialize(s0)
    r = s.relax(10000)
    assert r["iterations"] == 10000
    assert abs(s.describe()["mu"] - ref["mu"]) <= 1e-12 * ref["mu"]
    f = s.values().reshape(-1)
    got = f[np.array(ref["sample_index"])]
    assert np.abs(got - np.array(ref["sample_value"])).max() <= 1e-10 * ref["function_max"]
    assert abs(f.max() - ref["function_max"]) <= 1e-10 * ref["function_max"]


@pytest.mark.gpu
def test_sweep_division_is_correctly_rounded():
    """The sweep divides by way of a precomputed reciprocal; it must equal
    __ddiv_rn bit for bit on the relaxation's ranges and far outside them."""
    from vaikkari_gb300.gpe import debug_divide
    rng = np.random.default_rng(11)
    n = 1 << 22
    a = rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-320, 300, n)     # includes subnormal numerators
    b = rng.choice([-1.0, 1.0], n) * rng.uniform(1, 2, n) * 10.0 ** rng.uniform(-5, 8, n)
    a[:1000] = 0.0
    a[1000:2000] = np.nextafter(1.0, 2.0) * rng.integers(1, 1 << 20, 1000)
    b[2000:3000] = -(2.0 - 2.0 ** -52)                                 # all-ones significands
    ours, ref = debug_divide(a, b)
    np.testing.assert_array_equal(ours.view(np.int64), ref.view(np.int64))


@pytest.mark.gpu
def test_relax_small_numerators_take_the_exact_division(tmp_path):
    """Values near 1e-296 in the inner rows give numerators below 2^-900 (the
    sweep runs outwards in r, so the large outer values reach them one row per
    iteration), where the sweep's reciprocal-based division does not apply: the
    flagged sweep is redone with __ddiv_rn, and the result still equals the
    oracle bit for bit."""
    import struct
    o = orc.Vortex.from_range(6, 300.0, 0.0, 8.0, 6.0, 0.2, 0.2)
    f = o.f.reshape(o.rsize, o.zsize)
    f[: o.rsize // 2] *= 1e-296
    path = str(tmp_path / "tiny.dat")
    with open(path, "wb") as fh:
        fh.write(struct.pack("<IdIIdddd", o.kappa, o.g, o.rsize, o.zsize, o.rplug, o.rstep, o.zstep, o.mu))
        fh.write(o.f.astype("<f8").tobytes())
    lib = VortexState(path)
    res = lib.relax(3, eps=0.0)
    its, diff = o.iterate(3, eps=0.0, order=1)
    assert res["iterations"] == its == 3 and res["diff"] == diff
    assert lib.describe()["mu"] == o.mu
    got = lib.values().reshape(-1)
    assert np.abs(got[: o.zsize * (o.rsize // 2 - 5)]).max() < 1e-250      # the small region stayed small
    np.testing.assert_array_equal(got, o.f)
