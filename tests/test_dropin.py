"""The reference's solver call rebuilt on the library: VortexState reading,
psi sampling and integrateInTime's host set-up are bit-identical to the
reference's own code (fixtures made by running it), and the GPU run matches the
reference's own update kernel from that set-up."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from vaikkari_gb300.gpe import Precision, VortexState

SMALL = os.path.join(GOLDEN, "ref_state_small.dat")


def _state():
    return VortexState(SMALL)


def test_vortex_diagnostics_equal_reference():
    ref = golden("ref_vortex_small.json")
    info = _state().describe(1e-5)
    for k_ours, k_ref in (("kappa", "kappa"), ("g", "g"), ("mu", "mu"), ("function_max", "function_max"),
                          ("max_r", "maxr"), ("max_z", "maxz"), ("curvature", "curvature"),
                          ("block_scale", "block_scale")):
        assert info[k_ours] == ref[k_ref], k_ours


def test_vortex_psi_equals_reference_getpsi():
    ref = golden("ref_vortex_small.json")
    st = _state()
    for x, y, z, re, im in ref["psi_samples"]:
        c = st.psi((x, y, z))
        assert (c.real, c.imag) == (re, im), (x, y, z)


def test_integrate_setup_equals_reference():
    """Grid, factors, dt, odd phase and every array of integrateInTime's set-up
    (GPUGrossPitaevskii_BCC.cu:222-348) on the same state, bit for bit."""
    ref = golden("ref_setup_small.json")
    res, even, odd, V = _state().setup(ref["block_scale"], ref["minp"], ref["maxp"])
    for k in ("xsize", "ysize", "zsize"):
        assert res[k] == ref[k]
    assert res["steps_per_iteration"] == ref["steps_per_iteration"]
    assert res["p0"] == ref["p0"]
    for k_ours, k_ref in (("maxpot", "maxpot"), ("dt", "dt"), ("lapfac_dt", "lapfac_dt"),
                          ("lapfac0_dt", "lapfac0_dt"), ("g_dt", "g_dt")):
        assert res[k_ours] == ref[k_ref], k_ours
    assert res["odd_phase"] == ref["odd_phase"]
    n = res["values"]
    raw = np.fromfile(os.path.join(GOLDEN, "ref_setup_small.bin"), dtype=np.float64)
    re, ro, rp = raw[:2 * n], raw[2 * n:4 * n], raw[4 * n:]
    np.testing.assert_array_equal(even.reshape(-1), re)
    np.testing.assert_array_equal(odd.reshape(-1), ro)
    np.testing.assert_array_equal((V * res["dt"]).reshape(-1), rp)


def test_integrate_grid_equals_setup():
    """gpe_integrate_grid gives the set-up's grid without sampling."""
    ref = golden("ref_setup_small.json")
    st = _state()
    grid = st.grid(ref["block_scale"], ref["minp"], ref["maxp"])
    res = st.setup(ref["block_scale"], ref["minp"], ref["maxp"])[0]
    for k in ("xsize", "ysize", "zsize", "values", "p0"):
        assert grid[k] == res[k], k
    assert grid["maxpot"] == 0.0 and grid["steps_per_iteration"] == 0


def test_integrate_calls_refuse_bad_arguments():
    """The solver call and the grid query check their arguments before any GPU
    work: a non-positive block scale, a domain that does not fit, a precision the
    solver call does not take."""
    from vaikkari_gb300.gpe import GpeError, Status
    ref = golden("ref_setup_small.json")
    st = _state()
    with pytest.raises(GpeError) as e:
        st.grid(0.0, ref["minp"], ref["maxp"])
    assert e.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        st.grid(ref["block_scale"], ref["maxp"], ref["minp"])          # max below min
    assert e.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        st.integrate_in_time(ref["block_scale"], ref["minp"], ref["maxp"], 1.0, 0, precision=Precision.FP32C)
    assert e.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        st.integrate_in_time(ref["block_scale"], ref["minp"], ref["maxp"], 0.0, 1)
    assert e.value.status == Status.INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32])
def test_integrate_setup_on_gpu_equals_reference(prec):
    """The set-up inside gpe_integrate_in_time runs its per-value work on the GPU.
    With no iterations the fields it returns are the reference's own set-up
    (GPUGrossPitaevskii_BCC.cu:222-348, fixture made by running it) bit for bit,
    in FP32 after one rounding to float."""
    ref = golden("ref_setup_small.json")
    res, obs, even, odd = _state().integrate_in_time(ref["block_scale"], ref["minp"], ref["maxp"], 1.0, 0,
                                                     precision=prec)
    assert len(obs) == 1 and res["setup_ms"] > 0.0
    assert res["steps_per_iteration"] == ref["steps_per_iteration"]
    for k_ours, k_ref in (("maxpot", "maxpot"), ("dt", "dt"), ("lapfac_dt", "lapfac_dt"),
                          ("lapfac0_dt", "lapfac0_dt"), ("g_dt", "g_dt")):
        assert res[k_ours] == ref[k_ref], k_ours
    assert res["odd_phase"] == ref["odd_phase"]
    n = res["values"]
    raw = np.fromfile(os.path.join(GOLDEN, "ref_setup_small.bin"), dtype=np.float64)
    re, ro = raw[:2 * n], raw[2 * n:4 * n]
    if prec == Precision.FP32:
        re, ro = re.astype(np.float32).astype(np.float64), ro.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(even.reshape(-1), re)
    np.testing.assert_array_equal(odd.reshape(-1), ro)


@pytest.mark.gpu
def test_integrate_in_time_matches_reference_kernel():
    """Two iterations (2 x steps_per_iteration leapfrog steps) of the drop-in on
    the GPU against the reference's own update kernel (built for sm_103a) from the
    same set-up, and the CPU oracle: all three bit for bit."""
    import refkernel
    ref = golden("ref_setup_small.json")
    st = _state()
    res, even0, odd0, V = st.setup(ref["block_scale"], ref["minp"], ref["maxp"])
    iters = 2
    res2, obs, even, odd = st.integrate_in_time(ref["block_scale"], ref["minp"], ref["maxp"], 1.0, iters,
                                                precision=Precision.FP64)
    assert len(obs) == iters + 1 and all(np.isfinite(o["energy"]) for o in obs)
    steps = iters * res["steps_per_iteration"]
    X, Y, Z = res["xsize"], res["ysize"], res["zsize"]
    if refkernel.available():
        rk = refkernel.ReferenceUpdate(X, Y, Z)
        rk.upload(even0, odd0, V * res["dt"])
        rk.step(steps, ref["block_scale"], res["dt"], _state().describe()["g"])
        re, ro = rk.download()
        np.testing.assert_array_equal(even, re)
        np.testing.assert_array_equal(odd, ro)
    # the oracle, with the reference's own table (tests/golden)
    import oracle.oracle as orc
    from oracle.lattice import tables
    from vaikkari_gb300.gpe import Lattice
    info = tables(Lattice.TETRA12)
    g = orc.Grid(X, Y, Z, info["entry"], info["class_weight"], ref["block_scale"], res["dt"],
                 _state().describe()["g"])
    e, o = np.ascontiguousarray(even0), np.ascontiguousarray(odd0)
    g.leapfrog(e, o, np.ascontiguousarray(V * res["dt"]), steps)
    np.testing.assert_array_equal(even, e)
    np.testing.assert_array_equal(odd, o)
