"""The allocation-free observables entry point (gpe_observables_noalloc).

It serves callers that cannot allocate device memory; it takes the condensate
from the caller's device memory and keeps its scratch in one static device
array.  The GPU test checks it against the handle path (gpe_observables_get) on
two calls in a row, so that the second call runs on scratch the first call
left behind.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import interleave, random_state
from vaikkari_gb300 import gpe
from vaikkari_gb300.gpe import GpeError, Instance, Kernel, Lattice, Potential, Precision, Status, Stepper

KEYS = ("norm", "kinetic", "potential", "interaction", "energy", "mu")


def test_noalloc_rejects_bad_arguments_without_a_gpu():
    lib = gpe.load_library()
    out = gpe._Observables()
    big = Instance(2048, 2048, 4, 0.5, 1e-3, 1.0).c()   # 2048*2048*4*2 values > 16,777,216
    assert lib.gpe_observables_noalloc(1, 0, C.byref(big), C.c_void_p(16), None, None, C.byref(out)) == \
        Status.TOO_LARGE
    assert b"16,777,216" in lib.gpe_last_error()
    ok = Instance(4, 4, 4, 0.5, 1e-3, 1.0).c()
    assert lib.gpe_observables_noalloc(1, 0, C.byref(ok), None, None, None, C.byref(out)) == Status.INVALID_ARGUMENT
    assert lib.gpe_observables_noalloc(5, 0, C.byref(ok), C.c_void_p(16), None, None, C.byref(out)) == \
        Status.INVALID_ARGUMENT


@pytest.mark.gpu
def test_noalloc_matches_handle_observables_on_two_calls():
    import torch
    cases = [(Lattice.BCC2, Precision.FP64, (12, 10, 8)), (Lattice.TETRA12, Precision.FP64, (5, 7, 9)),
             (Lattice.BCC2, Precision.FP32, (33, 9, 6))]
    for call in range(2):
        for ci, (lattice, prec, dims) in enumerate(cases):
            T = np.float64 if prec == Precision.FP64 else np.float32
            bw = 8 ** 0.5 if lattice == Lattice.TETRA12 else 1.0
            bs = 0.4 / bw
            inst = Instance(*dims, block_scale=bs, dt=1e-3, g=300.0 + 50 * call,
                            origin=tuple(-0.5 * n * bs * bw for n in dims))
            st = Stepper([inst], lattice=lattice, precision=prec, kernel=Kernel.PLAIN, potential=Potential.ARRAY)
            shp = st.shape(0)
            psi = random_state(shp, 100 + 10 * call + ci, 0.1)
            V = np.random.default_rng(7 + call).uniform(0.0, 5.0, size=shp)
            st.upload(0, psi, psi, V)
            want = st.observables(0)[0]
            st.close()
            f = torch.from_numpy(interleave(psi, T)).cuda()
            v = torch.from_numpy(np.ascontiguousarray(V.astype(T))).cuda()
            torch.cuda.synchronize()
            got = gpe.observables_noalloc(lattice, prec, inst, f.data_ptr(), v.data_ptr())
            for k in KEYS:
                # The handle path stores V*dt in the handle's precision and divides by dt,
                # so in FP32 the potential-dependent sums carry that rounding (~6e-8).
                tol = 1e-12 if (prec == Precision.FP64 or k in ("norm", "kinetic", "interaction")) else 2e-7
                assert got[k] == pytest.approx(want[k], rel=tol, abs=1e-15), (call, lattice.name, prec.name, k)


@pytest.mark.gpu
def test_noalloc_trap_potential_and_caller_stream():
    """potential = NULL takes the harmonic trap of the instance (compared with a
    handle built with the trap form), and the call runs on a stream the caller
    passes (a torch stream here), twice in a row."""
    import torch
    lattice, prec = Lattice.BCC2, Precision.FP64
    inst = Instance(11, 9, 7, 0.37, 1e-3, 250.0, origin=(-2.0, -1.6, -1.3), trap=(1.0, 2.5, 0.6))
    st = Stepper([inst], lattice=lattice, precision=prec, kernel=Kernel.PLAIN, potential=Potential.TRAP)
    shp = st.shape(0)
    psi = random_state(shp, 41, 0.2)
    st.upload(0, psi, psi)
    want = st.observables(0)[0]
    st.close()
    s = torch.cuda.Stream()
    f = torch.from_numpy(interleave(psi, np.float64)).cuda()
    torch.cuda.synchronize()
    for call in range(2):
        with torch.cuda.stream(s):
            got = gpe.observables_noalloc(lattice, prec, inst, f.data_ptr(), 0, stream=s.cuda_stream)
        for k in KEYS:
            assert got[k] == pytest.approx(want[k], rel=1e-12, abs=1e-15), (call, k)


@pytest.mark.gpu
def test_noalloc_equals_the_oracle():
    """Against the CPU oracle directly (FP64 sums of the reference's stencil),
    for both lattices, with an array potential."""
    import torch
    import oracle.oracle as orc
    from oracle.lattice import tables
    for lattice, dims in ((Lattice.BCC2, (10, 7, 6)), (Lattice.TETRA12, (4, 5, 3))):
        t = tables(lattice)
        inst = Instance(*dims, block_scale=0.3, dt=2e-3, g=120.0)
        shp = (dims[2], dims[1], dims[0], t["slots"])
        psi = random_state(shp, 57, 0.3)
        V = np.random.default_rng(58).uniform(0.0, 3.0, size=shp)
        g = orc.Grid(*dims, t["entry"], t["class_weight"], inst.block_scale, inst.dt, inst.g)
        want = g.observables(interleave(psi, np.float64), np.ascontiguousarray(V * inst.dt),
                             t["cell_volume"] * inst.block_scale ** 3)
        f = torch.from_numpy(interleave(psi, np.float64)).cuda()
        v = torch.from_numpy(np.ascontiguousarray(V)).cuda()
        torch.cuda.synchronize()
        got = gpe.observables_noalloc(lattice, Precision.FP64, inst, f.data_ptr(), v.data_ptr())
        for k in KEYS:
            assert got[k] == pytest.approx(want[k], rel=1e-11, abs=1e-14), (lattice.name, k)


@pytest.mark.gpu
def test_noalloc_at_the_size_limit():
    """Exactly GPE_NOALLOC_MAX_ROWS * GPE_NOALLOC_VALUES_PER_ROW = 16,777,216
    values (BCC2, 256 x 256 x 128 blocks) fill every row of the scratch array and
    agree with the handle path; one more plane of blocks is refused."""
    import torch
    inst = Instance(256, 256, 128, 16.0 / 256, 1e-4, 800.0, origin=(-8.0, -8.0, -4.0), trap=(1.0, 1.0, 1.5))
    st = Stepper([inst], lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED,
                 potential=Potential.TRAP)
    shp = st.shape(0)
    assert np.prod(shp) == 16_777_216
    rng = np.random.default_rng(71)
    psi = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) * 1e-3
    st.upload(0, psi, psi)
    want = st.observables(0)[0]
    st.close()
    f = torch.from_numpy(interleave(psi, np.float32)).cuda()
    torch.cuda.synchronize()
    got = gpe.observables_noalloc(Lattice.BCC2, Precision.FP32, inst, f.data_ptr(), 0)
    for k in KEYS:
        # the handle forms V*dt from FP32 per-axis tables; here V is FP64 per value
        tol = 1e-10 if k in ("norm", "kinetic", "interaction") else 2e-7
        assert got[k] == pytest.approx(want[k], rel=tol), k
    over = Instance(256, 256, 129, 16.0 / 256, 1e-4, 800.0)
    with pytest.raises(GpeError) as e:
        gpe.observables_noalloc(Lattice.BCC2, Precision.FP32, over, f.data_ptr(), 0)
    assert e.value.status == Status.TOO_LARGE
