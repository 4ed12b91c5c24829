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
