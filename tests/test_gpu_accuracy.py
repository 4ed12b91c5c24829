"""The precision target on the reference configuration: FP32 storage and
arithmetic against FP64 of the same scheme after 1000 real-time steps (32^3
cells, g = 500, dt = 1e-4): relative L2 <= 1e-5 and norm drift <= 1e-6."""
import math

import numpy as np
import pytest

from vaikkari_gb300 import workloads
from vaikkari_gb300.gpe import Kernel, Lattice, Mode, Potential, Precision, Stepper

pytestmark = pytest.mark.gpu


def _run(prec, c, steps):
    st = Stepper([c.inst], lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=Potential.TRAP)
    st.upload(0, c.psi, c.psi)
    mu = st.observables(0)[0]["mu"]
    st.upload(0, c.psi, workloads.odd_from_even(c.psi, mu, c.inst.dt))
    st.step(steps)
    obs = st.observables(0)[0]
    f = st.download(0, odd=False)[0].astype(np.float64)
    st.close()
    return obs, f


def test_fp32_meets_l2_and_norm_targets_config1():
    c = workloads.config1()
    o64, f64 = _run(Precision.FP64, c, 1000)
    o32, f32 = _run(Precision.FP32, c, 1000)
    rel_l2 = math.sqrt(float(np.sum((f32 - f64) ** 2)) / float(np.sum(f64 ** 2)))
    assert rel_l2 <= 1e-5
    assert abs(o32["norm"] - o64["norm"]) / o64["norm"] <= 1e-6
    assert abs(o32["energy"] - o64["energy"]) / abs(o64["energy"]) <= 1e-5
