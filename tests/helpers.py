"""Helpers shared by the parity tests: oracle grids and potential arrays that
mirror what the library feeds its kernels.  The stencil tables, volumes and
value positions come from the oracle's own copy of the reference's tables
(oracle/lattice.py, read from tests/golden), never from the library under test."""
import numpy as np

import oracle.oracle as orc
from oracle.lattice import tables
from vaikkari_gb300.gpe import Potential, Precision


def grid_for(stepper, i):
    inst = stepper.instances[i]
    t = tables(stepper.lattice)
    return orc.Grid(inst.nx, inst.ny, inst.nz, t["entry"], t["class_weight"], inst.block_scale, inst.dt, inst.g)


def vol_for(stepper, i):
    return tables(stepper.lattice)["cell_volume"] * stepper.instances[i].block_scale ** 3


def vdt_for(stepper, i, V=None):
    """dt*V per value in the kernels' precision, computed the way the library
    does: ARRAY -> T(double(T(V)) * dt); TRAP -> per-axis tables
    T(0.5*trap*p*p*dt) summed as (Vx + Vy) + Vz in T."""
    inst = stepper.instances[i]
    T = np.float64 if stepper.precision == Precision.FP64 else np.float32
    if stepper.potential == Potential.ARRAY:
        return np.ascontiguousarray((np.asarray(V, dtype=T).astype(np.float64) * inst.dt).astype(T))
    t = tables(stepper.lattice)
    bw, pos = t["block_width"], t["position"]
    n = (inst.nx, inst.ny, inst.nz)
    tabs = []
    for axis in range(3):
        i_ = np.arange(n[axis])[None, :]
        p = inst.origin[axis] + inst.block_scale * (i_ * bw + pos[:, axis][:, None])   # [slot][i]
        tabs.append((0.5 * inst.trap[axis] * p * p * inst.dt).astype(T))
    tx, ty, tz = tabs
    # (nz, ny, nx, slots)
    v = (tx.T[None, None, :, :] + ty.T[None, :, None, :]).astype(T)
    v = (v + tz.T[:, None, None, :]).astype(T)
    return np.ascontiguousarray(v)


def interleave(psi, dtype):
    a = np.stack([psi.real, psi.imag], axis=-1) if np.iscomplexobj(psi) else psi
    return np.ascontiguousarray(a.astype(dtype))


def random_state(shape, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))
