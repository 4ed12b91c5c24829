"""Seeded synthetic condensates for the benchmark and parity configurations.

All five live on the BCC2 lattice over the domain [-8, 8]^3 (block grid of N^3
cubes of edge a = 16/N, origin at -8), with psi = 0 outside.  The same domain
in the reference's TETRA12 lattice uses block_scale = a / sqrt(8).

  config1  32^3, V = r^2/2, g = 500, Gaussian exp(-r^2/2) normalised, x (1 + 1e-3 (n1 + i n2)),
           n normal (seed 0); 1000 real-time steps at dt = 1e-4.
  config2  128^3, V = (x^2 + y^2 + 4 z^2)/2, g = 2000, uniform modulus, random phase (seed 1);
           imaginary time at dt = 5e-4 until |dmu| < 1e-9.
  config3  192^3, V = r^2/2, g = 3000, Thomas-Fermi sqrt(max(mu - V, 0)/g) normalised, times a
           ring-vortex phase (ring radius 3 in the z = 0 plane, unit winding); dt = 5e-5.
  config4  64 instances, N uniform over {24, 32, 48, 64, 96} (seed 2), g log-uniform in
           [100, 5000], trap frequencies per axis uniform in [0.5, 2] (V = sum w_a^2 x_a^2 / 2),
           Gaussian with 1e-3 noise; dt = 1e-4.
  config5  512^3, V = r^2/2, g = 1e4, Thomas-Fermi with phase noise 1e-2 (seed 3); dt = 2e-5.

The leapfrog's second field is the first rotated by half a step of the
chemical potential, odd = even * exp(+i mu dt / 2), as the reference does with
VortexState::getPhase(-dt/2) (GPUGrossPitaevskii_BCC.cu:325,342); mu is the
discrete chemical potential of the initial field.

Every builder takes the lattice's geometry (block width, value positions, cell
volume: the dict gpe.lattice_info returns) as `geometry`; by default it asks the
library.  This module imports no native code itself, so a caller that must not
load the library (the CPU baseline) can pass the oracle's tables instead and
get the same seeded condensates.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence, Optional

import numpy as np

from .instance import Instance, Lattice, value_positions

L_HALF = 8.0


@dataclass
class Condensate:
    inst: Instance
    psi: np.ndarray          # complex128, (nz, ny, nx, slots)
    V: Optional[np.ndarray]  # float64 potential per value (None when the trap form is used)


def _geom(lattice: Lattice, geometry: Optional[dict]) -> dict:
    if geometry is not None:
        return geometry
    from .gpe import lattice_info
    return lattice_info(lattice)


def bcc2_instance(n: int, dt: float, g: float, trap=(1.0, 1.0, 1.0)) -> Instance:
    a = 2 * L_HALF / n
    return Instance(nx=n, ny=n, nz=n, block_scale=a, dt=dt, g=g, origin=(-L_HALF,) * 3, trap=tuple(trap))


def tetra12_instance(n: int, dt: float, g: float, trap=(1.0, 1.0, 1.0)) -> Instance:
    a = 2 * L_HALF / n
    return Instance(nx=n, ny=n, nz=n, block_scale=a / math.sqrt(8.0), dt=dt, g=g, origin=(-L_HALF,) * 3,
                    trap=tuple(trap))


def _vol(inst: Instance, info: dict) -> float:
    return info["cell_volume"] * inst.block_scale ** 3


def normalise(psi: np.ndarray, vol: float) -> np.ndarray:
    return psi / math.sqrt(vol * float(np.sum(np.abs(psi) ** 2)))


def harmonic(pos: np.ndarray, trap) -> np.ndarray:
    return 0.5 * (trap[0] * pos[..., 0] ** 2 + trap[1] * pos[..., 1] ** 2 + trap[2] * pos[..., 2] ** 2)


def gaussian_state(inst: Instance, info: dict, rng: np.random.Generator, noise: float) -> np.ndarray:
    p = value_positions(inst, info)
    r2 = np.sum(p * p, axis=-1)
    psi = np.exp(-r2 / 2).astype(np.complex128)
    psi = normalise(psi, _vol(inst, info))
    n = rng.standard_normal(psi.shape) + 1j * rng.standard_normal(psi.shape)
    return psi * (1 + noise * n)


def thomas_fermi(inst: Instance, info: dict, V: np.ndarray) -> np.ndarray:
    """sqrt(max(mu - V, 0)/g) with mu chosen so that the density integrates to 1
    (bisection on a strided subsample of V for large grids; the result is then
    normalised exactly on the full grid)."""
    vol = _vol(inst, info)
    flat = V.reshape(-1)
    step = max(1, flat.size // 4_000_000)
    sub = flat[::step]
    wvol = vol * flat.size / sub.size
    lo, hi = 0.0, float(sub.max()) + inst.g
    for _ in range(100):
        mu = 0.5 * (lo + hi)
        n = wvol * float(np.sum(np.maximum(mu - sub, 0.0))) / inst.g
        lo, hi = (mu, hi) if n < 1.0 else (lo, mu)
    psi = np.sqrt(np.maximum(mu - V, 0.0) / inst.g).astype(np.complex128)
    return normalise(psi, vol)


def config1(lattice: Lattice = Lattice.BCC2, geometry: Optional[dict] = None, n: int = 32) -> Condensate:
    info = _geom(lattice, geometry)
    mk = bcc2_instance if lattice == Lattice.BCC2 else tetra12_instance
    inst = mk(n, dt=1e-4, g=500.0)
    rng = np.random.default_rng(0)
    psi = gaussian_state(inst, info, rng, 1e-3)
    V = harmonic(value_positions(inst, info), inst.trap)
    return Condensate(inst, psi, V)


def config2(lattice: Lattice = Lattice.BCC2, geometry: Optional[dict] = None, n: int = 128) -> Condensate:
    info = _geom(lattice, geometry)
    mk = bcc2_instance if lattice == Lattice.BCC2 else tetra12_instance
    inst = mk(n, dt=5e-4, g=2000.0, trap=(1.0, 1.0, 4.0))
    rng = np.random.default_rng(1)
    phase = rng.uniform(0.0, 2 * math.pi, size=(n, n, n, info["slots"]))
    psi = normalise(np.exp(1j * phase), _vol(inst, info))
    V = harmonic(value_positions(inst, info), inst.trap)
    return Condensate(inst, psi, V)


def config3(lattice: Lattice = Lattice.BCC2, geometry: Optional[dict] = None, n: int = 192) -> Condensate:
    info = _geom(lattice, geometry)
    mk = bcc2_instance if lattice == Lattice.BCC2 else tetra12_instance
    inst = mk(n, dt=5e-5, g=3000.0)
    p = value_positions(inst, info)
    V = harmonic(p, inst.trap)
    psi = thomas_fermi(inst, info, V)
    # Ring vortex of radius R in the z = 0 plane: the phase winds once around the
    # ring's core circle (rho = R, z = 0).
    R = 3.0
    rho = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2)
    w = (rho - R) + 1j * p[..., 2]
    psi = psi * w / np.maximum(np.abs(w), 1e-12)
    return Condensate(inst, normalise(psi, _vol(inst, info)), V)


def config4(lattice: Lattice = Lattice.BCC2, count: int = 64, sizes=(24, 32, 48, 64, 96),
            dt: float = 1e-4, shard: int = 0, geometry: Optional[dict] = None) -> List[Condensate]:
    """The 64-condensate batch (seed 2).  shard > 0 gives another batch of the
    same sizes with its own g, traps and noise: one rank's part of a job of
    64 x ranks condensates, as heavy as shard 0."""
    info = _geom(lattice, geometry)
    mk = bcc2_instance if lattice == Lattice.BCC2 else tetra12_instance
    rng = np.random.default_rng(2)
    ns = rng.choice(np.asarray(sizes), size=count)
    if shard:
        rng = np.random.default_rng((2, shard))
    gs = np.exp(rng.uniform(math.log(100.0), math.log(5000.0), size=count))
    om = rng.uniform(0.5, 2.0, size=(count, 3))
    out = []
    for i in range(count):
        inst = mk(int(ns[i]), dt=dt, g=float(gs[i]), trap=tuple(float(w) ** 2 for w in om[i]))
        psi = gaussian_state(inst, info, rng, 1e-3)
        out.append(Condensate(inst, psi, None))
    return out


def config5(lattice: Lattice = Lattice.BCC2, geometry: Optional[dict] = None, n: int = 512) -> Condensate:
    info = _geom(lattice, geometry)
    mk = bcc2_instance if lattice == Lattice.BCC2 else tetra12_instance
    inst = mk(n, dt=2e-5, g=1e4)
    p = value_positions(inst, info)
    V = harmonic(p, inst.trap)
    psi = thomas_fermi(inst, info, V)
    rng = np.random.default_rng(3)
    psi = psi * np.exp(1j * 1e-2 * rng.standard_normal(psi.shape))
    return Condensate(inst, normalise(psi, _vol(inst, info)), V)


def odd_from_even(psi: np.ndarray, mu: float, dt: float) -> np.ndarray:
    """odd = even * exp(+i mu dt/2) (GPUGrossPitaevskii_BCC.cu:325,342)."""
    return psi * complex(math.cos(0.5 * mu * dt), math.sin(0.5 * mu * dt))


def shard_by_size(instances: Sequence, world: int) -> List[List[int]]:
    """Splits independent condensates over `world` ranks by size: largest first,
    each to the rank with the fewest values so far (ties to the lowest rank).
    Returns the instance indices of every rank, each list in ascending order."""
    load = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    order = sorted(range(len(instances)), key=lambda i: (-instances[i].nx * instances[i].ny * instances[i].nz, i))
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        inst = instances[i]
        load[r] += inst.nx * inst.ny * inst.nz
    return [sorted(p) for p in parts]
