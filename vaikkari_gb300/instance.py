"""Plain descriptions of condensates: the lattice kinds, one instance's grid and
physics, and the positions of its values.  Pure Python and numpy: importing
this module loads no native code, so seeded workloads can be described (and
checked on the CPU) without the library.  vaikkari_gb300.gpe re-exports all
three names.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass
from typing import Sequence

import numpy as np


class Lattice(enum.IntEnum):
    TETRA12 = 0  # reference discretisation: 12 circumcentre values per block, 4 faces
    BCC2 = 1     # 2 lattice-point values per block, 14 Hodge-weighted edges


@dataclass
class Instance:
    """One condensate: nx*ny*nz blocks of the lattice; see include/gpe.h."""
    nx: int
    ny: int
    nz: int
    block_scale: float
    dt: float
    g: float
    origin: Sequence[float] = (0.0, 0.0, 0.0)
    trap: Sequence[float] = (1.0, 1.0, 1.0)

    def c(self):
        """The C struct gpe_instance (needs the library's ctypes layout)."""
        from .gpe import _Instance
        s = _Instance()
        s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
        s.block_scale, s.dt, s.g = self.block_scale, self.dt, self.g
        for k in range(3):
            s.origin[k] = self.origin[k]
            s.trap[k] = self.trap[k]
        return s


def value_positions(inst: Instance, info: dict) -> np.ndarray:
    """Positions of every value of an instance, shape (nz, ny, nx, slots, 3), in
    the reference's block order (GPUGrossPitaevskii_BCC.cu:258); `info` gives
    the lattice's block width and value positions (in block_scale units)."""
    bw = info["block_width"]
    i = np.arange(inst.nx)[None, None, :, None]
    j = np.arange(inst.ny)[None, :, None, None]
    k = np.arange(inst.nz)[:, None, None, None]
    pos = np.asarray(info["position"])
    out = np.empty((inst.nz, inst.ny, inst.nx, info["slots"], 3))
    out[..., 0] = inst.origin[0] + inst.block_scale * (i * bw + pos[None, None, None, :, 0])
    out[..., 1] = inst.origin[1] + inst.block_scale * (j * bw + pos[None, None, None, :, 1])
    out[..., 2] = inst.origin[2] + inst.block_scale * (k * bw + pos[None, None, None, :, 2])
    return out
