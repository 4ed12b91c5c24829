"""One condensate cut into z-slabs (the reference's domain decomposition,
koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi*.cu and _MPI.cu), each slab
an instance of one batch, neighbours linked so that the library exchanges
their boundary planes after every half-step.  On one GPU this runs the
decomposition's data flow end to end; the results equal the undivided grid's
bit for bit, which is what a multi-GPU split has to preserve.
"""
from __future__ import annotations

from dataclasses import replace
from typing import List

import numpy as np

from .gpe import Instance, Stepper


def split_z(nz: int, parts: int) -> List[int]:
    """Plane counts of `parts` slabs, as even as possible (the reference splits z
    the same way, GPUGrossPitaevskii_BCC_multi.cu:410-421)."""
    base, extra = divmod(nz, parts)
    return [base + (1 if k < extra else 0) for k in range(parts)]


class SlabStepper:
    def __init__(self, inst: Instance, slabs: int, **stepper_kw):
        if not 1 <= slabs <= inst.nz:
            raise ValueError("need 1 <= slabs <= nz")
        self.inst = inst
        self.counts = split_z(inst.nz, slabs)
        from .gpe import Lattice, lattice_info
        info = lattice_info(stepper_kw.get("lattice", Lattice.BCC2))
        edge = inst.block_scale * info["block_width"]
        parts, z0 = [], 0
        for n in self.counts:
            o = (inst.origin[0], inst.origin[1], inst.origin[2] + z0 * edge)
            parts.append(replace(inst, nz=n, origin=o))
            z0 += n
        self.starts = [sum(self.counts[:k]) for k in range(slabs)]
        self.stepper = Stepper(parts, **stepper_kw)
        for k in range(slabs - 1):
            self.stepper.link_z(k, k + 1)

    def upload(self, even, odd=None, potential=None):
        for k, (z0, n) in enumerate(zip(self.starts, self.counts)):
            sl = slice(z0, z0 + n)
            self.stepper.upload(k, even[sl], None if odd is None else odd[sl],
                                None if potential is None else potential[sl])

    def step(self, steps: int):
        self.stepper.step(steps)

    def download(self):
        parts = [self.stepper.download(k) for k in range(len(self.counts))]
        return np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts])

    def observables(self) -> dict:
        """Sums over the slabs (norm, kinetic, potential and interaction add)."""
        obs = self.stepper.observables(0)
        tot = {k: sum(o[k] for o in obs) for k in ("norm", "kinetic", "potential", "interaction")}
        tot["energy"] = tot["kinetic"] + tot["potential"] + tot["interaction"]
        tot["mu"] = (tot["kinetic"] + tot["potential"] + 2 * tot["interaction"]) / tot["norm"]
        return tot

    def close(self):
        self.stepper.close()
