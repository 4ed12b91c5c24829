"""Runs the REFERENCE's own update kernels through the CUDA driver API, compiled
unmodified for sm_103a by oracle/Makefile: GPUGrossPitaevskii_BCC.cu:176-216
(oracle/_ref/ref_bcc.cubin) and the Hodge form of GPUGrossPitaevskii_BCC_multi.cu:
329-397 (oracle/_ref/ref_multi.cubin), both under koodit/GrossPitaevskii.

Test infrastructure: lays out the reference's pitched BlockPsis/BlockPots arrays
(one padding block on every side, :269-287), builds its int2 neighbour table of
byte offsets from the reference's own getLaplacian output (tests/golden/
ref_tables.json), pre-scales the factors exactly as integrateInTime does
(:289-307) and launches update twice per step as its loop does (:475-481).
"""
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_bcc.cubin")
KERNEL = b"_Z6update10PitchedPtrS_S_P4int27double2d5uint3"  # update(PitchedPtr,PitchedPtr,PitchedPtr,int2*,double2,double,uint3)
BLOCK_PSIS = 12 * 16  # sizeof(BlockPsis)
BLOCK_POTS = 12 * 8   # sizeof(BlockPots)


class PitchedPtr(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("pitch", C.c_size_t), ("slicePitch", C.c_size_t)]


class Double2(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double)]


class UInt3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def available():
    return os.path.exists(CUBIN)


_drv = None


def _driver():
    global _drv
    if _drv is None:
        _drv = C.CDLL("libcuda.so.1")
    return _drv


def _ck(r, what):
    if r != 0:
        raise RuntimeError(f"{what} failed with CUresult {r}")


class ReferenceUpdate:
    """The reference kernel on one grid of X*Y*Z blocks (12 values each)."""

    cubin = CUBIN
    kernel = KERNEL

    def __init__(self, X, Y, Z):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        drv = _driver()
        self.mod = C.c_void_p()
        _ck(drv.cuModuleLoad(C.byref(self.mod), self.cubin.encode()), "cuModuleLoad")
        self.fn = C.c_void_p()
        _ck(drv.cuModuleGetFunction(C.byref(self.fn), self.mod, self.kernel), "cuModuleGetFunction")
        self.X, self.Y, self.Z = X, Y, Z
        # pitches as cudaMalloc3D would choose them (512-byte aligned rows)
        self.pitch = -(-(X + 2) * BLOCK_PSIS // 512) * 512
        self.slice = self.pitch * (Y + 2)
        self.ppitch = -(-(X + 2) * BLOCK_POTS // 512) * 512
        self.pslice = self.ppitch * (Y + 2)
        nbytes = self.slice * (Z + 2)
        self.even = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        self.odd = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        self.pot = torch.zeros(self.pslice * (Z + 2), dtype=torch.uint8, device="cuda")
        with open(os.path.join(HERE, "golden", "ref_tables.json")) as f:
            tab = json.load(f)
        # getLaplacian(ind, sizeof(BlockPsis), pitch, slicePitch): byte offset, slot
        ind = np.array([[dx * BLOCK_PSIS + dy * self.pitch + dz * self.slice, sl]
                        for dx, dy, dz, sl in tab["neighbours"]], dtype=np.int32)
        self.hodge = float(tab["hodge"])
        self.lapind = torch.from_numpy(ind.reshape(-1)).cuda()

    def _psi_ptr(self, t):
        return PitchedPtr(t.data_ptr() + self.slice + self.pitch + BLOCK_PSIS, self.pitch, self.slice)

    def _pack(self, t, host, rowbytes, pitch, slice_, block):
        """host: (Z, Y, X*block) bytes per row -> padded pitched device buffer."""
        buf = np.zeros(t.numel(), dtype=np.uint8)
        for z in range(self.Z):
            for y in range(self.Y):
                off = (z + 1) * slice_ + (y + 1) * pitch + block
                buf[off:off + rowbytes] = host[z, y]
        t.copy_(__import__("torch").from_numpy(buf))

    def upload(self, even, odd, pot_dt):
        """even/odd: float64 (Z, Y, X, 12, 2); pot_dt: V*dt, float64 (Z, Y, X, 12)."""
        X, Y, Z = self.X, self.Y, self.Z
        eb = np.ascontiguousarray(even, dtype=np.float64).view(np.uint8).reshape(Z, Y, X * BLOCK_PSIS)
        ob = np.ascontiguousarray(odd, dtype=np.float64).view(np.uint8).reshape(Z, Y, X * BLOCK_PSIS)
        pb = np.ascontiguousarray(pot_dt, dtype=np.float64).view(np.uint8).reshape(Z, Y, X * BLOCK_POTS)
        self._pack(self.even, eb, X * BLOCK_PSIS, self.pitch, self.slice, BLOCK_PSIS)
        self._pack(self.odd, ob, X * BLOCK_PSIS, self.pitch, self.slice, BLOCK_PSIS)
        self._pack(self.pot, pb, X * BLOCK_POTS, self.ppitch, self.pslice, BLOCK_POTS)

    def download(self):
        X, Y, Z = self.X, self.Y, self.Z
        out = []
        for t in (self.even, self.odd):
            buf = t.cpu().numpy()
            a = np.empty((Z, Y, X * BLOCK_PSIS), dtype=np.uint8)
            for z in range(Z):
                for y in range(Y):
                    off = (z + 1) * self.slice + (y + 1) * self.pitch + BLOCK_PSIS
                    a[z, y] = buf[off:off + X * BLOCK_PSIS]
            out.append(a.view(np.float64).reshape(Z, Y, X, 12, 2))
        return out

    def factors(self, block_scale, dt, g):
        """GPUGrossPitaevskii_BCC.cu:291-307, same operations in the same order."""
        lapfac = -0.5 * self.hodge / (block_scale * block_scale)
        lapfac0 = 4 * (-lapfac)
        return lapfac * dt, lapfac0 * dt, g * dt

    def step(self, steps, block_scale, dt, g, stream=0):
        lapfac, lapfac0, gdt = self.factors(block_scale, dt, g)
        drv = _driver()
        pot = PitchedPtr(self.pot.data_ptr() + self.pslice + self.ppitch + BLOCK_POTS, self.ppitch, self.pslice)
        lap = C.c_void_p(self.lapind.data_ptr())
        facs = Double2(lapfac, lapfac0)
        gg = C.c_double(gdt)
        dims = UInt3(self.X, self.Y, self.Z)
        ev, od = self._psi_ptr(self.even), self._psi_ptr(self.odd)
        gx, gy, gz = (self.X + 7) // 8, (self.Y + 7) // 8, self.Z
        for _ in range(steps):
            for nxt, prv in ((od, ev), (ev, od)):   # odd <- even, then even <- odd
                args = (C.c_void_p * 7)(*[C.cast(C.pointer(v), C.c_void_p) for v in
                                          (nxt, prv, pot, lap, facs, gg, dims)])
                _ck(drv.cuLaunchKernel(self.fn, gx, gy, gz, 8, 8, 12, 0, C.c_void_p(stream), args, None),
                    "cuLaunchKernel")
        _ck(drv.cuCtxSynchronize(), "cuCtxSynchronize")


MULTI_CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_multi.cubin")


def multi_available():
    return os.path.exists(MULTI_CUBIN)


class ReferenceHodgeUpdate(ReferenceUpdate):
    """The Hodge-form update of the reference's multi-GPU program
    (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi.cu:329-397), compiled
    unmodified for sm_103a by oracle/Makefile into oracle/_ref/ref_multi.cubin,
    on one GPU: the same pitched arrays, its own face tables (blockDirs,
    valueInds, hodges) scaled as its integrateInTime does (:476-483), and its
    launch shape, CTAs of 16 blocks x 12 values along x (:649-658)."""

    cubin = MULTI_CUBIN
    # update(PitchedPtr, PitchedPtr, PitchedPtr, int3*, int*, double*, double, uint3)
    kernel = b"_Z6update10PitchedPtrS_S_P4int3PiPdd5uint3"

    def step_faces(self, steps, table, block_scale, dt, g, stream=0):
        """`steps` leapfrog steps (odd <- even, then even <- odd, :816-881) with the
        48 face rows (dx, dy, dz, slot, hodge)."""
        import torch
        dirs = np.array([r[:3] for r in table], dtype=np.int32)
        slots = np.array([r[3] for r in table], dtype=np.int32)
        hodges = np.array([-0.5 * float(r[4]) / (block_scale * block_scale) * dt for r in table], dtype=np.float64)
        d_dirs = torch.from_numpy(dirs.reshape(-1)).cuda()
        d_slots = torch.from_numpy(slots).cuda()
        d_h = torch.from_numpy(hodges).cuda()
        drv = _driver()
        pot = PitchedPtr(self.pot.data_ptr() + self.pslice + self.ppitch + BLOCK_POTS, self.ppitch, self.pslice)
        pd, ps, ph = C.c_void_p(d_dirs.data_ptr()), C.c_void_p(d_slots.data_ptr()), C.c_void_p(d_h.data_ptr())
        gg = C.c_double(g * dt)
        dims = UInt3(self.X, self.Y, self.Z)
        ev, od = self._psi_ptr(self.even), self._psi_ptr(self.odd)
        gx, gy, gz = (self.X + 15) // 16, self.Y, self.Z
        for _ in range(steps):
            for nxt, prv in ((od, ev), (ev, od)):
                args = (C.c_void_p * 8)(*[C.cast(C.pointer(v), C.c_void_p) for v in
                                          (nxt, prv, pot, pd, ps, ph, gg, dims)])
                _ck(drv.cuLaunchKernel(self.fn, gx, gy, gz, 16 * 12, 1, 1, 0, C.c_void_p(stream), args, None),
                    "cuLaunchKernel")
        _ck(drv.cuCtxSynchronize(), "cuCtxSynchronize")
