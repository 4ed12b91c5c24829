"""Python binding of the CPU oracle (oracle/gpe_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, to check the library's results.  The product
never imports it.

It also restates, in numpy, how the reference turns a lattice and a time step
into the update's factors (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:
289-307: lapfac = -0.5*hodge/bs^2, lapfac0 = -(neighbours)*lapfac, both and g
and V multiplied by dt).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpe_oracle.so")


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("slots", C.c_int), ("neighbours", C.c_int),
                ("entry", C.POINTER(C.c_int)), ("Lc", C.c_double * 2), ("L0", C.c_double), ("gdt", C.c_double)]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        cc = os.environ.get("CC", "gcc")
        os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
        subprocess.run([cc, "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-fno-fast-math", os.path.join(HERE, "gpe_oracle.c"), os.path.join(HERE, "vortex_oracle.c"),
                        "-o", LIB_PATH, "-lm"], check=True)
    lib = C.CDLL(LIB_PATH)
    vp, dp = C.c_void_p, C.c_double
    G = C.POINTER(_Grid)
    lib.oracle_half_step_f64.argtypes = [G, vp, vp, vp, C.c_int, dp]
    lib.oracle_half_step_f32.argtypes = [G, vp, vp, vp, C.c_int, C.c_float]
    lib.oracle_half_step_bcc2_f64.argtypes = [G, vp, vp, vp, C.c_int, dp]
    lib.oracle_half_step_bcc2_f32.argtypes = [G, vp, vp, vp, C.c_int, C.c_float]
    lib.oracle_leapfrog_bcc2_f64.argtypes = [G, vp, vp, vp, C.c_long]
    lib.oracle_leapfrog_bcc2_f32.argtypes = [G, vp, vp, vp, C.c_long]
    lib.oracle_half_step_bcc2_f32c.argtypes = [G, vp, vp, vp, vp]
    lib.oracle_leapfrog_bcc2_f32c.argtypes = [G, vp, vp, vp, vp, vp, C.c_long]
    lib.oracle_leapfrog_bcc2_fast_f64.argtypes = [G, vp, vp, vp, C.c_long]
    lib.oracle_leapfrog_f64.argtypes = [G, vp, vp, vp, C.c_long]
    lib.oracle_leapfrog_f32.argtypes = [G, vp, vp, vp, C.c_long]
    lib.oracle_observables_f64.argtypes = [G, vp, vp, dp, dp, vp, vp]
    lib.oracle_observables_f32.argtypes = [G, vp, vp, dp, dp, vp, vp]
    lib.oracle_imaginary_f64.argtypes = [G, vp, vp, vp, dp, dp, vp, dp, C.c_long, dp, vp]
    lib.oracle_imaginary_f64.restype = C.c_long
    ci = C.c_int
    lib.oracle_half_step_faces_f64.argtypes = [ci, ci, ci, vp, vp, dp, vp, vp, vp, ci, dp]
    lib.oracle_half_step_faces_f32.argtypes = [ci, ci, ci, vp, vp, C.c_float, vp, vp, vp, ci, C.c_float]
    lib.oracle_leapfrog_faces_f64.argtypes = [ci, ci, ci, vp, vp, dp, vp, vp, vp, C.c_long]
    lib.oracle_leapfrog_faces_f32.argtypes = [ci, ci, ci, vp, vp, C.c_float, vp, vp, vp, C.c_long]
    ui, ul = C.c_uint, C.c_long
    lib.oracle_vortex_initial.argtypes = [ui, dp, dp, ui, dp, vp]
    lib.oracle_vortex_resample.argtypes = [vp, ui, ui, dp, dp, dp, vp, ui, ui, dp, dp, dp]
    lib.oracle_vortex_iterate.argtypes = [vp, ui, ui, dp, dp, dp, ui, dp, dp, C.POINTER(dp), ul, dp, C.c_int,
                                          C.c_int, C.POINTER(dp)]
    lib.oracle_vortex_iterate.restype = ul
    lib.oracle_vortex_function_max.argtypes = [vp, C.c_size_t]
    lib.oracle_vortex_function_max.restype = dp
    lib.oracle_vortex_min_r.argtypes = [vp, ui, ui, dp, dp, dp]
    lib.oracle_vortex_min_r.restype = dp
    lib.oracle_set_threads.argtypes = [C.c_int]
    lib.oracle_get_threads.restype = C.c_int
    _lib = lib
    return lib


def set_threads(n: int):
    load().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(load().oracle_get_threads())


def factors(class_weight, entry_classes, block_scale, dt, g):
    """Update factors as the reference computes them (GPUGrossPitaevskii_BCC.cu:291-307),
    one per weight class: Lc = -0.5*w_c/bs^2*dt, L0 = (0.5*sum_c n_c*w_c/bs^2)*dt
    (n_c = neighbours in class c; the reference's lapfac0 = 4*(-lapfac)), gdt = g*dt."""
    w = [cw / (block_scale * block_scale) for cw in class_weight]
    Lc = [-0.5 * wc * dt for wc in w] + [0.0] * (2 - len(w))
    counts = [sum(1 for c in entry_classes if c == k) for k in range(len(w))]
    wsum = counts[0] * w[0]
    if len(w) > 1:
        wsum = wsum + counts[1] * w[1]
    L0 = (0.5 * wsum) * dt
    return {"Lc": Lc, "L0": L0, "gdt": g * dt, "w": w + [0.0] * (2 - len(w))}


def comp_unit(hi):
    """The residual unit of stored FP32 values: ulp(hi)/256 = 2^(E - 31 - 127) for
    the biased exponent E of hi, E raised to 32 below 2^-95 (float32)."""
    e = np.asarray(hi, np.float32).view(np.uint32) & np.uint32(0x7F800000)
    e = np.maximum(e, np.uint32(32 << 23))
    return (e - np.uint32(31 << 23)).astype(np.uint32).view(np.float32)


def comp_encode(r, hi):
    """int8 residuals: r / unit(hi) rounded to nearest even, clipped to +-127."""
    q = np.rint(np.asarray(r, np.float32) / comp_unit(hi))
    return np.clip(q, -127, 127).astype(np.int8)


def comp_decode(q, hi):
    """float32 value of int8 residuals q of stored values hi."""
    return np.asarray(q, np.int8).astype(np.float32) * comp_unit(hi)


def split_comp(x):
    """Compensated storage of float64 values: hi = float32(x), lo = the int8
    residual of float32(x - hi) (comp_encode)."""
    x = np.asarray(x, np.float64)
    hi = x.astype(np.float32)
    return hi, comp_encode((x - hi.astype(np.float64)).astype(np.float32), hi)


def join_comp(hi, lo):
    """float64(hi) + float64(residual): the value a compensated field stands for."""
    return hi.astype(np.float64) + comp_decode(lo, hi).astype(np.float64)


class Grid:
    """A grid of nx*ny*nz blocks with a neighbour table entry[slot][k] = (dx,dy,dz,slot,class)."""

    def __init__(self, nx, ny, nz, entry, class_weight, block_scale, dt, g):
        self.entry = np.ascontiguousarray(np.asarray(entry, dtype=np.int32))
        self.slots, self.neighbours = self.entry.shape[0], self.entry.shape[1]
        f = factors(class_weight, [int(c) for c in self.entry[0, :, 4]], block_scale, dt, g)
        self.Lc, self.L0, self.gdt, self.w = f["Lc"], f["L0"], f["gdt"], f["w"]
        self.dt, self.g = dt, g
        self.nx, self.ny, self.nz = nx, ny, nz
        self._w = np.array(self.w, dtype=np.float64)
        self._g = _Grid(nx, ny, nz, self.slots, self.neighbours,
                        self.entry.ctypes.data_as(C.POINTER(C.c_int)), (C.c_double * 2)(*self.Lc), self.L0,
                        self.gdt)

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx, self.slots)

    def _p(self, a):
        return a.ctypes.data_as(C.c_void_p)

    def half_step(self, prev, next_, vdt, mode=0, sigma=1.0):
        lib = load()
        if prev.dtype == np.float64:
            lib.oracle_half_step_f64(C.byref(self._g), self._p(prev), self._p(next_), self._p(vdt), mode, sigma)
        else:
            lib.oracle_half_step_f32(C.byref(self._g), self._p(prev), self._p(next_), self._p(vdt), mode,
                                     C.c_float(sigma))

    def leapfrog(self, even, odd, vdt, steps):
        """In place: `steps` leapfrog steps (GPUGrossPitaevskii_BCC.cu:475-481)."""
        lib = load()
        for a in (even, odd, vdt):
            assert a.flags.c_contiguous
        fn = lib.oracle_leapfrog_f64 if even.dtype == np.float64 else lib.oracle_leapfrog_f32
        fn(C.byref(self._g), self._p(even), self._p(odd), self._p(vdt), int(steps))

    def leapfrog_bcc2(self, even, odd, vdt, steps):
        """In place, BCC2 only, in the fused GPU kernel's summation order."""
        lib = load()
        assert self.slots == 2 and self.neighbours == 14
        for a in (even, odd, vdt):
            assert a.flags.c_contiguous
        fn = lib.oracle_leapfrog_bcc2_f64 if even.dtype == np.float64 else lib.oracle_leapfrog_bcc2_f32
        fn(C.byref(self._g), self._p(even), self._p(odd), self._p(vdt), int(steps))

    def leapfrog_bcc2_comp(self, even, odd, even_lo, odd_lo, vdt, steps):
        """In place, BCC2, FP32 with compensated storage: even/odd float32
        (..., 2), even_lo/odd_lo int8 (..., 2) residuals (split_comp)."""
        lib = load()
        assert self.slots == 2 and even.dtype == np.float32 and even_lo.dtype == np.int8
        for a in (even, odd, even_lo, odd_lo, vdt):
            assert a.flags.c_contiguous
        lib.oracle_leapfrog_bcc2_f32c(C.byref(self._g), self._p(even), self._p(odd), self._p(even_lo),
                                      self._p(odd_lo), self._p(vdt), int(steps))

    def leapfrog_bcc2_fast(self, even, odd, vdt, steps):
        """FP64, BCC2: the box-order leapfrog with direct interior indexing (bit-identical)."""
        lib = load()
        assert self.slots == 2 and even.dtype == np.float64
        for a in (even, odd, vdt):
            assert a.flags.c_contiguous
        lib.oracle_leapfrog_bcc2_fast_f64(C.byref(self._g), self._p(even), self._p(odd), self._p(vdt), int(steps))

    def observables(self, psi, vdt, vol):
        lib = load()
        out = np.zeros(4)
        fn = lib.oracle_observables_f64 if psi.dtype == np.float64 else lib.oracle_observables_f32
        fn(C.byref(self._g), self._p(psi), self._p(vdt), self.dt, self.g, self._p(self._w), self._p(out))
        norm, kin, pot, inter = vol * out
        return {"norm": norm, "kinetic": kin, "potential": pot, "interaction": inter,
                "energy": kin + pot + inter, "mu": (kin + pot + 2 * inter) / norm}

    def imaginary(self, psi, vdt, vol, steps, tol):
        lib = load()
        work = np.zeros_like(psi)
        mu = np.zeros(max(int(steps), 1))
        conv = lib.oracle_imaginary_f64(C.byref(self._g), self._p(psi), self._p(work), self._p(vdt), self.dt,
                                        self.g, self._p(self._w), vol, int(steps), tol, self._p(mu))
        return int(conv), mu[: int(steps)]


class Vortex:
    """The axisymmetric vortex state f(r, z) of VortexState.cpp: rsize x zsize
    values, row i at r = rplug + i*rstep, column j at z = j*zstep."""

    def __init__(self, kappa, g, rsize, zsize, rplug, rstep, zstep, mu=1.0, f=None):
        self.kappa, self.g = int(kappa), float(g)
        self.rsize, self.zsize = int(rsize), int(zsize)
        self.rplug, self.rstep, self.zstep, self.mu = float(rplug), float(rstep), float(zstep), float(mu)
        self.f = np.zeros(self.rsize * self.zsize) if f is None else np.ascontiguousarray(f, dtype=np.float64)

    @classmethod
    def from_range(cls, kappa, g, rmin, rmax, zmax, rstep, zstep):
        """setKappa/setG/setRange with setDimensions' initial state (VortexState.cpp:12-47)."""
        rsize0 = int((rmax - rmin) / rstep + 0.5)
        zsize0 = int(zmax / zstep + 0.5)
        if rsize0 == 0 or zsize0 == 0:
            raise ValueError("range shorter than half a step")
        rs = max((rmax - rmin) / rsize0, 1e-13)
        zs = max(zmax / zsize0, 1e-13)
        rsize, zsize = max(rsize0, 1), max(zsize0, 1)
        v = cls(kappa, g, rsize, zsize, max(rmin, 0.0), rs, zs, 1.0)
        load().oracle_vortex_initial(rsize, rs, v.rplug, zsize, zs, v.f.ctypes.data_as(C.c_void_p))
        return v

    @classmethod
    def from_file(cls, path):
        """The binary format of VortexState::load (VortexState.cpp:49-72)."""
        import struct
        raw = open(path, "rb").read()
        kappa, g, rsize, zsize, rplug, rstep, zstep, mu = struct.unpack_from("<IdIIdddd", raw, 0)
        f = np.frombuffer(raw, dtype="<f8", count=rsize * zsize, offset=struct.calcsize("<IdIIdddd"))
        return cls(kappa, g, rsize, zsize, rplug, rstep, zstep, mu, f.copy())

    def initialize(self, src):
        """initialize(state) (VortexState.cpp:98-107): mu and a bilinear resampling of src."""
        self.mu = src.mu
        load().oracle_vortex_resample(src.f.ctypes.data_as(C.c_void_p), src.rsize, src.zsize, src.rplug, src.rstep,
                                      src.zstep, self.f.ctypes.data_as(C.c_void_p), self.rsize, self.zsize,
                                      self.rplug, self.rstep, self.zstep)

    def iterate(self, maxiters, eps=1e-29, ratio=0.1, order=0, chunk=16):
        """iterateSolution (VortexState.cpp:109-185) with potentialRZ; returns (iterations, last diff)."""
        mu = C.c_double(self.mu)
        diff = C.c_double(0.0)
        its = load().oracle_vortex_iterate(self.f.ctypes.data_as(C.c_void_p), self.rsize, self.zsize, self.rplug,
                                           self.rstep, self.zstep, self.kappa, self.g, ratio, C.byref(mu),
                                           int(maxiters), eps, int(order), int(chunk), C.byref(diff))
        self.mu = mu.value
        return int(its), diff.value

    def function_max(self):
        return load().oracle_vortex_function_max(self.f.ctypes.data_as(C.c_void_p), self.f.size)

    def min_r(self, eps):
        return load().oracle_vortex_min_r(self.f.ctypes.data_as(C.c_void_p), self.rsize, self.zsize, self.rplug,
                                          self.rstep, eps)

    def max_r(self, eps):
        idx = np.nonzero(self.f > eps)[0]
        return self.rplug + (int(idx[-1]) // self.zsize) * self.rstep if idx.size else 0.0

    def max_z(self, eps):
        cols = np.nonzero((self.f.reshape(self.rsize, self.zsize) > eps).any(axis=0))[0]
        return int(cols[-1]) * self.zstep if cols.size else 0.0


# The face order of the reference's multi-GPU update kernel: position k of slot s
# takes face 4*s + FACE_PERM[s][k] of its getLaplacian table
# (GPUGrossPitaevskii_BCC_multi.cu:314-327).
FACE_PERM = ((3, 2, 0, 1), (2, 0, 1, 3), (1, 0, 2, 3), (1, 0, 2, 3), (2, 0, 1, 3), (3, 1, 0, 2),
             (0, 1, 2, 3), (0, 1, 2, 3), (3, 1, 0, 2), (2, 3, 0, 1), (2, 3, 0, 1), (3, 2, 0, 1))


class Faces:
    """The face (Hodge) form of GPUGrossPitaevskii_BCC_multi.cu:329-397 on an
    nx*ny*nz grid of 12-slot blocks.  `table` is the reference's getLaplacian
    output, 48 rows (dx, dy, dz, slot, hodge) for face f = 4*slot + k; the weights
    are scaled as integrateInTime does (:483), -0.5 * hodge / bs^2 * dt, and the
    faces summed in FACE_PERM order."""

    def __init__(self, nx, ny, nz, table, block_scale, dt, g):
        self.nx, self.ny, self.nz = nx, ny, nz
        face, h = [], []
        for s in range(12):
            for k in range(4):
                row = table[4 * s + FACE_PERM[s][k]]
                face.extend(int(v) for v in row[:4])
                h.append(-0.5 * float(row[4]) / (block_scale * block_scale) * dt)
        self.face = np.array(face, dtype=np.int32)
        self.h = np.array(h, dtype=np.float64)
        self.h32 = self.h.astype(np.float32)
        self.gdt = g * dt

    def _args(self, dtype):
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        if dtype == np.float64:
            return (self.nx, self.ny, self.nz, p(self.face), p(self.h), self.gdt)
        return (self.nx, self.ny, self.nz, p(self.face), p(self.h32), float(np.float32(self.gdt)))

    def half_step(self, prev, next_, vdt, mode=0, sigma=1.0):
        lib = load()
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        fn = lib.oracle_half_step_faces_f64 if prev.dtype == np.float64 else lib.oracle_half_step_faces_f32
        fn(*self._args(prev.dtype), p(prev), p(next_), p(vdt), mode, sigma)

    def leapfrog(self, even, odd, vdt, steps):
        """In place: `steps` leapfrog steps, odd <- even then even <- odd."""
        lib = load()
        for a in (even, odd, vdt):
            assert a.flags.c_contiguous and a.dtype == even.dtype
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        fn = lib.oracle_leapfrog_faces_f64 if even.dtype == np.float64 else lib.oracle_leapfrog_faces_f32
        fn(*self._args(even.dtype), p(even), p(odd), p(vdt), int(steps))
