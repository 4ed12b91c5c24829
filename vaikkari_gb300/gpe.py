"""ctypes binding of the C ABI in include/gpe.h (libvaikkari_gpe.so).

This is the host-side mirror of the reference's solver call,
``integrateInTime(state, block_scale, minp, maxp, iteration_period,
number_of_iterations)`` (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC.cu:218):
a :class:`Stepper` owns the device fields of one or many condensates, takes host
arrays in the reference's block order, advances them with the GB300 kernels and
returns fields and FP64 observables.  Every failing call raises
:class:`GpeError` carrying the library's status and message (the reference
exits the process instead, helper_cuda.h checkCudaErrors).

There is no CPU fallback: if the native library is missing the import of the
library raises.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from typing import List, Optional

import numpy as np

from .instance import Instance, Lattice, value_positions  # noqa: F401  (re-exported)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvaikkari_gpe.so")


class Precision(enum.IntEnum):
    FP64 = 0
    FP32 = 1
    # FP32 fields with an int8 residual per component (units of ulp/256) carried
    # across real-time steps (BCC2, fused kernel); fields are exchanged as float64.
    FP32C = 2


class Mode(enum.IntEnum):
    REAL = 0
    IMAGINARY = 1


class Kernel(enum.IntEnum):
    AUTO = 0
    PLAIN = 1
    FUSED = 2


class Potential(enum.IntEnum):
    ARRAY = 0
    TRAP = 1


class Status(enum.IntEnum):
    OK = 0
    INVALID_ARGUMENT = 1
    CUDA = 2
    OUT_OF_MEMORY = 3
    NOT_FINITE = 4
    UNSUPPORTED = 5
    TOO_LARGE = 6
    INTERNAL = 7
    TIMEOUT = 8


class GpeError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = Status(status) if status in Status._value2member_map_ else status
        super().__init__(f"{self.status!r}: {message}")


class _LatticeInfo(C.Structure):
    _fields_ = [
        ("lattice", C.c_int32), ("slots", C.c_int32), ("neighbours", C.c_int32), ("classes", C.c_int32),
        ("block_width", C.c_double), ("cell_volume", C.c_double), ("class_weight", C.c_double * 2),
        ("position", (C.c_double * 3) * 12), ("entry", ((C.c_int32 * 5) * 14) * 12),
    ]


class _Instance(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("block_scale", C.c_double), ("origin", C.c_double * 3), ("dt", C.c_double), ("g", C.c_double),
        ("trap", C.c_double * 3),
    ]


class _Config(C.Structure):
    _fields_ = [
        ("lattice", C.c_int32), ("precision", C.c_int32), ("mode", C.c_int32), ("kernel", C.c_int32),
        ("potential", C.c_int32), ("num_instances", C.c_int32), ("instances", C.POINTER(_Instance)),
        ("graph_steps", C.c_int32), ("tile", C.c_int32), ("zchunk", C.c_int32), ("device", C.c_int32),
        ("faces", C.c_void_p),
    ]


class _FaceTable(C.Structure):
    _fields_ = [("dir", (C.c_int32 * 3) * 48), ("slot", C.c_int32 * 48), ("hodge", C.c_double * 48)]


def face_table(rows):
    """gpe_face_table from 48 rows (dx, dy, dz, slot, hodge), face f = 4*slot + k:
    the reference multi-GPU program's getLaplacian output
    (GPUGrossPitaevskii_BCC_multi.cu:73-271)."""
    rows = list(rows)
    if len(rows) != 48:
        raise ValueError("a face table has 48 rows (dx, dy, dz, slot, hodge)")
    t = _FaceTable()
    for f, r in enumerate(rows):
        for a in range(3):
            t.dir[f][a] = int(r[a])
        t.slot[f] = int(r[3])
        t.hodge[f] = float(r[4])
    return t


def default_face_table(weight=None):
    """The TETRA12 graph as a face table in this library's neighbour order, every
    weight the lattice's Hodge weight (1.5) unless `weight` is given."""
    info = lattice_info(Lattice.TETRA12)
    w = float(info["class_weight"][0]) if weight is None else float(weight)
    return [(*(int(v) for v in info["entry"][s][k][:4]), w) for s in range(12) for k in range(4)]


class _Observables(C.Structure):
    _fields_ = [
        ("norm", C.c_double), ("energy", C.c_double), ("mu", C.c_double), ("kinetic", C.c_double),
        ("potential", C.c_double), ("interaction", C.c_double), ("finite", C.c_int32), ("pad_", C.c_int32),
    ]


class _VortexInfo(C.Structure):
    _fields_ = [("kappa", C.c_uint32), ("rsize", C.c_uint32), ("zsize", C.c_uint32), ("pad_", C.c_uint32),
                ("g", C.c_double), ("mu", C.c_double), ("rplug", C.c_double), ("rstep", C.c_double),
                ("zstep", C.c_double), ("function_max", C.c_double), ("max_r", C.c_double), ("max_z", C.c_double),
                ("curvature", C.c_double), ("block_scale", C.c_double), ("min_r", C.c_double)]


class _RelaxDesc(C.Structure):
    _fields_ = [("maxiters", C.c_uint32), ("graph_iterations", C.c_uint32), ("eps", C.c_double),
                ("ratio", C.c_double), ("device", C.c_int32), ("pad_", C.c_int32)]


class _RelaxResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("pad_", C.c_uint32), ("diff", C.c_double), ("mu", C.c_double),
                ("device_ms", C.c_double)]


class _IntegrateDesc(C.Structure):
    _fields_ = [("block_scale", C.c_double), ("minp", C.c_double * 3), ("maxp", C.c_double * 3),
                ("iteration_period", C.c_double), ("number_of_iterations", C.c_uint32), ("seed", C.c_uint32),
                ("ratio", C.c_double), ("noise", C.c_double), ("precision", C.c_int32), ("device", C.c_int32)]


class _IntegrateResult(C.Structure):
    _fields_ = [("xsize", C.c_uint32), ("ysize", C.c_uint32), ("zsize", C.c_uint32),
                ("steps_per_iteration", C.c_uint32), ("values", C.c_uint64), ("p0", C.c_double * 3),
                ("maxpot", C.c_double), ("dt", C.c_double), ("lapfac_dt", C.c_double), ("lapfac0_dt", C.c_double),
                ("g_dt", C.c_double), ("odd_phase", C.c_double * 2), ("device_ms", C.c_double),
                ("setup_ms", C.c_double)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads (once) and returns the native library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"native library not built: {path} (run `python -m vaikkari_gb300.build`)")
    lib = C.CDLL(path)
    st = C.c_int
    lib.gpe_abi_version.restype = C.c_int32
    lib.gpe_status_string.restype = C.c_char_p
    lib.gpe_status_string.argtypes = [st]
    lib.gpe_last_error.restype = C.c_char_p
    lib.gpe_lattice_describe.restype = st
    lib.gpe_lattice_describe.argtypes = [C.c_int32, C.POINTER(_LatticeInfo)]
    lib.gpe_create.restype = st
    lib.gpe_create.argtypes = [C.POINTER(_Config), C.POINTER(C.c_void_p)]
    lib.gpe_destroy.restype = st
    lib.gpe_destroy.argtypes = [C.c_void_p]
    lib.gpe_upload.restype = st
    lib.gpe_upload.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gpe_download.restype = st
    lib.gpe_download.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    vpp = C.POINTER(C.c_void_p)
    lib.gpe_upload_many.restype = st
    lib.gpe_upload_many.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), vpp, vpp, vpp]
    lib.gpe_download_many.restype = st
    lib.gpe_download_many.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), vpp, vpp]
    lib.gpe_step.restype = st
    lib.gpe_step.argtypes = [C.c_void_p, C.c_int64]
    lib.gpe_round_trip.restype = st
    lib.gpe_round_trip.argtypes = [C.c_void_p, vpp, vpp, C.c_int64, vpp, vpp, C.POINTER(_Observables)]
    lib.gpe_synchronize.restype = st
    lib.gpe_synchronize.argtypes = [C.c_void_p]
    lib.gpe_observables_get.restype = st
    lib.gpe_observables_get.argtypes = [C.c_void_p, C.c_int32, C.POINTER(_Observables)]
    lib.gpe_imaginary_time.restype = st
    lib.gpe_imaginary_time.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    lib.gpe_launch_count.restype = C.c_int64
    lib.gpe_launch_count.argtypes = [C.c_void_p]
    lib.gpe_mapped_transfers.restype = C.c_int64
    lib.gpe_mapped_transfers.argtypes = [C.c_void_p]
    lib.gpe_stream.restype = C.c_void_p
    lib.gpe_stream.argtypes = [C.c_void_p]
    lib.gpe_time_steps.restype = st
    lib.gpe_time_steps.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float)]
    lib.gpe_variant_half_steps.restype = C.c_int32
    lib.gpe_variant_half_steps.argtypes = [C.c_int32]
    lib.gpe_set_host_precision.restype = st
    lib.gpe_set_host_precision.argtypes = [C.c_void_p, C.c_int32]
    lib.gpe_variant_kind.restype = C.c_int32
    lib.gpe_variant_kind.argtypes = [C.c_int32]
    lib.gpe_link_z.restype = st
    lib.gpe_link_z.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.gpe_debug_inject.restype = st
    lib.gpe_debug_inject.argtypes = [C.c_void_p, C.c_int32]
    lib.gpe_variant_count.restype = C.c_int32
    lib.gpe_variant_describe.restype = st
    lib.gpe_variant_describe.argtypes = [C.c_int32] + [C.POINTER(C.c_int32)] * 4
    lib.gpe_vortex_load.restype = st
    lib.gpe_vortex_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    lib.gpe_vortex_free.restype = None
    lib.gpe_vortex_free.argtypes = [C.c_void_p]
    lib.gpe_vortex_describe.restype = st
    lib.gpe_vortex_describe.argtypes = [C.c_void_p, C.c_double, C.POINTER(_VortexInfo)]
    lib.gpe_vortex_create.restype = st
    lib.gpe_vortex_create.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.POINTER(C.c_void_p)]
    lib.gpe_vortex_initialize.restype = st
    lib.gpe_vortex_initialize.argtypes = [C.c_void_p, C.c_void_p]
    lib.gpe_vortex_save.restype = st
    lib.gpe_vortex_save.argtypes = [C.c_void_p, C.c_char_p]
    lib.gpe_vortex_values.restype = st
    lib.gpe_vortex_values.argtypes = [C.c_void_p, C.c_void_p]
    lib.gpe_vortex_relax.restype = st
    lib.gpe_vortex_relax.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(_RelaxDesc),
                                     C.POINTER(_RelaxResult)]
    lib.gpe_debug_divide.restype = st
    lib.gpe_debug_divide.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]
    lib.gpe_vortex_psi.restype = st
    lib.gpe_vortex_psi.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.gpe_integrate_setup.restype = st
    lib.gpe_integrate_setup.argtypes = [C.c_void_p, C.POINTER(_IntegrateDesc), C.POINTER(_IntegrateResult),
                                        C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gpe_integrate_grid.restype = st
    lib.gpe_integrate_grid.argtypes = [C.POINTER(_IntegrateDesc), C.POINTER(_IntegrateResult)]
    lib.gpe_integrate_in_time.restype = st
    lib.gpe_integrate_in_time.argtypes = [C.c_void_p, C.POINTER(_IntegrateDesc), C.POINTER(_IntegrateResult),
                                          C.POINTER(_Observables), C.c_void_p, C.c_void_p]
    lib.gpe_volume_map.restype = st
    lib.gpe_volume_map.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_void_p]
    lib.gpe_slice_rgb.restype = st
    lib.gpe_slice_rgb.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p]
    lib.gpe_write_metaimage.restype = st
    lib.gpe_write_metaimage.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                        C.POINTER(C.c_double)]
    lib.gpe_write_bmp.restype = st
    lib.gpe_write_bmp.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32]
    lib.gpe_observables_noalloc.restype = st
    lib.gpe_observables_noalloc.argtypes = [C.c_int32, C.c_int32, C.POINTER(_Instance), C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.POINTER(_Observables)]
    _lib = lib
    return lib


def _check(status: int, what: str):
    if status != 0:
        msg = _lib.gpe_last_error().decode(errors="replace")
        raise GpeError(status, f"{what}: {msg}")


def lattice_info(lattice: Lattice) -> dict:
    """Stencil tables of a lattice (replaces getLaplacian/getPositions,
    GPUGrossPitaevskii_BCC.cu:69-142)."""
    lib = load_library()
    info = _LatticeInfo()
    _check(lib.gpe_lattice_describe(int(lattice), C.byref(info)), "gpe_lattice_describe")
    ns, nb = info.slots, info.neighbours
    entry = np.array([[list(info.entry[s][k]) for k in range(nb)] for s in range(ns)], dtype=np.int32)
    return {
        "lattice": Lattice(info.lattice), "slots": ns, "neighbours": nb, "classes": info.classes,
        "block_width": info.block_width, "cell_volume": info.cell_volume,
        "class_weight": [info.class_weight[0], info.class_weight[1]][: info.classes],
        "position": np.array([list(info.position[s]) for s in range(ns)]),
        "entry": entry,
    }


def observables_noalloc(lattice: Lattice, precision: Precision, inst: "Instance", field_ptr: int,
                        potential_ptr: int = 0, stream: int = 0) -> dict:
    """Observables of one condensate that already sits in device memory, without
    any allocation (gpe_observables_noalloc).  For callers that cannot allocate
    device memory: field_ptr / potential_ptr are device addresses of the
    condensate's values and potential in block order; potential_ptr = 0 uses the
    instance's harmonic trap.  Calls that overlap on one GPU share scratch memory
    and must not run concurrently."""
    lib = load_library()
    out = _Observables()
    c = inst.c()
    _check(lib.gpe_observables_noalloc(int(lattice), int(precision), C.byref(c), C.c_void_p(field_ptr),
                                       C.c_void_p(potential_ptr or None), C.c_void_p(stream or None), C.byref(out)),
           "gpe_observables_noalloc")
    return {k: getattr(out, k) for k in ("norm", "energy", "mu", "kinetic", "potential", "interaction")}


def variants() -> List[dict]:
    """The fused kernel's variants (gpe_config.tile values)."""
    lib = load_library()
    out = []
    for v in range(lib.gpe_variant_count()):
        t = [C.c_int32() for _ in range(4)]
        _check(lib.gpe_variant_describe(v, *[C.byref(x) for x in t]), "gpe_variant_describe")
        out.append({"tile": v, "tx": t[0].value, "ty": t[1].value, "stages": t[2].value, "min_blocks": t[3].value,
                    "half_steps": lib.gpe_variant_half_steps(v), "kind": lib.gpe_variant_kind(v),
                    "persistent": lib.gpe_variant_kind(v) == 2})
    return out


def write_metaimage(path: str, vol: np.ndarray, spacing) -> None:
    """MetaImage header `path` and data `path`.raw (gpe_write_metaimage); vol
    shape (dz, dy, dx) uint16."""
    lib = load_library()
    vol = np.ascontiguousarray(vol, dtype=np.uint16)
    sp = (C.c_double * 3)(*spacing)
    _check(lib.gpe_write_metaimage(path.encode(), vol.ctypes.data_as(C.c_void_p), vol.shape[2], vol.shape[1],
                                   vol.shape[0], sp), "gpe_write_metaimage")


def write_bmp(path: str, rgb: np.ndarray) -> None:
    """24-bit BMP (gpe_write_bmp); rgb shape (height, width, 3) uint8, row 0 first."""
    lib = load_library()
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    _check(lib.gpe_write_bmp(path.encode(), rgb.ctypes.data_as(C.c_void_p), rgb.shape[1], rgb.shape[0]),
           "gpe_write_bmp")


class Stepper:
    """Device state of a batch of condensates (wraps gpe_create/gpe_destroy)."""

    def __init__(self, instances: List[Instance], lattice=Lattice.BCC2, precision=Precision.FP32,
                 mode=Mode.REAL, kernel=Kernel.AUTO, potential=Potential.ARRAY, graph_steps=0, tile=0,
                 zchunk=0, device=0, faces=None):
        """faces: TETRA12 only, 48 rows (dx, dy, dz, slot, hodge) of the reference
        multi-GPU program's table; the update then takes its face (Hodge) form."""
        self.lib = load_library()
        self.instances = list(instances)
        self.lattice, self.precision, self.mode = Lattice(lattice), Precision(precision), Mode(mode)
        self.potential = Potential(potential)
        self.info = lattice_info(self.lattice)
        self.slots = self.info["slots"]
        self._carr = (_Instance * len(self.instances))(*[i.c() for i in self.instances])
        cfg = _Config()
        cfg.lattice, cfg.precision, cfg.mode = int(lattice), int(precision), int(mode)
        cfg.kernel, cfg.potential = int(kernel), int(potential)
        cfg.num_instances = len(self.instances)
        cfg.instances = C.cast(self._carr, C.POINTER(_Instance))
        cfg.graph_steps, cfg.tile, cfg.zchunk, cfg.device = graph_steps, tile, zchunk, device
        self.faces = None if faces is None else [tuple(r) for r in faces]
        if faces is not None:
            self._faces = face_table(faces)
            cfg.faces = C.cast(C.pointer(self._faces), C.c_void_p)
        h = C.c_void_p()
        _check(self.lib.gpe_create(C.byref(cfg), C.byref(h)), "gpe_create")
        self.h = h
        self.dtype = np.float64 if self.precision == Precision.FP64 else np.float32
        # element type of host field arrays (GPE_FP32C exchanges fields as double)
        self.field_dtype = np.float64 if self.precision != Precision.FP32 else np.float32

    # -- helpers ------------------------------------------------------------
    def shape(self, i: int):
        if not 0 <= i < len(self.instances):
            raise IndexError(f"instance {i} out of range")
        inst = self.instances[i]
        return (inst.nz, inst.ny, inst.nx, self.slots)

    def _carray(self, a, shape, complex_=True):
        """Host array in the handle's element type (fields: field_dtype); complex
        fields may be given as complex (shape) or interleaved real (shape + (2,))."""
        if a is None:
            return None, None
        a = np.asarray(a)
        if complex_:
            if np.iscomplexobj(a):
                a = np.stack([a.real, a.imag], axis=-1)
            want = tuple(shape) + (2,)
        else:
            if np.iscomplexobj(a):
                raise ValueError("the potential must be real")
            want = tuple(shape)
        if a.shape != want:
            raise ValueError(f"array shape {a.shape} does not match {want} "
                             "(block order (nz, ny, nx, slots), complex or interleaved (..., 2))")
        a = np.ascontiguousarray(a, dtype=self.field_dtype if complex_ else self.dtype)
        return a, a.ctypes.data_as(C.c_void_p)

    # -- API ----------------------------------------------------------------
    def set_host_precision(self, precision):
        """Element type of host field arrays: Precision.FP64 (default for FP32C)
        or Precision.FP32 (FP32C only: float in, float out; gpe_set_host_precision)."""
        _check(self.lib.gpe_set_host_precision(self.h, int(precision)), "gpe_set_host_precision")
        self.field_dtype = np.float64 if Precision(precision) == Precision.FP64 else np.float32

    def upload(self, i: int, even, odd=None, potential=None):
        """even/odd: complex arrays (nz, ny, nx, slots) or real (..., 2); potential: V (unscaled)."""
        shp = self.shape(i)
        e, pe = self._carray(even, shp)
        o, po = self._carray(odd, shp)
        v, pv = self._carray(potential, shp, complex_=False)
        _check(self.lib.gpe_upload(self.h, i, pe, po, pv), "gpe_upload")

    def download(self, i: int, odd: bool = True):
        shp = self.shape(i) + (2,)
        e = np.empty(shp, self.field_dtype)
        o = np.empty(shp, self.field_dtype) if odd else None
        _check(self.lib.gpe_download(self.h, i, e.ctypes.data_as(C.c_void_p),
                                     o.ctypes.data_as(C.c_void_p) if odd else None), "gpe_download")
        return e, o

    def upload_many(self, items):
        """items: (instance, even, odd, potential) tuples; one gpe_upload_many
        call (every copy queued, one wait at the end)."""
        keep, idx, pe, po, pv = [], [], [], [], []
        for i, even, odd, potential in items:
            shp = self.shape(i)
            e, p_e = self._carray(even, shp)
            o, p_o = self._carray(odd, shp)
            v, p_v = self._carray(potential, shp, complex_=False)
            keep += [e, o, v]
            idx.append(int(i))
            pe.append(p_e)
            po.append(p_o)
            pv.append(p_v)
        n = len(idx)
        arr = lambda xs: (C.c_void_p * n)(*[x.value if x is not None else None for x in xs])
        _check(self.lib.gpe_upload_many(self.h, n, (C.c_int32 * n)(*idx), arr(pe), arr(po), arr(pv)),
               "gpe_upload_many")

    def download_many(self, indices, outs=None, odd: bool = True):
        """Fields of several instances in one gpe_download_many call.  outs:
        optional (even, odd) arrays to fill (e.g. pinned); returns the list."""
        indices = [int(i) for i in indices]
        if outs is None:
            outs = []
            for i in indices:
                shp = self.shape(i) + (2,)
                outs.append((np.empty(shp, self.field_dtype), np.empty(shp, self.field_dtype) if odd else None))
        for i, (e, o) in zip(indices, outs):
            want = self.shape(i) + (2,)
            for a in (e, o):
                if a is not None and (a.shape != want or a.dtype != self.field_dtype or not a.flags.c_contiguous):
                    raise ValueError(f"output array for instance {i} must be C-contiguous {self.field_dtype} {want}")
        n = len(indices)
        pe = (C.c_void_p * n)(*[e.ctypes.data for e, _ in outs])
        po = (C.c_void_p * n)(*[o.ctypes.data if o is not None else None for _, o in outs])
        _check(self.lib.gpe_download_many(self.h, n, (C.c_int32 * n)(*indices), pe, po), "gpe_download_many")
        return outs

    def step(self, steps: int):
        _check(self.lib.gpe_step(self.h, int(steps)), "gpe_step")

    def round_trip(self, inputs, steps: int, outs=None, observables: bool = True):
        """gpe_round_trip: upload every instance, `steps` steps, the observables
        of field 0, download.  inputs: one (even, odd) pair per instance in the
        host element type (odd may be None in imaginary time); outs: (even, odd)
        arrays to fill (None entries are not downloaded; default: new arrays).
        Returns (outs, observables list or None)."""
        n = len(self.instances)
        if len(inputs) != n:
            raise ValueError(f"round_trip takes one input pair per instance ({n})")
        keep, pe, po = [], [], []
        for i, (even, odd) in enumerate(inputs):
            shp = self.shape(i)
            e, p_e = self._carray(even, shp)
            o, p_o = self._carray(odd, shp)
            keep += [e, o]
            pe.append(p_e)
            po.append(p_o)
        if outs is None:
            outs = [(np.empty(self.shape(i) + (2,), self.field_dtype), np.empty(self.shape(i) + (2,), self.field_dtype))
                    for i in range(n)]
        for i, (e, o) in enumerate(outs):
            want = self.shape(i) + (2,)
            for a in (e, o):
                if a is not None and (a.shape != want or a.dtype != self.field_dtype or not a.flags.c_contiguous):
                    raise ValueError(f"output array for instance {i} must be C-contiguous {self.field_dtype} {want}")
        arr = lambda xs: (C.c_void_p * n)(*[x.value if x is not None else None for x in xs])
        oe = (C.c_void_p * n)(*[e.ctypes.data if e is not None else None for e, _ in outs])
        oo = (C.c_void_p * n)(*[o.ctypes.data if o is not None else None for _, o in outs])
        obs = (_Observables * n)() if observables else None
        st = self.lib.gpe_round_trip(self.h, arr(pe), arr(po) if any(x is not None for x in po) else None,
                                     int(steps), oe, oo, obs)
        res = None
        if observables:
            res = [{k: getattr(o, k) for k in ("norm", "energy", "mu", "kinetic", "potential", "interaction")}
                   | {"finite": bool(o.finite)} for o in obs]
        _check(st, "gpe_round_trip")
        return outs, res

    def synchronize(self):
        _check(self.lib.gpe_synchronize(self.h), "gpe_synchronize")

    def observables(self, field_: int = 0) -> List[dict]:
        n = len(self.instances)
        arr = (_Observables * n)()
        st = self.lib.gpe_observables_get(self.h, field_, arr)
        out = [{k: getattr(o, k) for k in ("norm", "energy", "mu", "kinetic", "potential", "interaction")}
               | {"finite": bool(o.finite)} for o in arr]
        _check(st, "gpe_observables_get")
        return out

    def imaginary_time(self, max_steps: int, tol: float):
        steps = C.c_int64()
        conv = C.c_int32()
        mu = (C.c_double * len(self.instances))()
        _check(self.lib.gpe_imaginary_time(self.h, int(max_steps), float(tol), C.byref(steps), C.byref(conv), mu),
               "gpe_imaginary_time")
        return steps.value, bool(conv.value), list(mu)

    def time_steps(self, steps: int) -> float:
        """Device milliseconds of `steps` steps, timed with CUDA events on the
        library's stream (gpe_time_steps)."""
        ms = C.c_float()
        _check(self.lib.gpe_time_steps(self.h, int(steps), C.byref(ms)), "gpe_time_steps")
        return float(ms.value)

    def link_z(self, lower: int, upper: int):
        """Instance `upper` continues `lower` along +z; halos exchanged every half-step."""
        _check(self.lib.gpe_link_z(self.h, int(lower), int(upper)), "gpe_link_z")

    def debug_inject(self, plane: int):
        """Test hook: make the fused kernel's bounded wait run out (see gpe.h)."""
        _check(self.lib.gpe_debug_inject(self.h, int(plane)), "gpe_debug_inject")

    def volume_map(self, i: int, unit: float, field_: int = 0, reference_sum: bool = False) -> np.ndarray:
        """Per-block density volume over the padded block grid, uint16, shape
        (nz+2, ny+2, nx+2) (gpe_volume_map)."""
        inst = self.instances[i]
        out = np.empty((inst.nz + 2, inst.ny + 2, inst.nx + 2), dtype=np.uint16)
        _check(self.lib.gpe_volume_map(self.h, i, field_, float(unit), int(reference_sum),
                                       out.ctypes.data_as(C.c_void_p)), "gpe_volume_map")
        return out

    def slice_rgb(self, i: int, z_padded: int, slot: int = 0, gain: float = 5.0, field_: int = 0) -> np.ndarray:
        """RGB image of one block plane, shape (ny+2, nx+2, 3) (gpe_slice_rgb)."""
        inst = self.instances[i]
        out = np.empty((inst.ny + 2, inst.nx + 2, 3), dtype=np.uint8)
        _check(self.lib.gpe_slice_rgb(self.h, i, field_, int(z_padded), int(slot), float(gain),
                                      out.ctypes.data_as(C.c_void_p)), "gpe_slice_rgb")
        return out

    def launch_count(self) -> int:
        return int(self.lib.gpe_launch_count(self.h))

    def mapped_transfers(self) -> int:
        """Host buffers converted in place (mapped page-locked memory, no staging copy)."""
        return int(self.lib.gpe_mapped_transfers(self.h))

    def stream_handle(self) -> int:
        """The cudaStream_t the library launches on (as an integer)."""
        return int(self.lib.gpe_stream(self.h) or 0)

    def total_values(self) -> int:
        return sum(i.nx * i.ny * i.nz for i in self.instances) * self.slots

    def close(self):
        if getattr(self, "h", None):
            st = self.lib.gpe_destroy(self.h)
            self.h = None
            _check(st, "gpe_destroy")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VortexState:
    """A vortex state file in the reference's VortexState format, and the
    reference's solver call on it (integrateInTime, GPUGrossPitaevskii_BCC.cu:218)."""

    def __init__(self, path: str = None, _handle=None):
        self.lib = load_library()
        if _handle is not None:
            self.h = _handle
            return
        h = C.c_void_p()
        _check(self.lib.gpe_vortex_load(path.encode(), C.byref(h)), "gpe_vortex_load")
        self.h = h

    @classmethod
    def create(cls, kappa: int, g: float, rmin: float, rmax: float, zmax: float, rstep: float, zstep: float):
        """setKappa/setG/setRange with the initial profile (VortexState.cpp:12-47)."""
        lib = load_library()
        h = C.c_void_p()
        _check(lib.gpe_vortex_create(int(kappa), g, rmin, rmax, zmax, rstep, zstep, C.byref(h)), "gpe_vortex_create")
        return cls(_handle=h)

    def initialize(self, src: "VortexState"):
        """initialize(src) (VortexState.cpp:98-107)."""
        _check(self.lib.gpe_vortex_initialize(self.h, src.h), "gpe_vortex_initialize")

    def save(self, path: str):
        _check(self.lib.gpe_vortex_save(self.h, path.encode()), "gpe_vortex_save")

    def values(self) -> np.ndarray:
        """f as an array (rsize, zsize)."""
        d = self.describe()
        f = np.empty((d["rsize"], d["zsize"]))
        _check(self.lib.gpe_vortex_values(self.h, f.ctypes.data_as(C.c_void_p)), "gpe_vortex_values")
        return f

    def relax(self, maxiters: int = 10000, eps: float = 1e-29, **kw) -> dict:
        """iterateSolution(potentialRZ, maxiters, eps) on the GPU (VortexState.cpp:109-185)."""
        return relax([self], maxiters, eps, **kw)[0]

    def describe(self, eps_fraction: float = 1e-5) -> dict:
        info = _VortexInfo()
        _check(self.lib.gpe_vortex_describe(self.h, eps_fraction, C.byref(info)), "gpe_vortex_describe")
        return {k: getattr(info, k) for k, _ in _VortexInfo._fields_ if k != "pad_"}

    def psi(self, p) -> complex:
        pp = (C.c_double * 3)(*p)
        out = (C.c_double * 2)()
        _check(self.lib.gpe_vortex_psi(self.h, pp, out), "gpe_vortex_psi")
        return complex(out[0], out[1])

    @staticmethod
    def _desc(block_scale, minp, maxp, iteration_period=1.0, number_of_iterations=1, seed=54363, ratio=0.1,
              noise=0.01, precision=Precision.FP64, device=0):
        d = _IntegrateDesc()
        d.block_scale, d.iteration_period = block_scale, iteration_period
        d.number_of_iterations, d.seed, d.ratio, d.noise = number_of_iterations, seed, ratio, noise
        d.precision, d.device = int(precision), device
        for k in range(3):
            d.minp[k], d.maxp[k] = minp[k], maxp[k]
        return d

    @staticmethod
    def _res(r: _IntegrateResult) -> dict:
        out = {k: getattr(r, k) for k, _ in _IntegrateResult._fields_}
        out["p0"] = list(r.p0)
        out["odd_phase"] = list(r.odd_phase)
        return out

    def grid(self, block_scale, minp, maxp, **kw):
        """The grid integrateInTime builds (sizes, values, p0), without sampling."""
        d = self._desc(block_scale, minp, maxp, **kw)
        r = _IntegrateResult()
        _check(self.lib.gpe_integrate_grid(C.byref(d), C.byref(r)), "gpe_integrate_grid")
        return self._res(r)

    def setup(self, block_scale, minp, maxp, **kw):
        """integrateInTime's host set-up: (result, even, odd, V) with fields in
        block order, shape (zsize, ysize, xsize, 12, 2)."""
        d = self._desc(block_scale, minp, maxp, **kw)
        r = _IntegrateResult()
        _check(self.lib.gpe_integrate_grid(C.byref(d), C.byref(r)), "gpe_integrate_grid")
        shp = (r.zsize, r.ysize, r.xsize, 12)
        even = np.empty(shp + (2,))
        odd = np.empty(shp + (2,))
        V = np.empty(shp)
        _check(self.lib.gpe_integrate_setup(self.h, C.byref(d), C.byref(r), even.ctypes.data_as(C.c_void_p),
                                            odd.ctypes.data_as(C.c_void_p), V.ctypes.data_as(C.c_void_p)),
               "gpe_integrate_setup")
        return self._res(r), even, odd, V

    def integrate_in_time(self, block_scale, minp, maxp, iteration_period=1.0, number_of_iterations=1, **kw):
        """The reference's solver call on the GPU.  Returns (result, observables
        per iteration, final even, final odd)."""
        d = self._desc(block_scale, minp, maxp, iteration_period, number_of_iterations, **kw)
        r = _IntegrateResult()
        _check(self.lib.gpe_integrate_grid(C.byref(d), C.byref(r)), "gpe_integrate_grid")
        shp = (r.zsize, r.ysize, r.xsize, 12, 2)
        even = np.empty(shp)
        odd = np.empty(shp)
        obs = (_Observables * (number_of_iterations + 1))()
        _check(self.lib.gpe_integrate_in_time(self.h, C.byref(d), C.byref(r), obs, even.ctypes.data_as(C.c_void_p),
                                              odd.ctypes.data_as(C.c_void_p)), "gpe_integrate_in_time")
        ob = [{k: getattr(o, k) for k in ("norm", "energy", "mu", "kinetic", "potential", "interaction")}
              for o in obs]
        return self._res(r), ob, even, odd

    def close(self):
        if getattr(self, "h", None):
            self.lib.gpe_vortex_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def relax(states: List["VortexState"], maxiters: int = 10000, eps: float = 1e-29, ratio: float = 0.1,
          graph_iterations: int = 0, device: int = 0) -> List[dict]:
    """iterateSolution for several independent vortex states in one GPU call
    (gpe_vortex_relax); every state is updated in place."""
    lib = load_library()
    d = _RelaxDesc()
    d.maxiters, d.graph_iterations, d.eps, d.ratio, d.device = int(maxiters), int(graph_iterations), eps, ratio, \
        int(device)
    n = len(states)
    hs = (C.c_void_p * n)(*[s.h.value if isinstance(s.h, C.c_void_p) else s.h for s in states])
    res = (_RelaxResult * n)()
    _check(lib.gpe_vortex_relax(hs, n, C.byref(d), res), "gpe_vortex_relax")
    return [{"iterations": r.iterations, "diff": r.diff, "mu": r.mu, "device_ms": r.device_ms} for r in res]


def debug_divide(a: np.ndarray, b: np.ndarray, device: int = 0):
    """The relaxation sweep's division and __ddiv_rn on the GPU (test hook)."""
    lib = load_library()
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    assert a.shape == b.shape
    ours, ref = np.empty_like(a), np.empty_like(a)
    _check(lib.gpe_debug_divide(a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                ours.ctypes.data_as(C.c_void_p), ref.ctypes.data_as(C.c_void_p), a.size, device),
           "gpe_debug_divide")
    return ours, ref
