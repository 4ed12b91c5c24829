"""The C-ABI library: loads, exports every function include/gpe.h declares, and
returns status codes (never exits) on bad input.  No GPU needed."""
import ctypes as C

import numpy as np
import os
import re
import subprocess

import pytest

from conftest import ROOT
from vaikkari_gb300 import gpe
from vaikkari_gb300.gpe import GpeError, Instance, Lattice, Status, Stepper


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(gpe_[a-z0-9_]+)\s*\(", txt))
    return names


def test_every_declared_symbol_is_exported():
    lib = gpe.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", gpe.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gpe_[a-z0-9_]+)$", out, flags=re.M))
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    for name in declared:
        getattr(lib, name)


def test_version_and_status_strings():
    lib = gpe.load_library()
    assert lib.gpe_abi_version() == 2
    for s in Status:
        assert lib.gpe_status_string(int(s))
    assert lib.gpe_status_string(999) == b"unknown status"


def test_invalid_arguments_return_status():
    lib = gpe.load_library()
    assert lib.gpe_create(None, None) == Status.INVALID_ARGUMENT
    assert b"null" in lib.gpe_last_error()
    assert lib.gpe_step(None, 1) == Status.INVALID_ARGUMENT
    assert lib.gpe_upload(None, 0, None, None, None) == Status.INVALID_ARGUMENT
    assert lib.gpe_destroy(None) == Status.OK
    assert lib.gpe_lattice_describe(7, None) == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        Stepper([Instance(0, 4, 4, 0.5, 1e-3, 1.0)])
    assert e.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        Stepper([Instance(4, 4, 4, -1.0, 1e-3, 1.0)])
    assert e.value.status == Status.INVALID_ARGUMENT
    with pytest.raises(GpeError) as e:
        Stepper([Instance(4, 4, 4, 0.5, 1e-3, 1.0)], lattice=Lattice.TETRA12, kernel=gpe.Kernel.FUSED,
                precision=gpe.Precision.FP64)  # the fused TETRA12 kernel is FP32 only
    assert e.value.status == Status.UNSUPPORTED
    with pytest.raises(GpeError) as e:
        Stepper([Instance(4, 4, 6000, 0.5, 1e-3, 1.0)], lattice=Lattice.TETRA12)
    assert e.value.status == Status.TOO_LARGE


def test_no_gpu_is_a_cuda_status_not_a_crash(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(GpeError) as e:
        Stepper([Instance(4, 4, 4, 0.5, 1e-3, 1.0)])
    assert e.value.status == Status.CUDA


def test_binding_rejects_wrong_shapes():
    """A raw pointer carries no size: the binding checks array shapes before the
    library copies nx*ny*nz*slots values from them."""
    st = Stepper.__new__(Stepper)
    st.instances = [Instance(4, 3, 2, 0.5, 1e-3, 1.0)]
    st.slots = 2
    st.dtype = st.field_dtype = np.float32
    shp = st.shape(0)
    assert shp == (2, 3, 4, 2)
    with pytest.raises(ValueError):
        st._carray(np.ones(shp), shp)           # real without the (re, im) axis
    with pytest.raises(ValueError):
        st._carray(np.ones((2, 3, 4, 3), complex), shp)
    with pytest.raises(ValueError):
        st._carray(np.ones(shp, complex), shp, complex_=False)
    a, p = st._carray(np.ones(shp, complex), shp)
    assert a.shape == shp + (2,) and a.dtype == np.float32
    a, p = st._carray(np.ones(shp), shp, complex_=False)
    assert a.shape == shp
    with pytest.raises(IndexError):
        st.shape(1)


def test_batched_transfer_bindings_check_arrays_first():
    """upload_many / download_many check every array before the library sees a
    pointer (no GPU needed: the checks raise before any call)."""
    st = Stepper.__new__(Stepper)
    st.instances = [Instance(4, 3, 2, 0.5, 1e-3, 1.0), Instance(2, 2, 2, 0.5, 1e-3, 1.0)]
    st.slots = 2
    st.dtype = st.field_dtype = np.float32
    shp0 = st.shape(0)
    with pytest.raises(ValueError):
        st.upload_many([(0, np.ones(shp0, complex), np.ones(st.shape(1), complex), None)])   # odd of the wrong size
    with pytest.raises(IndexError):
        st.upload_many([(2, np.ones(shp0, complex), None, None)])
    with pytest.raises(ValueError):
        st.download_many([0], outs=[(np.empty(shp0 + (2,), np.float64), None)])              # wrong element type
    with pytest.raises(ValueError):
        st.download_many([1], outs=[(np.empty(shp0 + (2,), np.float32), None)])              # wrong shape
    with pytest.raises(ValueError):
        st.download_many([0], outs=[(np.empty(shp0 + (2,), np.float32)[..., ::-1], None)])   # not contiguous


_C_CLIENT = r"""
#include "gpe.h"
#include <stdio.h>

int main(void)
{
    gpe_integrate_desc d = {0};
    d.block_scale = 0.5;
    for (int k = 0; k < 3; k++) { d.minp[k] = -2.0; d.maxp[k] = 2.0; }
    gpe_integrate_result r;
    if (gpe_integrate_grid(&d, &r) != GPE_OK) return 1;
    gpe_lattice_info info;
    if (gpe_lattice_describe(GPE_LATTICE_TETRA12, &info) != GPE_OK) return 2;
    gpe_face_table faces;
    for (int s = 0; s < 12; s++)
        for (int k = 0; k < 4; k++) {
            const int f = 4 * s + k;
            for (int a = 0; a < 3; a++) faces.dir[f][a] = info.entry[s][k][a];
            faces.slot[f] = info.entry[s][k][3];
            faces.hodge[f] = 1.5;
        }
    gpe_instance inst = {0};
    inst.nx = inst.ny = inst.nz = 4;
    inst.block_scale = 0.5;
    inst.dt = 1e-3;
    inst.g = 1.0;
    gpe_config cfg = {0};
    cfg.lattice = GPE_LATTICE_TETRA12;
    cfg.precision = GPE_FP64;
    cfg.kernel = GPE_KERNEL_PLAIN;
    cfg.num_instances = 1;
    cfg.instances = &inst;
    cfg.faces = &faces;
    gpe_handle h = 0;
    gpe_status s = gpe_create(&cfg, &h);
    printf("%d %u %u %u %llu\n", (int)s, r.xsize, r.ysize, r.zsize, (unsigned long long)r.values);
    if (s == GPE_OK) gpe_destroy(h);
    return 0;
}
"""


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_builds_and_links_as_c_and_cpp(tmp_path, lang):
    """include/gpe.h is plain C and C++: a client that fills a face table and
    asks for the solver call's grid compiles, links against the library and runs
    (gpe_create answers with a status; without a GPU that is GPE_ERR_CUDA)."""
    gpe.load_library()
    src = tmp_path / ("client.c" if lang == "c" else "client.cpp")
    src.write_text(_C_CLIENT)
    exe = tmp_path / "client"
    libdir = os.path.dirname(gpe.LIB_PATH)
    cc = ["gcc", "-std=c11"] if lang == "c" else ["g++", "-std=c++17"]
    subprocess.run(cc + ["-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                         "-L", libdir, "-lvaikkari_gpe", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    status, xs, ys, zs, values = (int(v) for v in out)
    assert status in (Status.OK, Status.CUDA)
    assert xs == ys == zs == int(4.0 / (0.5 * np.sqrt(8.0))) + 1 and values == 12 * xs * ys * zs
