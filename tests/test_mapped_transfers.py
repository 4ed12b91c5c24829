"""Transfers from and into mapped page-locked host memory: the conversion kernels
read and write such buffers in place (gpe_mapped_transfers counts them), other
buffers go through device staging.  Both paths must give the same fields, bit
for bit, in every storage, for single and batched calls, and a buffer that is
misaligned for the kernels' vector accesses must fall back to staging."""
import numpy as np
import pytest

from helpers import random_state
from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper

pytestmark = pytest.mark.gpu

DIMS = [(1, 1, 1), (5, 3, 7), (17, 9, 4), (33, 12, 6)]


def _insts():
    return [Instance(nx, ny, nz, 0.3 + 0.05 * k, 1e-3, 20.0 + k, origin=(-0.15 * nx, -0.15 * ny, -0.15 * nz))
            for k, (nx, ny, nz) in enumerate(DIMS)]


def _pinned(shape, dtype, offset_bytes=0):
    """A C-contiguous numpy view of page-locked memory (torch's pinned allocator),
    starting offset_bytes into the block."""
    import torch
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    blk = torch.empty(n + offset_bytes + 64, dtype=torch.uint8, pin_memory=True)
    a = blk.numpy()[offset_bytes:offset_bytes + n].view(dtype).reshape(shape)
    return a, blk  # the caller keeps blk alive while a is in use


CASES = [(Precision.FP32, Potential.ARRAY, None), (Precision.FP64, Potential.TRAP, None),
         (Precision.FP32C, Potential.TRAP, None), (Precision.FP32C, Potential.ARRAY, Precision.FP32)]


@pytest.mark.parametrize("prec,potential,host", CASES)
def test_mapped_buffers_equal_staged(prec, potential, host):
    insts = _insts()
    kw = dict(lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=potential)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    if host is not None:
        a.set_host_precision(host)
        b.set_host_precision(host)
    fdt = a.field_dtype
    vdt = np.float32 if prec != Precision.FP64 else np.float64
    rng = np.random.default_rng(5)
    keep = []
    staged, mapped = [], []
    for i in range(len(insts)):
        shp = a.shape(i)
        ze, zo = random_state(shp, 30 + i, 0.3), random_state(shp, 40 + i, 0.3)
        e = np.stack([ze.real, ze.imag], -1).astype(fdt)
        o = np.stack([zo.real, zo.imag], -1).astype(fdt)
        V = rng.uniform(0, 5, shp).astype(vdt) if potential == Potential.ARRAY else None
        pe, be = _pinned(e.shape, fdt)
        po, bo = _pinned(o.shape, fdt)
        pe[...] = e
        po[...] = o
        keep += [be, bo]
        pv = None
        if V is not None:
            pv, bv = _pinned(V.shape, vdt)
            pv[...] = V
            keep.append(bv)
        staged.append((i, e, o, V))
        mapped.append((i, pe, po, pv))
    # instance 0 by the single call, the rest batched
    a.upload(*staged[0])
    a.upload_many(staged[1:])
    b.upload(*mapped[0])
    b.upload_many(mapped[1:])
    n_up = b.mapped_transfers()
    assert a.mapped_transfers() == 0
    assert n_up == 2 * len(insts) + (len(insts) if potential == Potential.ARRAY else 0)
    a.step(5)
    b.step(5)
    want = [a.download(i) for i in range(len(insts))]
    outs = []
    for i in range(len(insts)):
        shp = a.shape(i) + (2,)
        pe, be = _pinned(shp, fdt)
        po, bo = _pinned(shp, fdt)
        keep += [be, bo]
        outs.append((pe, po))
    b.download_many(range(1, len(insts)), outs=outs[1:])
    e0, o0 = outs[0]
    assert b.lib.gpe_download(b.h, 0, e0.ctypes.data, o0.ctypes.data) == 0  # the single call, into pinned buffers
    b.synchronize()
    assert b.mapped_transfers() == n_up + 2 * len(insts)
    for (we, wo), (ge, go) in zip(want, outs):
        np.testing.assert_array_equal(ge, we)
        np.testing.assert_array_equal(go, wo)
    a.close()
    b.close()


def test_misaligned_mapped_buffer_falls_back_to_staging():
    insts = _insts()
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32, kernel=Kernel.FUSED, potential=Potential.TRAP)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    i = 3
    shp = a.shape(i) + (2,)
    z = random_state(a.shape(i), 7, 0.3)
    e = np.stack([z.real, z.imag], -1).astype(np.float32)
    pe, be = _pinned(shp, np.float32, offset_bytes=4)   # float pairs need 8-byte alignment
    pe[...] = e
    po, bo = _pinned(shp, np.float32, offset_bytes=64)  # aligned, inside the block
    po[...] = e[::-1].copy()
    a.upload(i, e, e[::-1].copy())
    b.upload(i, pe, po)
    assert b.mapped_transfers() == 1                    # the odd field only
    a.step(3)
    b.step(3)
    for f in (a, b):
        f.synchronize()
    want = a.download(i)
    got = b.download(i)
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])
    del be, bo
    a.close()
    b.close()


def test_mixed_mapped_and_pageable_batch():
    """Batched calls with some buffers mapped and some pageable: the mapped ones
    are converted in place, the rest staged, and the fields are the same."""
    insts = _insts()
    kw = dict(lattice=Lattice.BCC2, precision=Precision.FP32C, kernel=Kernel.FUSED, potential=Potential.TRAP)
    a, b = Stepper(insts, **kw), Stepper(insts, **kw)
    keep, staged, mixed = [], [], []
    for i in range(len(insts)):
        shp = a.shape(i)
        ze, zo = random_state(shp, 60 + i, 0.3), random_state(shp, 70 + i, 0.3)
        e = np.stack([ze.real, ze.imag], -1)
        o = np.stack([zo.real, zo.imag], -1)
        staged.append((i, e, o, None))
        if i % 2 == 0:  # even field pinned on even instances
            pe, be = _pinned(e.shape, np.float64)
            pe[...] = e
            keep.append(be)
            mixed.append((i, pe, o, None))
        else:
            mixed.append((i, e, o, None))
    a.upload_many(staged)
    b.upload_many(mixed)
    assert b.mapped_transfers() == (len(insts) + 1) // 2
    a.step(4)
    b.step(4)
    want = a.download_many(range(len(insts)))
    outs = []
    for i in range(len(insts)):
        shp = a.shape(i) + (2,)
        if i % 2:
            po, bo = _pinned(shp, np.float64)
            keep.append(bo)
            outs.append((np.empty(shp), po))
        else:
            outs.append((np.empty(shp), np.empty(shp)))
    b.download_many(range(len(insts)), outs=outs)
    assert b.mapped_transfers() == (len(insts) + 1) // 2 + len(insts) // 2
    for (we, wo), (ge, go) in zip(want, outs):
        np.testing.assert_array_equal(ge, we)
        np.testing.assert_array_equal(go, wo)
    a.close()
    b.close()
