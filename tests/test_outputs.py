"""Field outputs against the files the reference's own writers produced
(tests/golden/ref_slice_small.bmp, ref_volume_small.mhd/.raw: Picture::save and
saveVolumeMap on the even field of the small integrateInTime set-up)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from vaikkari_gb300 import gpe
from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper


def _setup_even():
    s = golden("ref_setup_small.json")
    n = s["xsize"] * s["ysize"] * s["zsize"] * 12
    raw = np.fromfile(os.path.join(GOLDEN, "ref_setup_small.bin"), dtype=np.float64)
    return s, raw[:2 * n].reshape(s["zsize"], s["ysize"], s["xsize"], 12, 2)


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


def _compare(tmp_path, vol, rgb, spacing):
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        gpe.write_metaimage("ref_volume_small.mhd", vol, spacing)
        gpe.write_bmp("ref_slice_small.bmp", rgb)
    finally:
        os.chdir(cwd)
    for name in ("ref_volume_small.mhd", "ref_volume_small.mhd.raw", "ref_slice_small.bmp"):
        assert _bytes(os.path.join(tmp_path, name)) == _bytes(os.path.join(GOLDEN, name)), name


def _host_outputs(s, even, unit, k):
    """The same per-block/per-pixel arithmetic, on the host."""
    Z, Y, X = s["zsize"], s["ysize"], s["xsize"]
    pad = np.zeros((Z + 2, Y + 2, X + 2, 12, 2))
    pad[1:-1, 1:-1, 1:-1] = even
    x0, y0 = pad[..., 0, 0], pad[..., 0, 1]
    d0 = x0 * x0 + y0 * y0
    acc = np.zeros_like(d0)
    for _ in range(12):
        acc = acc + d0
    acc = acc * unit
    vol = np.where(acc > 65535.0, 65535, np.trunc(acc)).astype(np.uint16)
    x, y = pad[k, :, :, 0, 0], pad[k, :, :, 0, 1]
    norm = np.sqrt(x * x + y * y)
    rgb = np.stack([256.0 * (5.0 * x), 256.0 * (5.0 * norm), 256.0 * (5.0 * y)], -1)
    rgb = np.where(rgb < 1.0, 0, np.where(rgb > 255.0, 255, np.trunc(rgb))).astype(np.uint8)
    return vol, rgb


def test_writers_reproduce_reference_files(tmp_path):
    s, even = _setup_even()
    o = golden("ref_outputs_small.json")
    vol, rgb = _host_outputs(s, even, o["unit"], o["slice_k"])
    _compare(tmp_path, vol, rgb, [s["block_scale"] * 8 ** 0.5] * 3)


@pytest.mark.gpu
def test_device_outputs_reproduce_reference_files(tmp_path):
    s, even = _setup_even()
    o = golden("ref_outputs_small.json")
    inst = Instance(s["xsize"], s["ysize"], s["zsize"], s["block_scale"], s["dt"], 1.0, origin=s["p0"])
    st = Stepper([inst], lattice=Lattice.TETRA12, precision=Precision.FP64, kernel=Kernel.PLAIN,
                 potential=Potential.TRAP)
    st.upload(0, even, even)
    vol = st.volume_map(0, o["unit"], reference_sum=True)
    rgb = st.slice_rgb(0, o["slice_k"], slot=0, gain=5.0)
    host_vol, host_rgb = _host_outputs(s, even, o["unit"], o["slice_k"])
    np.testing.assert_array_equal(vol, host_vol)
    np.testing.assert_array_equal(rgb, host_rgb)
    total = st.volume_map(0, o["unit"], reference_sum=False)   # the block's full density
    assert total.shape == vol.shape
    st.close()
    _compare(tmp_path, vol, rgb, [s["block_scale"] * 8 ** 0.5] * 3)
