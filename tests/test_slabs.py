"""z-slab domain decomposition (the reference's multi-GPU strategy,
koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi.cu:399-917): one condensate
cut along z into slabs that exchange their boundary planes after every
half-step evolves exactly as the undivided grid.

CPU: the oracle on gloo ranks (world size 2), each rank a slab with one ghost
plane per side, halo planes sent between ranks; bit-identical to the undivided
oracle.  GPU: SlabStepper (slabs of one batch, exchanged by the library) against
one Stepper on the whole grid, bit-identical, plain and fused kernels, and with
compensated storage (halo planes carry the FP32 values; residuals are needed
only where values are updated)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from helpers import interleave, random_state
from vaikkari_gb300.slabs import split_z


def test_split_z_balanced():
    for nz in (1, 7, 64, 97):
        for parts in range(1, min(nz, 9) + 1):
            c = split_z(nz, parts)
            assert sum(c) == nz and len(c) == parts and max(c) - min(c) <= 1 and min(c) >= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case(lattice_name, dims, seed):
    from oracle.lattice import tables
    from vaikkari_gb300.gpe import Lattice
    info = tables(Lattice[lattice_name])
    nx, ny, nz = dims
    shp = (nz, ny, nx, info["slots"])
    e = interleave(random_state(shp, seed, 0.3), np.float64)
    o = interleave(random_state(shp, seed + 1, 0.3), np.float64)
    v = np.ascontiguousarray(np.random.default_rng(seed).uniform(0, 0.01, shp))
    return info, e, o, v


def _slab_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    import oracle.oracle as orc
    dist.init_process_group("gloo", rank=rank, world_size=world)
    steps = 7
    import json
    with open(os.path.join(here, "golden", "ref_multi_tables.json")) as fh:
        table = [tuple(r) for r in json.load(fh)["faces"]]

    def make_grid(name, info, nx, ny, nz):
        if name == "FACES":   # the multi-GPU program's face form, its own table
            return orc.Faces(nx, ny, nz, table, 0.3, 1e-3, 50.0)
        return orc.Grid(nx, ny, nz, info["entry"], info["class_weight"], 0.3, 1e-3, 50.0)

    for name, dims in (("BCC2", (5, 4, 9)), ("TETRA12", (3, 3, 7)), ("FACES", (3, 3, 7))):
        lattice_name = "TETRA12" if name == "FACES" else name
        info, e, o, v = _case(lattice_name, dims, 11)
        nx, ny, nz = dims
        counts = split_z(nz, world)
        z0 = sum(counts[:rank])
        n = counts[rank]
        # the rank's slab with one ghost plane below and above
        def ext(a):
            g = np.zeros((n + 2,) + a.shape[1:], a.dtype)
            g[1:n + 1] = a[z0:z0 + n]
            return g
        fields = [ext(e), ext(o)]
        vext = ext(v)
        grid = make_grid(name, info, nx, ny, n + 2)

        def exchange(f):
            # send my boundary planes, receive the neighbours' into my ghosts
            reqs = []
            lo = torch.zeros(f[0].shape, dtype=torch.float64)
            hi = torch.zeros(f[0].shape, dtype=torch.float64)
            if rank > 0:
                reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(f[1])), rank - 1))
                reqs.append(dist.irecv(lo, rank - 1))
            if rank < world - 1:
                reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(f[n])), rank + 1))
                reqs.append(dist.irecv(hi, rank + 1))
            for r in reqs:
                r.wait()
            f[0] = lo.numpy()     # zero at the global boundary: Dirichlet
            f[n + 1] = hi.numpy()

        exchange(fields[0])
        exchange(fields[1])
        for _ in range(steps):
            for src in (0, 1):
                grid.half_step(fields[src], fields[1 - src], vext)
                exchange(fields[1 - src])
        mine = (fields[0][1:n + 1], fields[1][1:n + 1])
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        if rank == 0:
            ref = make_grid(name, info, nx, ny, nz)
            ref.leapfrog(e, o, v, steps)
            got_e = np.concatenate([g[0] for g in gathered])
            got_o = np.concatenate([g[1] for g in gathered])
            out[name] = (bool(np.array_equal(got_e, e)), bool(np.array_equal(got_o, o)), float(np.abs(e).max()))
    dist.barrier()
    dist.destroy_process_group()


def test_slab_halo_exchange_on_cpu_ranks_is_exact():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_slab_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    for name in ("BCC2", "TETRA12", "FACES"):
        same_e, same_o, scale = res[name]
        assert scale > 0.1          # the state did not decay to nothing
        assert same_e and same_o, name


# ---------------------------------------------------------------- GPU ---------

@pytest.mark.gpu
@pytest.mark.parametrize("lattice_name,precision,kernel,potential,slabs,steps", [
    ("BCC2", "FP32", "FUSED", "TRAP", 3, 250),
    ("BCC2", "FP64", "FUSED", "ARRAY", 2, 120),
    ("BCC2", "FP32", "PLAIN", "ARRAY", 4, 37),
    ("TETRA12", "FP64", "PLAIN", "ARRAY", 3, 130),
    ("BCC2", "FP32C", "FUSED", "TRAP", 3, 130),
])
def test_slab_stepper_equals_undivided_grid(lattice_name, precision, kernel, potential, slabs, steps):
    """Slabs of one batch with library-side halo exchange against the whole grid
    in one instance, bit for bit (graphs of 100 steps plus a remainder).  Block
    scale and origin are dyadic so that the trap's per-axis tables of a slab,
    made from its shifted origin, hold the same numbers as the whole grid's."""
    from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper
    from vaikkari_gb300.slabs import SlabStepper
    lat = Lattice[lattice_name]
    dims = (40, 24, 29) if lat == Lattice.BCC2 else (12, 10, 11)
    info, e, o, v = _case(lattice_name, dims, 21)
    inst = Instance(*dims, 0.25, 1e-3, 40.0, origin=(-5.0, -3.0, -3.5), trap=(1.0, 1.5, 0.5))
    kw = dict(lattice=lat, precision=Precision[precision], kernel=Kernel[kernel], potential=Potential[potential])
    dt = np.float32 if precision == "FP32" else np.float64
    pot = None if potential == "TRAP" else v
    whole = Stepper([inst], **kw)
    whole.upload(0, e.astype(dt), o.astype(dt), pot)
    whole.step(steps)
    we, wo = whole.download(0)
    whole.close()
    sl = SlabStepper(inst, slabs, **kw)
    sl.upload(e.astype(dt), o.astype(dt), pot)
    sl.step(steps)
    se, so = sl.download()
    obs = sl.observables()
    sl.close()
    assert np.abs(we).max() > 0.05
    np.testing.assert_array_equal(se, we)
    np.testing.assert_array_equal(so, wo)
    assert np.isfinite(obs["energy"]) and obs["norm"] > 0


@pytest.mark.gpu
def test_link_z_rejects_bad_links():
    from vaikkari_gb300.gpe import GpeError, Instance, Lattice, Mode, Stepper
    a = Instance(8, 8, 4, 0.25, 1e-3, 1.0)
    b = Instance(8, 6, 4, 0.25, 1e-3, 1.0)
    s = Stepper([a, a, b], lattice=Lattice.BCC2)
    with pytest.raises(GpeError):
        s.link_z(0, 2)              # different ny
    with pytest.raises(GpeError):
        s.link_z(1, 1)
    s.link_z(0, 1)
    with pytest.raises(GpeError):
        s.link_z(0, 1)              # one neighbour per side
    s.close()
    im = Stepper([a, a], lattice=Lattice.BCC2, mode=Mode.IMAGINARY)
    with pytest.raises(GpeError):
        im.link_z(0, 1)
    im.close()


def test_halo_slots_are_the_references_packing():
    """The slots a slab boundary exchanges are those the stencil reads across z:
    for TETRA12 {2, 6} from above and {0, 9, 10, 11} from below, the reference's
    packed halo (GPUGrossPitaevskii_BCC_MPI.cu:220-221); for BCC2 both slots."""
    from vaikkari_gb300.gpe import Lattice, lattice_info
    for lat, above, below in ((Lattice.TETRA12, [2, 6], [0, 9, 10, 11]), (Lattice.BCC2, [0, 1], [0, 1])):
        e = lattice_info(lat)["entry"]
        assert sorted({int(x[3]) for row in e for x in row if x[2] > 0}) == above
        assert sorted({int(x[3]) for row in e for x in row if x[2] < 0}) == below
