"""Benchmark: vertex-updates/s of the GPE stepper on one GB300 (or N ranks).

Default workload (the batched configuration the headline metric is quoted on):
64 independent condensates on the BCC2 lattice, grid edge per instance uniform
over {24, 32, 48, 64, 96} cells (seed 2), g log-uniform in [100, 5000], trap
frequencies per axis uniform in [0.5, 2], Gaussian initial state with 1e-3
noise, dt = 1e-4; FP32 storage and arithmetic, trap potential evaluated in the
kernel, one fused launch per half-step for the whole batch, CUDA graphs of 100
steps.  One bench step = one leapfrog step (two half-steps) of every instance.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Multi-GPU: the condensates are independent, so
each rank advances its own shard with no collective on the data path; value =
all ranks' vertex-updates / max-over-ranks time.  --scaling weak (default): 64
condensates per rank, same sizes, own g / trap / noise; rank 0 holds the batch
above.  --scaling strong: the batch above split over the ranks by size.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertex-updates/s"
BYTES_PER_VERTEX_STEP = 48  # FP32, trap potential in-kernel: 2 half-steps x (read prev 8 B + RMW next 16 B)
BYTES_PER_VERTEX_STEP_COMP = 56  # FP32C: plus the next field's int8 x 2 residual, read and written (2 x 4 B)
L2_BYTES = 129e6
HEADLINE_WORKLOAD = "batch64_bcc2_trap_realtime"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_traffic(name):
    """DRAM bytes per launch of a kernel from a committed ncu summary under
    profiles/, with the kernel variant the capture ran (lines
    `traffic_bytes_per_launch_full_batch:` and `traffic_variant:`)."""
    p = os.path.join(ROOT, "profiles", name)
    out = {"bytes": None, "variant": None, "source": f"profiles/{name}"}
    if not os.path.exists(p):
        return out
    for line in open(p):
        key, _, val = line.partition(":")
        try:
            if key == "traffic_bytes_per_launch_full_batch":
                out["bytes"] = float(val.strip())
            elif key == "traffic_variant":
                out["variant"] = int(val.strip())
        except ValueError:
            pass
    return out


def roofline_block(verts, bytes_per_vertex_step, steps, window_s, launches, kernel, profile, variant):
    """Roofline of the dominant kernel, the only kernel in the timed window:
    achieved = algorithmic bytes per launch / average launch duration, i.e. the
    window's algorithmic bytes (vertices x bytes per vertex-step x steps) over
    the window's device time (CUDA events), whether the window holds two
    launches per step or one persistent launch; traffic from the ncu summary of
    the same kernel variant on this workload (null if the profiled variant
    differs)."""
    peak, peak_kind = _peaks()
    window_bytes = verts * bytes_per_vertex_step * steps
    achieved = window_bytes / window_s / 1e9
    prof = _profile_traffic(profile)
    same = prof["variant"] == variant
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": prof["bytes"] if same else None,
            "traffic_source": (f"ncu capture summarised in {prof['source']} (variant {prof['variant']}, "
                               f"full batch, one launch)" if same else
                               f"none for variant {variant}: {prof['source']} holds variant {prof['variant']}"),
            "algorithmic_bytes_per_vertex_step": bytes_per_vertex_step,
            "algorithmic_bytes_per_launch": window_bytes / max(launches, 1), "launches_per_window": launches,
            "peak_source": f"{peak_kind} hbm_gbs (of {peak_kind})", "kernel": kernel}


class ClockSampler:
    """nvidia-smi clock/throttle sampling (every 100 ms) around the run; the
    summary covers the samples taken inside the timed region (between
    start_region() and end_region())."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []  # (perf_counter, fields)
        self.proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.perf_counter(), parts))

    def wait_first(self, timeout=10.0):
        """Waits (bounded) until nvidia-smi has printed its first sample."""
        end = time.perf_counter() + timeout
        while self.proc and not self.samples and time.perf_counter() < end and self.proc.poll() is None:
            time.sleep(0.02)

    def start_region(self):
        self.t0 = time.perf_counter()

    def end_region(self):
        self.t1 = time.perf_counter()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        t0 = self.t0 if self.t0 is not None else -math.inf
        t1 = self.t1 if self.t1 is not None else math.inf
        inside = [p for t, p in self.samples if t0 <= t <= t1]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0,
                    "samples_total": len(self.samples)}
        num = lambda v: v.replace(".", "").isdigit()
        sm = [float(p[1]) for p in inside if num(p[1])]
        mx = [float(p[2]) for p in inside if num(p[2])]
        pw = [float(p[3]) for p in inside if num(p[3])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for p in inside for k in range(4) if p[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_median": statistics.median(pw) if pw else None, "reasons": reasons,
                "samples": len(inside), "region_s": (t1 - t0) if self.t0 is not None else None}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _init_pg(ws, backend):
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend=backend)
        return dist
    return None


def _max_over_ranks(dist, v, device=None):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(dist, v, device=None):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_value(vertices_per_rank, world_size, steps, ms_max):
    """Whole-job vertex-updates/s when every rank advances a batch of equal size
    (no data-path collective); the job takes as long as the slowest rank."""
    return vertices_per_rank * world_size * steps / (ms_max * 1e-3)


def job_value(vertices_all_ranks, steps, ms_max):
    """Whole-job vertex-updates/s from the vertices of all ranks together."""
    return vertices_all_ranks * steps / (ms_max * 1e-3)


def build_batch(rank=0, world_size=1, scaling="weak"):
    """This rank's condensates.  weak: a job of 64 x world_size independent
    condensates, 64 per rank, every rank the same size sequence (equal work) with
    its own g, traps and noise; rank 0 holds the single-GPU batch.  strong: the
    single-GPU batch split over the ranks by size (largest first onto the rank
    with the fewest vertices).  No data-path exchange either way."""
    from vaikkari_gb300 import workloads
    if scaling == "weak":
        return workloads.config4(shard=rank)
    conds = workloads.config4()
    part = workloads.shard_by_size([c.inst for c in conds], world_size)[rank]
    return [conds[i] for i in part]


def prepare_fields(stepper, conds, precision_dtype):
    """Uploads the batch; odd = even * exp(i mu dt / 2) with mu from the library's
    observables of the initial field (GPUGrossPitaevskii_BCC.cu:325,342)."""
    from vaikkari_gb300.workloads import odd_from_even
    for i, c in enumerate(conds):
        stepper.upload(i, c.psi, c.psi, c.V)
    obs = stepper.observables(0)
    evens, odds = [], []
    for i, c in enumerate(conds):
        odd = odd_from_even(c.psi, obs[i]["mu"], c.inst.dt)
        evens.append(np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1).astype(precision_dtype)))
        odds.append(np.ascontiguousarray(np.stack([odd.real, odd.imag], -1).astype(precision_dtype)))
        stepper.upload(i, evens[-1], odds[-1], c.V)
    return evens, odds


def _oracle_grid(inst, lattice=1):
    """An oracle grid and dt*V (FP64, trap form) for one condensate, from the
    oracle's own copy of the reference's stencil tables (oracle/lattice.py);
    nothing of the library is loaded."""
    import oracle.oracle as orc
    from oracle.lattice import harmonic, tables, value_positions
    t = tables(lattice)
    g = orc.Grid(inst.nx, inst.ny, inst.nz, t["entry"], t["class_weight"], inst.block_scale, inst.dt, inst.g)
    pos = value_positions(inst.nx, inst.ny, inst.nz, inst.block_scale, inst.origin, lattice)
    return g, np.ascontiguousarray(harmonic(pos, inst.trap) * inst.dt)


def loaded_native_libraries():
    """Shared objects under this repository mapped into this process (from
    /proc/self/maps; empty where that file does not exist)."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and ".so" in os.path.basename(path):
                    out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def cpu_sample(conds, evens64, odds64, budget_s, threads, lattice=1):
    """Oracle FP64 leapfrog (the reference's update restated in C, all threads)
    over the batch, as many whole steps as fit the time budget (>= 1)."""
    import oracle.oracle as orc
    from oracle.lattice import tables
    orc.set_threads(threads)
    grids, vdts, es, os_ = [], [], [], []
    for c, e, o in zip(conds, evens64, odds64):
        g, vdt = _oracle_grid(c.inst, lattice)
        grids.append(g)
        vdts.append(vdt)
        es.append(e.copy())
        os_.append(o.copy())
    slots = tables(lattice)["slots"]
    verts = sum(c.inst.nx * c.inst.ny * c.inst.nz * slots for c in conds)
    t0 = time.perf_counter()
    steps = 0
    while True:
        for g, e, o, v in zip(grids, es, os_, vdts):
            if int(lattice) == 1:
                g.leapfrog_bcc2_fast(e, o, v, 1)
            else:
                g.leapfrog(e, o, v, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 1000:
            break
    return verts * steps / el, steps, el, verts


def cpu_single_core(conds, budget_s):
    """The same port on one thread, over the batch's instances in turn until the
    budget is used (vertex-updates/s)."""
    import oracle.oracle as orc
    orc.set_threads(1)
    done, t0 = 0, time.perf_counter()
    try:
        for c in conds:
            inst = c.inst
            g, vdt = _oracle_grid(inst)
            e = np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1))
            g.leapfrog_bcc2_fast(e, e.copy(), vdt, 1)
            done += inst.nx * inst.ny * inst.nz * 2
            if time.perf_counter() - t0 >= budget_s:
                break
    finally:
        orc.set_threads(0)
    return done / (time.perf_counter() - t0)


def run_reference(args):
    """--impl reference: the reference's update loop on the host cores.  The
    reference's stepping exists only as a CUDA kernel, so this runs the oracle
    port (its update and leapfrog restated in C, FP64, OpenMP over all host
    threads); each step is one leapfrog step over a bounded sample of the batch.
    The condensates are the same seeded batch, built with the oracle's stencil
    tables; the GPU library is never loaded (the line lists the repository's
    shared objects this process mapped)."""
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    import oracle.oracle as orc
    from oracle.lattice import tables
    from vaikkari_gb300 import workloads
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    conds = workloads.config4(geometry=tables(1))
    items = []
    for c in conds:
        inst = c.inst
        g, vdt = _oracle_grid(inst)
        e = np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1))
        items.append((g, e, e.copy(), vdt, inst.nx * inst.ny * inst.nz * 2))
    # calibrate on one step of the whole batch, then bound the per-step sample so
    # that warmup + steps fit in about two minutes
    t0 = time.perf_counter()
    for g, e, o, v, n in items:
        g.leapfrog_bcc2_fast(e, o, v, 1)
    full = time.perf_counter() - t0
    per_step_budget = 120.0 / max(args.steps + args.warmup, 1)
    frac = min(1.0, per_step_budget / max(full, 1e-9))
    total = sum(it[4] for it in items)
    sample, acc = [], 0
    for it in items:
        if sample and acc + it[4] > frac * total:
            break
        sample.append(it)
        acc += it[4]
    for _ in range(args.warmup):
        for g, e, o, v, n in sample:
            g.leapfrog_bcc2_fast(e, o, v, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for g, e, o, v, n in sample:
            g.leapfrog_bcc2_fast(e, o, v, 1)
    el = time.perf_counter() - t0
    value = acc * args.steps / el
    desc = (f"{len(sample)} of {len(items)} instances ({acc} of {total} vertices) per step, FP64 oracle port of "
            f"GPUGrossPitaevskii_BCC.cu:176-216,475-481 (BCC2 table from the reference's Mesh-library Hodge "
            f"data, direct interior indexing), {threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": HEADLINE_WORKLOAD, "instances": len(items), "sample_instances": len(sample),
                   "vertices_per_step": acc, "dt": 1e-4, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": loaded_native_libraries(),
    }
    print(json.dumps(line), flush=True)
    return 0


def time_windows(st, stream, steps, dist, clk, min_seconds, min_windows=5, max_windows=5000):
    """Times windows of exactly `steps` steps with CUDA events on the library's
    stream, each bracketed by a barrier (N > 1) and a device synchronisation on
    both sides, until at least `min_windows` windows and `min_seconds` of wall
    time (so the clock sampler sees the region).  Returns the per-window times
    (ms) and the kernel launches of one window."""
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, launches = [], 0
    clk.start_region()
    end = time.perf_counter() + min_seconds
    while len(times) < max_windows and (len(times) < min_windows or time.perf_counter() < end):
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        n0 = st.launch_count()
        ev0.record(stream)
        st.step(steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = st.launch_count() - n0
        times.append(ev0.elapsed_time(ev1))
    clk.end_region()
    return times, launches


def graph_steps_for(steps):
    """A step graph of exactly `steps` steps (up to 1000), so the timed region
    is graph replays, never the direct launches a shorter call falls back to."""
    return steps if steps <= 1000 else 100


def run_ours(args):
    ws, rank, local = _dist()
    import torch
    torch.cuda.set_device(local)
    dist = _init_pg(ws, "nccl")
    from vaikkari_gb300.gpe import Kernel, Lattice, Potential, Precision, Stepper
    conds = build_batch(rank, ws, args.scaling)
    insts = [c.inst for c in conds]
    verts = sum(i.nx * i.ny * i.nz for i in insts) * 2
    dev = torch.device("cuda", local)
    verts_job = _sum_over_ranks(dist, verts, device=dev)
    tile, zchunk, tuned = args.tile, args.zchunk, None
    comp_main = args.precision == "fp32c"
    prec = Precision.FP32C if comp_main else Precision.FP32
    host_t = np.float64 if comp_main else np.float32
    bytes_vs = BYTES_PER_VERTEX_STEP_COMP if comp_main else BYTES_PER_VERTEX_STEP
    clk = ClockSampler(local).__enter__()
    try:
        if tile < 0:
            # untimed: pick the kernel variant and z-chunk for this batch (cached per device)
            from vaikkari_gb300.autotune import autotune
            tuned = autotune(insts, precision=prec, potential=Potential.TRAP, device=local)
            tile, zchunk = tuned["tile"], tuned["zchunk"]
        gsteps = graph_steps_for(args.steps)
        st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED,
                     potential=Potential.TRAP, graph_steps=gsteps, tile=tile, zchunk=zchunk, device=local)
        evens, odds = prepare_fields(st, conds, host_t)
        # Warm-up: W steps, then one call of K steps, which instantiates the step
        # graph before the timed region.
        st.step(args.warmup)
        st.step(args.steps)
        st.synchronize()
        stream = torch.cuda.ExternalStream(st.stream_handle(), device=local)
        clk.wait_first()
        times, launches = time_windows(st, stream, args.steps, dist, clk, args.window_seconds)
        ms = statistics.median(times)
        ms_max = _max_over_ranks(dist, ms, device=dev)
        value = job_value(verts_job, args.steps, ms_max)
        roof = roofline_block(verts, bytes_vs, args.steps, ms * 1e-3, launches,
                              "fused_bcc2_kernel<float, MODE 2 (compensated)>" if comp_main
                              else "fused_bcc2_kernel<float, MODE 0>",
                              "fused_bcc2_fp32c_batch64.md" if comp_main else "fused_bcc2_batch64.md", tile)
        clocks = clk.summary()
    finally:
        clk.__exit__()

    # End to end through the public API with pinned host buffers.  One call
    # uploads every instance (one batched call), runs the K steps, reads the
    # observables and downloads every field (one batched call).  One untimed
    # call first: the handle allocates the transfers' device staging, copy
    # stream and events on first use.  e2e = the median of several calls.
    # Host fields are float in both storages (a GPE_FP32C handle takes float
    # with gpe_set_host_precision; its residual starts at zero, and the
    # accuracy block measures that path too).
    if comp_main:
        st.set_host_precision(Precision.FP32)
    pinned_e, pinned_o = [], []
    tt = torch.float32
    for e, o in zip(evens, odds):
        pe = torch.empty(e.shape, dtype=tt, pin_memory=True).numpy()
        po = torch.empty(o.shape, dtype=tt, pin_memory=True).numpy()
        pe[...] = e
        po[...] = o
        pinned_e.append(pe)
        pinned_o.append(po)
    h2d = sum(a.nbytes for a in pinned_e) + sum(a.nbytes for a in pinned_o)
    d2h = h2d + len(insts) * 56  # both fields back, plus one gpe_observables record per instance

    pairs = list(zip(pinned_e, pinned_o))

    def one_call():
        # gpe_round_trip: the copy engines move instance groups up and down
        # while the SMs step the others
        t0 = time.perf_counter()
        _, obs_ = st.round_trip(pairs, args.steps, outs=pairs)
        return time.perf_counter() - t0, obs_

    def one_call_sequential():
        t0 = time.perf_counter()
        st.upload_many([(i, pinned_e[i], pinned_o[i], None) for i in range(len(insts))])
        st.step(args.steps)
        obs_ = st.observables(0)
        st.download_many(range(len(insts)), outs=pairs)
        st.synchronize()
        return time.perf_counter() - t0, obs_

    def timed_calls(fn):
        fn()
        out, obs_ = [], None
        for _ in range(max(5, args.e2e_calls)):
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            el, obs_ = fn()
            out.append(el)
        return out, obs_

    seq_calls, _ = timed_calls(one_call_sequential)
    calls, obs = timed_calls(one_call)
    e2e_s = _max_over_ranks(dist, statistics.median(calls), device=dev)
    e2e_value = verts_job * args.steps / e2e_s
    seq_s = _max_over_ranks(dist, statistics.median(seq_calls), device=dev)
    h2d_job = _sum_over_ranks(dist, h2d, device=dev)
    d2h_job = _sum_over_ranks(dist, d2h, device=dev)
    finite = all(o["finite"] for o in obs)
    st.close()

    # Accuracy at this workload after 1000 steps: FP32, FP32C and FP64 (same scheme).
    acc = None
    if rank == 0 and not args.skip_accuracy:
        acc = accuracy_block(conds, insts, local, timed="fp32c" if comp_main else "fp32")

    # The batch in the other FP32 storage (plain FP32 when the headline is FP32C).
    other = None
    if rank == 0 and not args.skip_comp:
        other = storage_block(conds, insts, local, args.steps, args.warmup, args.window_seconds,
                              Precision.FP32 if comp_main else Precision.FP32C, tune=args.tile < 0)

    # The FP64 plain path, one instance at a time (the drop-in denominator).
    fp64 = None
    if rank == 0 and not args.skip_fp64:
        fp64 = fp64_plain_rate(conds, insts, local, args.fp64_steps)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        e64 = [np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1)) for c in conds]
        o64 = [a.copy() for a in e64]
        threads = os.cpu_count() or 1
        v, steps, el, nv = cpu_sample(conds, e64, o64, args.cpu_budget, threads)
        v1 = cpu_single_core(conds, 3.0)
        cpu = {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
               "sample": f"{steps} leapfrog step(s) of the whole batch ({nv} vertices), FP64 oracle port "
                         f"(GPUGrossPitaevskii_BCC.cu:176-216,475-481 restated, BCC2 table from the "
                         f"reference's Mesh-library Hodge data), {el:.1f} s",
               "value_1core": v1}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": args.scaling, "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": HEADLINE_WORKLOAD,
                       "storage": "fp32 + int8 residual per component (GPE_FP32C)" if comp_main else "fp32",
                       "instances": len(insts), "vertices": verts, "vertices_all_ranks": verts_job,
                       "sizes": sorted({i.nx for i in insts}), "dt": 1e-4,
                       "graph_steps": gsteps, "kernel": "fused", "variant": tile, "zchunk": zchunk,
                       "autotuned": tuned is not None,
                       "parallelism": (f"condensate shards x{ws} ({args.scaling}), no collective"
                                       if ws > 1 else "single"),
                       "l2": f"inputs larger than L2 (fields {2 * 8 * verts / 1e6:.0f} MB vs {L2_BYTES / 1e6:.0f} MB)",
                       "timing": (f"median of {len(times)} windows of {args.steps} steps (one graph replay each), "
                                  f"CUDA events on the library stream"),
                       "window_ms": {"min": min(times), "median": ms, "max": max(times)}},
            "roofline": roof,
            "gpu_launches": launches,
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d_job / args.steps,
                    "d2h_bytes_per_step": d2h_job / args.steps, "h2d_bytes_per_call": h2d_job,
                    "d2h_bytes_per_call": d2h_job, "steps_per_call": args.steps,
                    "seconds_median": e2e_s, "seconds_all": calls, "calls": len(calls), "finite": finite,
                    "host_format": "float32 complex (8 B per value and field)",
                    "call": "gpe_round_trip (pinned host buffers, outputs written over the inputs): upload, "
                            "steps, observables and download of every instance, instance groups' copies "
                            "overlapping other groups' steps",
                    "sequential": {"value": verts_job * args.steps / seq_s, "seconds_median": seq_s,
                                   "seconds_all": seq_calls,
                                   "call": "gpe_upload_many + gpe_step + gpe_observables_get + "
                                           "gpe_download_many, one after another"}},
            "cpu_baseline": cpu,
            "accuracy": acc,
            ("plain_fp32" if comp_main else "compensated"): other,
            "fp64_plain": fp64,
            "native_libraries": loaded_native_libraries(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def accuracy_block(conds, insts, device, timed="fp32c"):
    """FP32 and FP32C against FP64 of the same scheme after 1000 real-time steps
    of the whole batch: aggregate and worst-instance relative L2, and the worst
    norm and energy drift.  `timed` names the storage the headline timed; its
    figures are repeated under "timed"."""
    from vaikkari_gb300.gpe import Kernel, Lattice, Potential, Precision, Stepper
    steps = 1000
    outs = {}
    runs = ((Precision.FP32, np.float32, "fp32"), (Precision.FP64, np.float64, "fp64"),
            (Precision.FP32C, np.float64, "fp32c"), (Precision.FP32C, np.float32, "fp32c_host_fp32"))
    for prec, dt_, tag in runs:
        st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, potential=Potential.TRAP,
                     graph_steps=100, device=device)
        if prec == Precision.FP32C and dt_ == np.float32:
            st.set_host_precision(Precision.FP32)  # the e2e call's host format
        prepare_fields(st, conds, dt_)
        o0 = st.observables(0)
        st.step(steps)
        o1 = st.observables(0)
        fields = [st.download(i, odd=False)[0].astype(np.float64) for i in range(len(insts))]
        st.close()
        outs[tag] = (o0, o1, fields)
    f64 = outs["fp64"][2]
    den = sum(float(np.sum(b ** 2)) for b in f64)
    n64 = [o["norm"] for o in outs["fp64"][1]]
    e64 = [o["energy"] for o in outs["fp64"][1]]
    n0 = [o["norm"] for o in outs["fp64"][0]]
    res = {"steps": steps, "reference": "FP64 run of the same scheme (fused kernel, same inputs)",
           "max_norm_drift_fp64_scheme": max(abs(a - b) / b for a, b in zip(n64, n0)),
           "fp32c_host_fp32": "GPE_FP32C started from float fields and read back as float (the e2e host format)"}
    for tag in ("fp32", "fp32c", "fp32c_host_fp32"):
        f = outs[tag][2]
        num = sum(float(np.sum((a - b) ** 2)) for a, b in zip(f, f64))
        per = [math.sqrt(float(np.sum((a - b) ** 2)) / float(np.sum(b ** 2))) for a, b in zip(f, f64)]
        nn = [o["norm"] for o in outs[tag][1]]
        ee = [o["energy"] for o in outs[tag][1]]
        res[f"rel_l2_{tag}_vs_fp64"] = math.sqrt(num / den)
        res[f"max_instance_rel_l2_{tag}"] = max(per)
        res[f"instances_over_1e-5_{tag}"] = sum(1 for v in per if v > 1e-5)
        res[f"max_norm_drift_{tag}_vs_fp64"] = max(abs(a - b) / b for a, b in zip(nn, n64))
        res[f"max_energy_drift_{tag}_vs_fp64"] = max(abs(a - b) / abs(b) for a, b in zip(ee, e64))
    res["timed"] = {"storage": timed, "rel_l2_vs_fp64": res[f"rel_l2_{timed}_vs_fp64"],
                    "max_instance_rel_l2": res[f"max_instance_rel_l2_{timed}"],
                    "max_norm_drift_vs_fp64": res[f"max_norm_drift_{timed}_vs_fp64"],
                    "max_energy_drift_vs_fp64": res[f"max_energy_drift_{timed}_vs_fp64"],
                    "meets_l2_1e-5": res[f"rel_l2_{timed}_vs_fp64"] <= 1e-5,
                    "meets_norm_drift_1e-6": res[f"max_norm_drift_{timed}_vs_fp64"] <= 1e-6}
    return res


def storage_block(conds, insts, device, steps, warmup, window_seconds, prec, tune=True):
    """The batch in another storage (Precision.FP32 or FP32C): its own autotuned
    variant, timed like the headline (median of windows of K steps after W + K
    warm-up steps), with its roofline."""
    import torch
    from vaikkari_gb300.gpe import Kernel, Lattice, Potential, Precision, Stepper
    comp = prec == Precision.FP32C
    tile, zchunk = 0, 0
    if tune:
        from vaikkari_gb300.autotune import autotune
        t = autotune(insts, precision=prec, potential=Potential.TRAP, device=device)
        tile, zchunk = t["tile"], t["zchunk"]
    st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED,
                 potential=Potential.TRAP, graph_steps=graph_steps_for(steps), tile=tile, zchunk=zchunk,
                 device=device)
    prepare_fields(st, conds, np.float64 if comp else np.float32)
    st.step(warmup)
    st.step(steps)
    st.synchronize()
    stream = torch.cuda.ExternalStream(st.stream_handle(), device=device)
    clk = ClockSampler(device)
    times, launches = time_windows(st, stream, steps, None, clk, min(window_seconds, 0.5))
    ms = statistics.median(times)
    verts = sum(i.nx * i.ny * i.nz for i in insts) * 2
    st.close()
    bytes_vs = BYTES_PER_VERTEX_STEP_COMP if comp else BYTES_PER_VERTEX_STEP
    roof = roofline_block(verts, bytes_vs, steps, ms * 1e-3, launches,
                          "fused_bcc2_kernel<float, MODE 2 (compensated)>" if comp else
                          "fused_bcc2_kernel<float, MODE 0>",
                          "fused_bcc2_fp32c_batch64.md" if comp else "fused_bcc2_batch64.md", tile)
    return {"value": verts * steps / (ms * 1e-3), "unit": METRIC, "ms_per_step": ms / steps, "steps": steps,
            "windows": len(times), "variant": tile, "zchunk": zchunk, "gpu_launches": launches, "roofline": roof,
            "storage": ("FP32 value + int8 residual per component (10 B per value and field)" if comp
                        else "FP32 (8 B per value and field)")}


def fp64_plain_rate(conds, insts, device, steps):
    """The plain FP64 path, one instance at a time, same inputs and trap form."""
    import torch
    from vaikkari_gb300.gpe import Kernel, Lattice, Potential, Precision, Stepper
    total_ms = 0.0
    verts_total = 0
    for c in conds:
        st = Stepper([c.inst], lattice=Lattice.BCC2, precision=Precision.FP64, kernel=Kernel.PLAIN,
                     potential=Potential.TRAP, graph_steps=100, device=device)
        prepare_fields(st, [c], np.float64)
        st.step(3)
        st.step(100)
        st.synchronize()
        stream = torch.cuda.ExternalStream(st.stream_handle(), device=device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        st.step(steps)
        b.record(stream)
        torch.cuda.synchronize()
        total_ms += a.elapsed_time(b)
        verts_total += c.inst.nx * c.inst.ny * c.inst.nz * 2
        st.close()
    value = verts_total * steps / (total_ms * 1e-3)
    return {"value": value, "unit": METRIC, "steps": steps, "dtype": "f64", "kernel": "plain",
            "note": "each instance advanced alone (one launch per instance per half-step)"}


# ---------------------------------------------------------------------------
# The other configurations: parity and accuracy cases (not the headline line).

def _stepper(conds, prec, kernel, mode, tile=0, graph_steps=100, device=0, zchunk=0, lattice=None):
    from vaikkari_gb300.gpe import Lattice, Potential, Stepper
    return Stepper([c.inst for c in conds], lattice=Lattice.BCC2 if lattice is None else lattice, precision=prec,
                   kernel=kernel, mode=mode, potential=Potential.TRAP, graph_steps=graph_steps, tile=tile,
                   device=device, zchunk=zchunk)


def _rel_l2(a, b):
    num = sum(float(np.sum((x.astype(np.float64) - y.astype(np.float64)) ** 2)) for x, y in zip(a, b))
    den = sum(float(np.sum(y.astype(np.float64) ** 2)) for y in b)
    return math.sqrt(num / den)


def _rel_l2_phase(a, b):
    """Relative L2 after aligning the global phase of a to b (ground states are
    defined up to a constant phase)."""
    num = den = 0.0
    for x, y in zip(a, b):
        xc = x[..., 0].astype(np.float64) + 1j * x[..., 1].astype(np.float64)
        yc = y[..., 0].astype(np.float64) + 1j * y[..., 1].astype(np.float64)
        ov = np.vdot(xc, yc)
        xc = xc * (ov / abs(ov) if abs(ov) > 0 else 1.0)
        num += float(np.sum(np.abs(xc - yc) ** 2))
        den += float(np.sum(np.abs(yc) ** 2))
    return math.sqrt(num / den)


def _download(st, n):
    return [st.download(i, odd=False)[0] for i in range(n)]


def _cpu_config_rate(conds, budget_s=5.0, lattice=None):
    """FP64 oracle port on all host threads: whole leapfrog steps of every
    condensate for about `budget_s` seconds (at least one step)."""
    e64 = [np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1)) for c in conds]
    v, n, el, nv = cpu_sample(conds, e64, [a.copy() for a in e64], budget_s, os.cpu_count() or 1,
                              1 if lattice is None else int(lattice))
    return {"value": v, "unit": METRIC, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{n} leapfrog step(s), {nv} vertices, FP64 oracle port, {el:.2f} s"}


def run_config_realtime(name, conds, checkpoints, fp64_steps=None, tile=-1, lattice=None):
    """FP32 against FP64 of the same scheme at each checkpoint, plus throughput.
    BCC2 (config-mode): the fused kernel, and the FP64 plain path beside it.
    TETRA12 (ref-mode, the reference's discretisation): the fused TETRA12 kernel
    in FP32 (the line's value), the plain kernel in FP32 and FP64 beside it."""
    from vaikkari_gb300.gpe import Kernel, Lattice, Mode, Precision
    lattice = Lattice.BCC2 if lattice is None else Lattice(lattice)
    ref_mode = lattice == Lattice.TETRA12
    insts = [c.inst for c in conds]
    slots = 12 if ref_mode else 2
    verts = sum(i.nx * i.ny * i.nz for i in insts) * slots
    kern = Kernel.PLAIN if ref_mode else Kernel.FUSED
    zchunk = 0
    if ref_mode:
        tile = 0
    elif tile < 0:
        from vaikkari_gb300.autotune import autotune
        t = autotune(insts)
        tile, zchunk = t["tile"], t["zchunk"]
    fp64_last = fp64_steps or checkpoints[-1]
    runs = {}
    for prec, dt_, last in ((Precision.FP64, np.float64, fp64_last), (Precision.FP32, np.float32, checkpoints[-1])):
        k_ = Kernel.PLAIN if (ref_mode and prec == Precision.FP64) else (Kernel.FUSED if ref_mode else kern)
        st = _stepper(conds, prec, k_, Mode.REAL, tile=tile, lattice=lattice, zchunk=zchunk)
        prepare_fields(st, conds, dt_)
        o0 = st.observables(0)
        done, cps = 0, {}
        for cp in checkpoints:
            if cp > last:
                break
            st.step(cp - done)
            done = cp
            cps[cp] = (st.observables(0), _download(st, len(insts)))
        runs[prec] = (o0, cps)
        st.close()
    acc = []
    o64_0 = runs[Precision.FP64][0]
    for cp, (o32, f32) in runs[Precision.FP32][1].items():
        row = {"step": cp,
               "norm_fp32": [o["norm"] for o in o32], "energy_fp32": [o["energy"] for o in o32],
               "norm_drift_fp32_vs_initial": max(abs(a["norm"] - b["norm"]) / b["norm"] for a, b in zip(o32, o64_0))}
        if cp in runs[Precision.FP64][1]:
            o64, f64 = runs[Precision.FP64][1][cp]
            row["rel_l2_fp32_vs_fp64"] = _rel_l2(f32, f64)
            row["norm_drift_fp32_vs_fp64"] = max(abs(a["norm"] - b["norm"]) / b["norm"] for a, b in zip(o32, o64))
            row["energy_drift_fp32_vs_fp64"] = max(abs(a["energy"] - b["energy"]) / abs(b["energy"])
                                                   for a, b in zip(o32, o64))
            row["norm_drift_fp64_vs_initial"] = max(abs(a["norm"] - b["norm"]) / b["norm"] for a, b in zip(o64, o64_0))
            row["energy_fp64"] = [o["energy"] for o in o64]
        acc.append(row)
    # throughput, device time: windows of 200 steps (one graph replay each) after
    # warm-up, median, with the clocks sampled over the FP32 windows
    rates, rooflines, clocks = {}, {}, None
    cases = ((("fp32_fused", Precision.FP32, Kernel.FUSED), ("fp32_plain", Precision.FP32, Kernel.PLAIN),
              ("fp64_plain", Precision.FP64, Kernel.PLAIN)) if ref_mode
             else (("fp32_fused", Precision.FP32, Kernel.FUSED), ("fp32c_fused", Precision.FP32C, Kernel.FUSED),
                   ("fp64_fused", Precision.FP64, Kernel.FUSED), ("fp64_plain", Precision.FP64, Kernel.PLAIN)))
    head = "fp32_fused"
    for key, prec, kern_ in cases:
        tk, zk = (tile, zchunk) if kern_ == kern and prec != Precision.FP32C else (0, 0)
        if prec == Precision.FP32C:
            from vaikkari_gb300.autotune import autotune
            tc = autotune(insts, precision=Precision.FP32C)
            tk, zk = tc["tile"], tc["zchunk"]
        st = _stepper(conds, prec, kern_, Mode.REAL, tile=tk, lattice=lattice, zchunk=zk, graph_steps=200)
        prepare_fields(st, conds, np.float64 if prec in (Precision.FP64, Precision.FP32C) else np.float32)
        rates[key], rooflines[key], clk = _windowed_rate(st, verts, 200, key == head, prec, kern_, tk)
        if clk is not None:
            clocks = clk
        st.close()
    return {"metric": METRIC, "value": rates[head], "unit": METRIC, "dtype": "f32",
            "config": {"workload": name, "lattice": lattice.name, "instances": len(insts), "vertices": verts,
                       "dt": insts[0].dt, "variant": tile, "zchunk": zchunk,
                       "timing": "median of windows of 200 steps (one graph replay each), CUDA events",
                       "mode": "ref-mode (12 values per block, block scale a/sqrt(8))" if ref_mode
                       else "config-mode (2 values per cell)"},
            "roofline": rooflines[head], "clocks": clocks, "rates": rates, "rooflines": rooflines,
            "accuracy": acc, "cpu_baseline": _cpu_config_rate(conds, lattice=lattice)}


def _windowed_rate(st, verts, steps, sample_clocks, prec, kern, tile, seconds=1.0, imaginary=False):
    """Vertex-updates/s of a prepared stepper: median of windows of `steps`
    steps after one untimed call; the roofline at the algorithmic bytes of the
    trap form (real time: 24 B per value and half-step in FP32, 28 B in FP32C,
    48 B in FP64; the two-step variants move 16 / 32 B per value and half-step;
    imaginary time: one pass per step reading psi and writing the next field,
    16 B per value in FP32, 32 B in FP64)."""
    import torch
    from vaikkari_gb300.gpe import Precision, variants
    st.step(3)
    st.step(steps)
    st.synchronize()
    stream = torch.cuda.ExternalStream(st.stream_handle(), device=torch.cuda.current_device())
    clk = ClockSampler(torch.cuda.current_device())
    if sample_clocks:
        clk.__enter__()
        clk.wait_first()
    try:
        times, launches = time_windows(st, stream, steps, None, clk, seconds)
    finally:
        if sample_clocks:
            clk.__exit__()
    ms = statistics.median(times)
    half_steps = steps if imaginary else 2 * steps
    per_value_half = {Precision.FP32: 24, Precision.FP32C: 28, Precision.FP64: 48}[prec]
    if imaginary:
        per_value_half = {Precision.FP32: 16, Precision.FP64: 32}[prec]
    vinfo = {v["tile"]: v for v in variants()}
    if kern.name == "FUSED" and tile in vinfo and vinfo[tile]["half_steps"] == 2:
        per_value_half = per_value_half * 2 // 3  # both fields read once and written once per step
    peak, kind = _peaks()
    # the stepping kernel is the only kernel in the window: its average launch
    # moves the window's algorithmic bytes / launches in window time / launches
    achieved = verts * per_value_half * half_steps / (ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "traffic_source": "not captured for this workload",
            "algorithmic_bytes_per_vertex_step": per_value_half * half_steps // steps, "launches_per_window": launches,
            "peak_source": f"{kind} hbm_gbs (of {kind})"}
    return verts * steps / (ms * 1e-3), roof, (clk.summary() if sample_clocks else None)


def run_config_imaginary(name, conds, tol=1e-9, max_steps=200000, tile=-1, lattice=None):
    """BCC2: FP64 fused to the criterion, FP32 fused over the same steps.  TETRA12
    (ref-mode): both precisions over a fixed `max_steps`, FP32 on the fused TETRA12
    kernel (the line's value), FP64 on the plain kernel."""
    from vaikkari_gb300.gpe import Kernel, Lattice, Mode, Precision
    lattice = Lattice.BCC2 if lattice is None else Lattice(lattice)
    ref_mode = lattice == Lattice.TETRA12
    insts = [c.inst for c in conds]
    verts = sum(i.nx * i.ny * i.nz for i in insts) * (12 if ref_mode else 2)
    kern = Kernel.PLAIN if ref_mode else Kernel.FUSED
    zchunk = 0
    if ref_mode:
        tile, tol = 0, 0.0
    elif tile < 0:
        from vaikkari_gb300.autotune import autotune
        best = autotune(insts, mode=Mode.IMAGINARY, zchunks=(0, 16, 32, 64))
        tile, zchunk = best["tile"], best["zchunk"]
    res = {}
    steps64 = None
    for prec in (Precision.FP64, Precision.FP32):
        k_ = Kernel.PLAIN if (ref_mode and prec == Precision.FP64) else (Kernel.FUSED if ref_mode else kern)
        st = _stepper(conds, prec, k_, Mode.IMAGINARY, tile=tile, zchunk=zchunk, lattice=lattice)
        for i, c in enumerate(conds):
            st.upload(i, c.psi)
        t0 = time.perf_counter()
        # Both run to the criterion: FP64 tests |dmu| < tol every step; FP32
        # tests the mean |dmu| per step over the last 1000 steps with mu from the
        # FP64 observables (gpe_imaginary_time).
        lim, crit = max_steps, tol
        steps, conv, mu = st.imaginary_time(lim, crit)
        st.synchronize()
        wall = time.perf_counter() - t0
        obs = st.observables(0)
        fields = _download(st, len(insts))
        if prec == Precision.FP64:
            steps64 = steps
        st.close()
        res[prec] = {"steps": steps, "converged": conv, "mu": mu, "energy": [o["energy"] for o in obs],
                     "mu_obs": [o["mu"] for o in obs], "fields": fields, "wall_s": wall}
    r64, r32 = res[Precision.FP64], res[Precision.FP32]
    acc = {"steps_fp64": r64["steps"], "converged_fp64": r64["converged"], "steps_fp32": r32["steps"],
           "converged_fp32": r32["converged"], "mu_fp64": r64["mu_obs"], "mu_fp32": r32["mu_obs"],
           "rel_mu_fp32_vs_fp64": max(abs(a - b) / abs(b) for a, b in zip(r32["mu_obs"], r64["mu_obs"])),
           "rel_energy_fp32_vs_fp64": max(abs(a - b) / abs(b) for a, b in zip(r32["energy"], r64["energy"])),
           "rel_l2_fp32_vs_fp64": _rel_l2_phase(r32["fields"], r64["fields"])}
    # throughput of the imaginary-time step (FP32), device time: median of
    # windows of 1000 steps (ten graph replays), clocks sampled over them
    kern = Kernel.FUSED  # FP32: the fused kernel of either lattice
    st = _stepper(conds, Precision.FP32, kern, Mode.IMAGINARY, tile=tile, zchunk=zchunk, lattice=lattice)
    for i, c in enumerate(conds):
        st.upload(i, c.psi)
    rate, roof, clocks = _windowed_rate(st, verts, 1000, True, Precision.FP32, kern, tile, imaginary=True)
    st.close()
    return {"metric": METRIC, "value": rate, "unit": METRIC, "dtype": "f32", "roofline": roof, "clocks": clocks,
            "config": {"workload": name, "lattice": lattice.name, "instances": len(insts), "vertices": verts,
                       "dt": insts[0].dt, "tol": tol, "max_steps": max_steps, "mode": "imaginary", "variant": tile,
                       "zchunk": zchunk, "kernel": kern.name.lower()},
            "accuracy": acc, "cpu_baseline": _cpu_imag_rate(conds, lattice=lattice)}


def _cpu_imag_rate(conds, budget_s=5.0, lattice=None):
    """FP64 oracle imaginary-time steps (observables, then the normalised Euler
    step, all host threads for the step) of every condensate for about
    `budget_s` seconds; stencil tables from the oracle's own copy."""
    import oracle.oracle as orc
    from oracle.lattice import tables
    lat = 1 if lattice is None else int(lattice)
    t = tables(lat)
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    jobs = []
    for c in conds:
        inst = c.inst
        g, vdt = _oracle_grid(inst, lat)
        psi = np.ascontiguousarray(np.stack([c.psi.real, c.psi.imag], -1), dtype=np.float64)
        jobs.append((g, psi, vdt, t["cell_volume"] * inst.block_scale ** 3))
    verts = sum(c.inst.nx * c.inst.ny * c.inst.nz * t["slots"] for c in conds)
    steps, t0 = 0, time.perf_counter()
    while True:
        for g, psi, vdt, vol in jobs:
            g.imaginary(psi, vdt, vol, 2, 0.0)
        steps += 2
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 1000:
            break
    return {"value": verts * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} imaginary-time step(s), {verts} vertices, FP64 oracle port, {el:.2f} s"}


def run_relax(args):
    """main()'s vortex construction (GPUGrossPitaevskii_BCC.cu:509-531) on the GPU:
    the coarse relaxation (0.2 grid, up to 10000 iterations), the fine one (0.03
    grid resampled from it, 10000 iterations), and a batch of fine relaxations
    over a range of g in one call.  The unit is one Gauss-Seidel point update
    (with its share of the norm sums): (rsize - 1) * zsize per iteration."""
    from vaikkari_gb300.gpe import VortexState, relax
    unit = "point-updates/s"
    t0 = time.perf_counter()
    s0 = VortexState.create(20, 5000.0, 0.0, 15.0, 35.0, 0.2, 0.2)
    r0 = s0.relax(10000)
    d0 = s0.describe(1e-5)
    fine_args = (d0["min_r"], d0["max_r"], d0["max_z"], 0.03, 0.03)
    s = VortexState.create(20, 5000.0, *fine_args)
    s.initialize(s0)
    r1 = s.relax(10000)
    wall = time.perf_counter() - t0
    d = s.describe()
    R0, Z0 = d0["rsize"], d0["zsize"]
    R, Z = d["rsize"], d["zsize"]
    fine_rate = (R - 1) * Z * r1["iterations"] / (r1["device_ms"] * 1e-3)
    coarse_rate = (R0 - 1) * Z0 * r0["iterations"] / (r0["device_ms"] * 1e-3)
    # a batch: the same fine grid for 19 values of g, one call
    nb = max(1, args.relax_batch)
    gs = np.linspace(4000.0, 6000.0, nb)
    batch = []
    for gv in gs:
        v = VortexState.create(20, float(gv), *fine_args)
        v.initialize(s0)
        batch.append(v)
    its = args.relax_batch_iters
    rb = relax(batch, its, eps=0.0)
    batch_rate = nb * (R - 1) * Z * its / (rb[0]["device_ms"] * 1e-3)
    # CPU: the reference-order oracle on one thread (the reference's loop is serial)
    cpu = None
    if not args.skip_cpu:
        import oracle.oracle as orc
        path = _tmp_save(s0)
        o0 = orc.Vortex.from_file(path)
        os.remove(path)
        o = orc.Vortex.from_range(20, 5000.0, *fine_args)
        o.initialize(o0)
        n, el = 0, 0.0
        tc = time.perf_counter()
        while el < args.cpu_budget and n < 10000:
            o.iterate(100, eps=0.0)
            n += 100
            el = time.perf_counter() - tc
        cpu = {"value": (R - 1) * Z * n / el, "unit": unit, "cores": 1, "kind": "port",
               "sample": f"{n} iterations of the fine state ({R}x{Z}), FP64 oracle in the reference's order, "
                         f"{el:.1f} s"}
    line = {"metric": unit, "value": fine_rate, "unit": unit, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
            "higher_is_better": True,
            "config": {"workload": "vortex_relaxation_main", "kappa": 20, "g": 5000.0, "coarse": [R0, Z0],
                       "fine": [R, Z], "ratio": 0.1},
            "coarse": {"iterations": r0["iterations"], "device_ms": r0["device_ms"], "rate": coarse_rate},
            "fine": {"iterations": r1["iterations"], "device_ms": r1["device_ms"], "mu": d["mu"]},
            "batch": {"states": nb, "iterations": its, "device_ms": rb[0]["device_ms"], "rate": batch_rate},
            "construction_wall_s": wall, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    return 0


def run_production(args):
    """The reference's main() at production size (GPUGrossPitaevskii_BCC.cu:501-555),
    kappa 20, g 5000, on the GPU: both relaxations, the set-up of integrateInTime at
    main()'s block scale, and `--production-iters` iterations of the solver call in
    FP64 (the reference's arithmetic) and FP32.  The unit is one value update (one
    of the 12 values of a block, one leapfrog step)."""
    from vaikkari_gb300.gpe import Precision, VortexState
    unit = "value-updates/s"
    t0 = time.perf_counter()
    s0 = VortexState.create(20, 5000.0, 0.0, 15.0, 35.0, 0.2, 0.2)
    r0 = s0.relax(10000)
    d0 = s0.describe(1e-5)
    s = VortexState.create(20, 5000.0, d0["min_r"], d0["max_r"], d0["max_z"], 0.03, 0.03)
    s.initialize(s0)
    r1 = s.relax(10000)
    relax_s = time.perf_counter() - t0
    d = s.describe(1e-5)
    bs, mr, mz = d["block_scale"], d["max_r"], d["max_z"]
    lo, hi = (-mr, -mr, -mz), (mr, mr, mz)
    its = max(1, args.production_iters)
    rates = {}
    for name, prec in (("fp64", Precision.FP64), ("fp32", Precision.FP32)):
        res, obs, _, _ = s.integrate_in_time(bs, lo, hi, 1.0, its, precision=prec)
        rates[name] = {"value": res["values"] * its * res["steps_per_iteration"] / (res["device_ms"] * 1e-3),
                       "device_ms": res["device_ms"], "setup_seconds": res["setup_ms"] * 1e-3,
                       "energy": [o["energy"] for o in obs]}
    t1 = time.perf_counter()
    s.setup(bs, lo, hi)
    host_setup_s = time.perf_counter() - t1
    line = {"metric": unit, "value": rates["fp64"]["value"], "unit": unit, "n_gpus": 1, "dtype": "f64",
            "data": "synthetic", "higher_is_better": True,
            "config": {"workload": "production_main", "kappa": 20, "g": 5000.0, "block_scale": bs,
                       "blocks": [res["xsize"], res["ysize"], res["zsize"]], "values": res["values"],
                       "steps_per_iteration": res["steps_per_iteration"], "iterations_timed": its},
            "relax": {"seconds": relax_s, "device_ms": [r0["device_ms"], r1["device_ms"]],
                      "iterations": [r0["iterations"], r1["iterations"]]},
            "setup_seconds": rates["fp64"]["setup_seconds"], "host_setup_seconds": host_setup_s,
            "fp64": rates["fp64"], "fp32": rates["fp32"]}
    print(json.dumps(line), flush=True)
    return 0


def _tmp_save(v):
    import tempfile
    fd, path = tempfile.mkstemp(suffix=".dat")
    os.close(fd)
    v.save(path)
    return path


def run_tetra12(args):
    """The drop-in's arithmetic on the production grid: TETRA12 (the reference's
    discretisation, 12 values per block), plain kernel, array potential, one
    instance of 87 x 87 x 302 blocks (main()'s grid at block scale 0.06997) with
    seeded random fields.  FP64 (bit-identical to the reference's kernel) and FP32,
    then both again in the face (Hodge) form of the multi-GPU program, each timed
    with CUDA events over --steps steps (best of three) after a graph of 100 steps."""
    from vaikkari_gb300.gpe import Instance, Kernel, Lattice, Potential, Precision, Stepper, default_face_table
    rng = np.random.default_rng(5)
    inst = Instance(87, 87, 302, 0.06997, 1e-4, 100.0, origin=(-3.0, -3.0, -10.0))
    shp = (inst.nz, inst.ny, inst.nx, 12)
    e = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) * 0.3
    o = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) * 0.3
    V = rng.uniform(0.0, 10.0, shp)
    vals = inst.nx * inst.ny * inst.nz * 12
    rates = {}
    faces = default_face_table()
    for name, prec, fc, kern in (("fp64", Precision.FP64, None, Kernel.PLAIN),
                                 ("fp32", Precision.FP32, None, Kernel.PLAIN),
                                 ("fp32_fused", Precision.FP32, None, Kernel.FUSED),
                                 ("fp64_faces", Precision.FP64, faces, Kernel.PLAIN),
                                 ("fp32_faces", Precision.FP32, faces, Kernel.PLAIN),
                                 ("fp32_faces_fused", Precision.FP32, faces, Kernel.FUSED)):
        st = Stepper([inst], lattice=Lattice.TETRA12, precision=prec, kernel=kern,
                     potential=Potential.ARRAY, graph_steps=100, faces=fc, tile=3 if kern == Kernel.FUSED else 0)
        st.upload(0, e, o, V)
        st.time_steps(100)
        ms = min(st.time_steps(args.steps) for _ in range(3))
        st.close()
        rates[name] = vals * args.steps / (ms * 1e-3)
    line = {"metric": METRIC, "value": rates["fp64"], "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "tetra12_plain_production_grid", "values": vals, "blocks": [87, 87, 302],
                       "lattice": "TETRA12", "kernel": "plain", "potential": "array"},
            "fp32": rates["fp32"],
            "fp32_fused": rates["fp32_fused"],
            "faces": {"fp64": rates["fp64_faces"], "fp32": rates["fp32_faces"], "fp32_fused": rates["fp32_faces_fused"],
                      "form": "Hodge (face) form of GPUGrossPitaevskii_BCC_multi.cu:329-397, weights 1.5"},
            "note": "FP64 performs the reference kernel's rounded operations and equals its results bit for "
                    "bit; the per-value constant L0 + V*dt is added once per potential upload, leaving 15 FP64 "
                    "operations per value and half-step; the bound is this GPU's FP64 rate"}
    print(json.dumps(line), flush=True)
    return 0


def run_batch_imaginary(args):
    """The 64-condensate batch in imaginary time: all condensates advance in one
    fused launch per step, each renormalised every step.  FP32 and FP64 run
    --imag-steps steps from the same random-phase start (seed 4); the line
    reports the FP32 rate (autotuned, device time of 300 steps) and mu / energy
    of FP32 against FP64 per condensate."""
    from vaikkari_gb300 import workloads
    from vaikkari_gb300.autotune import autotune
    from vaikkari_gb300.gpe import Kernel, Lattice, Mode, Potential, Precision, Stepper
    conds = workloads.config4()
    insts = [c.inst for c in conds]
    verts = sum(i.nx * i.ny * i.nz for i in insts) * 2
    rng = np.random.default_rng(4)
    psis = [np.exp(1j * rng.uniform(0, 2 * np.pi, size=(i.nz, i.ny, i.nx, 2))) for i in insts]
    t = autotune(insts, precision=Precision.FP32, potential=Potential.TRAP, mode=Mode.IMAGINARY,
                 zchunks=(0, 16, 32, 64))
    tile, zchunk = t["tile"], t["zchunk"]
    res = {}
    for prec in (Precision.FP64, Precision.FP32):
        st = Stepper(insts, lattice=Lattice.BCC2, precision=prec, kernel=Kernel.FUSED, mode=Mode.IMAGINARY,
                     potential=Potential.TRAP, graph_steps=100, tile=tile, zchunk=zchunk)
        for i, p in enumerate(psis):
            st.upload(i, p)
        steps, conv, mu = st.imaginary_time(args.imag_steps, 0.0)
        obs = st.observables(0)
        if prec == Precision.FP32:
            st.time_steps(100)
            ms = min(st.time_steps(300) for _ in range(2))
            res["rate"] = verts * 300 / (ms * 1e-3)
            res["ms_per_step"] = ms / 300
        st.close()
        res[prec] = (mu, [o["energy"] for o in obs])
    mu64, e64 = res[Precision.FP64]
    mu32, e32 = res[Precision.FP32]
    line = {"metric": METRIC, "value": res["rate"], "unit": METRIC, "n_gpus": 1, "dtype": "f32",
            "data": "synthetic", "ms_per_step": res["ms_per_step"],
            "config": {"workload": "batch64_bcc2_imaginary", "instances": len(insts), "vertices": verts,
                       "steps": args.imag_steps, "variant": tile, "zchunk": zchunk, "kernel": "fused"},
            "accuracy": {"max_rel_mu_fp32_vs_fp64": max(abs(a - b) / abs(b) for a, b in zip(mu32, mu64)),
                         "max_rel_energy_fp32_vs_fp64": max(abs(a - b) / abs(b) for a, b in zip(e32, e64)),
                         "mu_fp64_range": [min(mu64), max(mu64)]}}
    print(json.dumps(line), flush=True)
    return 0


def run_workload(args):
    from vaikkari_gb300 import workloads
    name = args.workload
    if name == "batch64_imag":
        return run_batch_imaginary(args)
    if name == "relax":
        return run_relax(args)
    if name == "tetra12":
        return run_tetra12(args)
    if name == "production":
        return run_production(args)
    from vaikkari_gb300.gpe import Lattice
    lat = Lattice.TETRA12 if args.lattice == "tetra12" else Lattice.BCC2
    tag = lat.name.lower()
    if name == "config1":
        line = run_config_realtime(f"config1_{tag}_32_realtime_1000", [workloads.config1(lat)], [1000],
                                   tile=args.tile, lattice=lat)
    elif name == "config2":
        if lat == Lattice.TETRA12:
            line = run_config_imaginary(f"config2_{tag}_128_imaginary_2000_steps", [workloads.config2(lat)],
                                        max_steps=2000, lattice=lat)
        else:
            line = run_config_imaginary(f"config2_{tag}_128_imaginary", [workloads.config2(lat)], tile=args.tile)
    elif name == "config3":
        line = run_config_realtime(f"config3_{tag}_192_vortex_ring", [workloads.config3(lat)], [1000, 5000, 10000],
                                   tile=args.tile, lattice=lat)
    elif name == "config4":
        line = run_config_realtime(f"config4_{tag}_batch64_realtime_1000", workloads.config4(lat), [1000],
                                   tile=args.tile, lattice=lat)
    elif name == "config5":
        line = run_config_realtime(f"config5_{tag}_512_realtime", [workloads.config5(lat)], [200, 2000],
                                   fp64_steps=200, tile=args.tile, lattice=lat)
    else:
        raise SystemExit(f"unknown workload {name}")
    line["n_gpus"] = 1
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tile", type=int, default=-1, help="kernel variant; -1 = autotune")
    ap.add_argument("--zchunk", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--fp64-steps", type=int, default=200)
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-comp", action="store_true", help="skip the timing of the other FP32 storage")
    ap.add_argument("--precision", default="fp32c", choices=["fp32", "fp32c"],
                    help="batch64: storage of the timed path (fp32c = FP32 + int8 residuals, the storage that "
                         "meets relative L2 <= 1e-5 after 1000 steps; fp32 = plain FP32)")
    ap.add_argument("--window-seconds", type=float, default=2.0,
                    help="keep timing windows of --steps steps for at least this long (median reported)")
    ap.add_argument("--e2e-calls", type=int, default=5, help="timed end-to-end calls (median reported)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--workload", default="batch64",
                    help="batch64 (the headline), config1/config2/config3/config5 (accuracy cases), relax "
                         "(the vortex relaxation), production (main() at production size), tetra12 (the "
                         "drop-in's FP64/FP32 kernel on the production grid) or batch64_imag (the batch in "
                         "imaginary time)")
    ap.add_argument("--lattice", default="bcc2", choices=["bcc2", "tetra12"],
                    help="config1-5: config-mode (bcc2, 2 values per cell) or ref-mode (tetra12, the reference's "
                         "12 values per block)")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="multi-GPU split: weak = 64 condensates per rank, strong = the 64 split over ranks")
    ap.add_argument("--imag-steps", type=int, default=2000, help="batch64_imag: imaginary-time steps")
    ap.add_argument("--production-iters", type=int, default=2)
    ap.add_argument("--relax-batch", type=int, default=19)
    ap.add_argument("--relax-batch-iters", type=int, default=2000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "batch64":
        return run_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
