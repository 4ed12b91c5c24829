"""Autotuner for the fused kernel: picks the kernel variant (tile shape,
pipeline depth, register cap) and the z-chunk length per work item for a given
batch, by timing each candidate on the GPU with CUDA events on the library's
stream, and caches the choice per workload signature and device.

    from vaikkari_gb300.autotune import autotune
    best = autotune(instances, fields=[(even, odd), ...])   # -> {"tile": .., "zchunk": .., ...}

Cache: vaikkari_gb300/_tune/cache.json (not versioned).  Set
GPE_AUTOTUNE_CACHE to use another file, or cache=False to always measure.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
from typing import List, Optional, Sequence

import numpy as np

from .gpe import Instance, Kernel, Lattice, Mode, Potential, Precision, Stepper, variants

CACHE = os.environ.get("GPE_AUTOTUNE_CACHE",
                       os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune", "cache.json"))


def _device_name(device: int) -> str:
    try:
        out = subprocess.run(["nvidia-smi", f"--id={device}", "--query-gpu=name", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        return out or "unknown"
    except Exception:
        return "unknown"


def signature(instances: Sequence[Instance], lattice, precision, potential, device_name: str, mode=Mode.REAL) -> str:
    dims = sorted((i.nx, i.ny, i.nz) for i in instances)
    fields = {"dims": dims, "lattice": int(lattice), "precision": int(precision), "potential": int(potential),
              "device": device_name}
    if mode != Mode.REAL:
        fields["mode"] = int(mode)
    key = json.dumps(fields)
    return hashlib.sha1(key.encode()).hexdigest()


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(db):
    """Writes the cache atomically; ranks of one job may store at the same time,
    so each writes its own temporary file and the last replace wins (entries a
    concurrent writer added in between are re-measured on a later run)."""
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = f"{CACHE}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1)
    os.replace(tmp, CACHE)


def measure(instances: List[Instance], tile: int, zchunk: int, fields=None, lattice=Lattice.BCC2,
            precision=Precision.FP32, potential=Potential.TRAP, steps: int = 200, device: int = 0,
            mode=Mode.REAL) -> float:
    """Vertex-updates per second of one candidate (best of three timed runs)."""
    st = Stepper(instances, lattice=lattice, precision=precision, kernel=Kernel.FUSED, potential=potential,
                 graph_steps=100, tile=tile, zchunk=zchunk, device=device, mode=mode)
    try:
        for i in range(len(instances)):
            if fields is not None:
                e, o = fields[i][0], fields[i][1]
                v = fields[i][2] if len(fields[i]) > 2 else None
            else:
                shp = st.shape(i)
                e = o = np.full(shp + (2,), 1e-3, dtype=st.field_dtype)
                v = np.zeros(shp, dtype=st.dtype) if potential == Potential.ARRAY else None
            st.upload(i, e, None if mode != Mode.REAL else o, v)
        st.time_steps(103)      # warm-up, graph instantiation
        best = min(st.time_steps(steps) for _ in range(3))
        vals = st.total_values()
    finally:
        st.close()
    return vals * steps / (best * 1e-3)


def autotune(instances: List[Instance], fields=None, lattice=Lattice.BCC2, precision=Precision.FP32,
             potential=Potential.TRAP, device: int = 0, steps: int = 200, cache: bool = True,
             zchunks: Sequence[int] = (0, 8, 16, 32), verbose: bool = False, mode=Mode.REAL) -> dict:
    """Best (tile, zchunk) for this batch.  Every variant is timed with the
    automatic z-chunk, then the three fastest with each z-chunk in `zchunks`.
    Imaginary time and compensated storage (Precision.FP32C) skip the variants
    that advance whole real-time steps; imaginary time also skips the persistent
    variants (real time only).  The variants are the BCC2 fused kernel's; other
    lattices are refused (the fused TETRA12 kernel's six tiles are chosen with
    gpe_config.tile directly)."""
    if Lattice(lattice) != Lattice.BCC2:
        raise ValueError("autotune times the BCC2 fused kernel's variants; pass tile directly for other lattices")
    name = _device_name(device)
    sig = signature(instances, lattice, precision, potential, name, mode)
    db = _load() if cache else {}
    if sig in db:
        return db[sig]
    results = []
    for v in variants():
        if (mode != Mode.REAL or Precision(precision) == Precision.FP32C) and v["half_steps"] != 1:
            continue
        if mode != Mode.REAL and v["persistent"]:  # real time only
            continue
        r = measure(instances, v["tile"], 0, fields, lattice, precision, potential, steps, device, mode)
        results.append({"tile": v["tile"], "zchunk": 0, "vups": r})
        if verbose:
            print("autotune", v, f"{r:.4g}", flush=True)
    top = sorted(results, key=lambda r: -r["vups"])[:3]
    for t in top:
        for zc in zchunks:
            if zc == 0:
                continue
            r = measure(instances, t["tile"], zc, fields, lattice, precision, potential, steps, device, mode)
            results.append({"tile": t["tile"], "zchunk": zc, "vups": r})
            if verbose:
                print("autotune", t["tile"], zc, f"{r:.4g}", flush=True)
    best = max(results, key=lambda r: r["vups"])
    entry = {"tile": best["tile"], "zchunk": best["zchunk"], "vups": best["vups"], "device": name,
             "candidates": results}
    if cache:
        db = _load()  # entries other processes stored meanwhile
        db[sig] = entry
        _store(db)
    return entry
