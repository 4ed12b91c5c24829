"""Regenerate the golden fixtures in this folder from the reference's own code.

Runs only where the reference source tree is present (it is read, never
copied): builds ``oracle/_ref/ref_fixtures`` with ``make -C oracle ref`` (the
reference's GPUGrossPitaevskii_BCC.cu host code, VortexState, Mesh library and
MT19937, compiled from their sources) and records what it prints.

    python tests/golden/make_golden.py [--ref DIR]     (DIR: $VAIKKARI_REFERENCE, else /root/reference)

Outputs (committed):
  ref_tables.json        getPositions/getLaplacian (GPUGrossPitaevskii_BCC.cu:73-142)
  ref_multi_tables.json  the face tables of the multi-GPU program's Hodge-form update
                         (GPUGrossPitaevskii_BCC_multi.cu:73-271), from oracle/_ref/ref_multi_tables
  ref_mesh_hodge.json    Mesh-library Hodge weights around interior BCC nodes/bodies
  ref_vortex_state.json  state.dat diagnostics, psi/phase samples, Random(54363) stream
  ref_vortex_state2.json the same for state2.dat
  ref_setup_bs2.json/.bin  integrateInTime host set-up (GPUGrossPitaevskii_BCC.cu:222-348)
                           at block_scale 2.0 on state.dat
  ref_state_header.json  the binary header fields of state.dat (VortexState.cpp:49-72)
  ref_state_small.dat    a coarse vortex state made by the reference's iterateSolution
  ref_vortex_small.json  its diagnostics; ref_setup_small.json/.bin the set-up on it
  ref_slice_small.bmp, ref_volume_small.mhd/.raw, ref_outputs_small.json
                         the reference's picture and volume outputs of that set-up
  ref_state_main.json    digest of the reference's shipped state.dat (main()'s two-stage
                         relaxation, GPUGrossPitaevskii_BCC.cu:509-531): header, SHA-256 of
                         the values, and a seeded sample of values
"""
import argparse
import json
import os
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")


def run(args):
    out = subprocess.run(args, check=True, capture_output=True, text=True).stdout
    start = out.find("{")   # the reference's solver prints progress lines before the JSON
    return json.loads(out[start:])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("VAIKKARI_REFERENCE", "/root/reference"),
                    help="reference source tree (default: $VAIKKARI_REFERENCE, else /root/reference)")
    a = ap.parse_args()
    gp = os.path.join(a.ref, "koodit", "GrossPitaevskii")
    if not os.path.isdir(gp):
        sys.exit(f"reference tree not found at {a.ref}")
    subprocess.run(["make", "-C", ORACLE, "ref", f"REF={a.ref}", "-j8"], check=True,
                   stdout=subprocess.DEVNULL)
    exe = os.path.join(ORACLE, "_ref", "ref_fixtures")

    def dump(name, obj):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)
            f.write("\n")

    dump("ref_tables.json", run([exe, "tables"]))
    dump("ref_multi_tables.json", run([os.path.join(ORACLE, "_ref", "ref_multi_tables")]))
    dump("ref_mesh_hodge.json", run([exe, "mesh"]))
    dump("ref_vortex_state.json", run([exe, "vortex", os.path.join(gp, "state.dat")]))
    dump("ref_vortex_state2.json", run([exe, "vortex", os.path.join(gp, "state2.dat")]))
    binp = os.path.join(HERE, "ref_setup_bs2.bin")
    dump("ref_setup_bs2.json", run([exe, "setup", os.path.join(gp, "state.dat"), "2.0", binp]))

    # A small vortex state from the reference's own relaxation solver (kappa 20,
    # g 5000, r/z step 0.25), its diagnostics, and the integrateInTime set-up on it.
    small = os.path.join(HERE, "ref_state_small.dat")
    dump("ref_state_small.json", run([exe, "makestate", small]))
    dump("ref_vortex_small.json", run([exe, "vortex", small]))
    dump("ref_setup_small.json", run([exe, "setup", small, "1.5", os.path.join(HERE, "ref_setup_small.bin")]))

    # The reference's BMP slice and MetaImage volume of the small set-up's even
    # field, written by its own Picture::save / saveVolumeMap (relative paths, so
    # that the .mhd names its .raw without a directory).
    setup = json.load(open(os.path.join(HERE, "ref_setup_small.json")))
    vortex = json.load(open(os.path.join(HERE, "ref_vortex_small.json")))
    out = subprocess.run([exe, "outputs", "ref_setup_small.bin", str(setup["xsize"]), str(setup["ysize"]),
                          str(setup["zsize"]), repr(setup["block_scale"]), repr(vortex["function_max"]),
                          "ref_slice_small.bmp", "ref_volume_small.mhd"],
                         check=True, capture_output=True, text=True, cwd=HERE).stdout
    dump("ref_outputs_small.json", json.loads(out))

    # The shipped state.dat is main()'s relaxation output: its digest and a sample.
    import hashlib
    import numpy as np
    with open(os.path.join(gp, "state.dat"), "rb") as f:
        raw = f.read()
    hdr = struct.calcsize("<IdIIdddd")
    kappa, g, rsize, zsize, rplug, rstep, zstep, mu = struct.unpack_from("<IdIIdddd", raw, 0)
    vals = np.frombuffer(raw, dtype="<f8", count=rsize * zsize, offset=hdr)
    idx = np.sort(np.random.default_rng(7).choice(rsize * zsize, 512, replace=False))
    dump("ref_state_main.json", {
        "source": "koodit/GrossPitaevskii/state.dat (main(), GPUGrossPitaevskii_BCC.cu:509-531)",
        "kappa": kappa, "g": g, "rsize": rsize, "zsize": zsize, "rplug": rplug, "rstep": rstep, "zstep": zstep,
        "mu": mu, "values_sha256": hashlib.sha256(vals.tobytes()).hexdigest(),
        "function_max": float(vals.max()),
        "sample_index": [int(i) for i in idx], "sample_value": [float(vals[i]) for i in idx]})

    # Header of the state file, decoded with the field order of VortexState::load.
    with open(os.path.join(gp, "state.dat"), "rb") as f:
        raw = f.read()
    kappa, g, rsize, zsize, rplug, rstep, zstep, mu = struct.unpack_from("<IdIIdddd", raw, 0)
    dump("ref_state_header.json", {
        "source": "koodit/GrossPitaevskii/VortexState.cpp:49-72 (state.dat)",
        "kappa": kappa, "g": g, "rsize": rsize, "zsize": zsize, "rplug": rplug,
        "rstep": rstep, "zstep": zstep, "mu": mu, "file_bytes": len(raw)})
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
