"""Build the native library in-tree: vaikkari_gb300/_lib/libvaikkari_gpe.so.

Each translation unit under csrc/ is compiled by its own nvcc process (in
parallel) for sm_103a only, then linked with the CUDA runtime.  Also builds the
CPU oracle (oracle/_build/libgpe_oracle.so), which only tests and the benchmark's
CPU baseline load.

    python -m vaikkari_gb300.build [--oracle-only | --lib-only] [-v]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libvaikkari_gpe.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libgpe_oracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gpe_lattice.cpp", "gpe_api.cpp", "gpe_vortex.cpp", "gpe_plain.cu", "gpe_fused.cu", "gpe_fused_t12.cu", "gpe_persistent.cu", "gpe_output.cu", "gpe_noalloc.cu", "gpe_relax.cu",
           "gpe_setup.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build_lib(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nv = nvcc()
    # -ffp-contract=off: host code must not fuse a*b+c (GCC does by default on
    # aarch64), so that positions, trap tables and factors round identically on
    # every host and match the oracle; device arithmetic on the parity paths uses
    # explicit rounded intrinsics.
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")]
    jobs = []
    for src in SOURCES:
        obj = os.path.join(OBJDIR, src + ".o")
        path = os.path.join(CSRC, src)
        if src.endswith(".cu"):
            cmd = [nv, *common, *ARCH, "-lineinfo", "-Xptxas", "-v", "-c", path, "-o", obj]
        else:
            cmd = [nv, *common, "-x", "c++", "-c", path, "-o", obj]
        jobs.append((cmd, obj))
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        futs = {ex.submit(_run, cmd, verbose): obj for cmd, obj in jobs}
        for f in cf.as_completed(futs):
            logs[futs[f]] = f.result()
    with open(os.path.join(OBJDIR, "ptxas.log"), "w") as f:
        for k in sorted(logs):
            f.write(f"== {os.path.basename(k)}\n{logs[k]}\n")
    tmp = LIB + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp, *[o for _, o in jobs], "-lcudart"], verbose)
    os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose=False):
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    srcs = [os.path.join(ORACLE_DIR, n) for n in ("gpe_oracle.c", "vortex_oracle.c")]
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", *srcs,
          "-o", tmp, "-lm"], verbose)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle-only", action="store_true")
    ap.add_argument("--lib-only", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    if not a.oracle_only:
        print(build_lib(a.verbose))
    if not a.lib_only:
        print(build_oracle(a.verbose))


if __name__ == "__main__":
    sys.exit(main())
