"""Builds the CUDA library libhmr_gb300.so in-tree (sm_103a only).

hmr_faces.cu is compiled once per arithmetic form -- the exact form
(-DHMR_FAST=0 --fmad=false, the reference's operation order, bitwise equal to
it) and the fast form (-DHMR_FAST=1) -- flow model (-DHMR_MODEL=0/1/2) and
scheme set (-DHMR_SCHEME_SET=0: WCNS5-JS/WCNS6-LD, 1: WCNS5-Z/WCNS6-CU-M2),
twelve translation units compiled in parallel.  The cell-data kernels are always exact.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libhmr_gb300.so")
PEAK_LIB = os.path.join(OUT, "libhmr_peak.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps the reference's rounding too (aarch64 GCC would fuse multiply-adds).
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(HERE, "..", "include")]

UNITS = [
    ("hmr_cells.cu", "hmr_cells.o", ["-DHMR_FAST=0", "--fmad=false"]),
    ("hmr_abi.cu", "hmr_abi.o", ["-DHMR_FAST=0", "--fmad=false"]),
    ("hmr_noalloc.cu", "hmr_noalloc.o", ["-DHMR_FAST=0", "--fmad=false"]),
] + [
    ("hmr_faces.cu", "hmr_faces_%s_m%d_s%d.o" % (form, model, sset),
     ["-DHMR_FAST=%d" % fast, "--fmad=%s" % ("true" if fast else "false"), "-DHMR_MODEL=%d" % model,
      "-DHMR_SCHEME_SET=%d" % sset])
    for form, fast in (("exact", 0), ("fast", 1)) for model in (0, 1, 2) for sset in (0, 1)
] + [
    ("hmr_vjp.cu", "hmr_vjp_m%d.o" % model, ["-DHMR_FAST=0", "--fmad=true", "-DHMR_MODEL=%d" % model])
    for model in (0, 1, 2)
] + [
    ("hmr_diffusive.cu", "hmr_diffusive_%s.o" % form, ["-DHMR_FAST=%d" % fast, "--fmad=%s" % ("true" if fast else "false")])
    for form, fast in (("exact", 0), ("fast", 1))
]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def sources_newer_than(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "hmr.h")
    return os.path.getmtime(hdr) > t


def build(force=False, verbose=False, extra=()):
    """Compile every translation unit in parallel and link the shared library."""
    if not force and not sources_newer_than(LIB):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    exe = nvcc()
    procs = []
    for src, obj, flags in UNITS:
        cmd = [exe] + ARCH + COMMON + list(flags) + list(extra) + ["-c", os.path.join(CSRC, src),
                                                                  "-o", os.path.join(OUT, obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    # measurement and self-check utilities: the FP64 peak and the integer-pipe FP64 check
    peak = [exe] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                           os.path.join(CSRC, "hmr_peak.cu"), os.path.join(CSRC, "hmr_emu_check.cu"),
                           "-o", PEAK_LIB + ".tmp"]
    subprocess.check_call(peak)
    os.replace(PEAK_LIB + ".tmp", PEAK_LIB)
    tmp = LIB + ".tmp"
    link = [exe] + ARCH + ["-shared", "-o", tmp] + [os.path.join(OUT, o) for _, o, _ in UNITS] + ["-lcudart"]
    subprocess.check_call(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
