"""Builds libmedyan_mech.so in-tree with nvcc for sm_103a.

Translation units are compiled in parallel; the FP64 excluded-volume object
is compiled without FMA contraction (see mech_exvol.cu).

With MECH_TRACE=1 in the environment, a diagnostic variant is built into (and
loaded from) _lib_trace/ instead: every kernel block appends a (start, end,
kernel, block) record to a timeline that mech_minimize writes to the file
named by MECH_TRACE_FILE.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
TRACE = bool(os.environ.get("MECH_TRACE"))
OUTDIR = os.path.join(HERE, "_lib_trace" if TRACE else "_lib")
LIBNAME = "libmedyan_mech.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]

# (source, object, extra flags)
UNITS = [
    ("mech_ff.cu", "mech_ff.o", []),
    ("mech_exvol.cu", "mech_exvol_f64.o", ["-DMECH_EXVOL_REAL=double", "-fmad=false"]),
    ("mech_exvol.cu", "mech_exvol_f32.o", ["-DMECH_EXVOL_REAL=float"]),
    ("mech_nl.cu", "mech_nl.o", []),
    ("mech_host.cu", "mech_host.o", []),
    ("mech_static.cu", "mech_static.o", []),
    ("mech_hvp.cu", "mech_hvp.o", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> str:
    return os.path.join(OUTDIR, LIBNAME)


def _stale(obj: str, srcs) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUTDIR, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "medyan_mech.h"))
    jobs = []
    for src, obj, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUTDIR, obj)
        if force or ptxas_info or _stale(o, [s] + headers):
            cmd = [nv, *ARCH, *COMMON, *extra, *(["-DMECH_TRACE"] if TRACE else []), "-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append(cmd)
    if failed:
        raise RuntimeError(f"nvcc failed for {len(failed)} unit(s)")
    out = lib_path()
    objs = [os.path.join(OUTDIR, o) for _, o, _ in UNITS]
    if force or jobs or _stale(out, objs):
        cmd = [nv, *ARCH, "-shared", "-o", out, *objs, "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return out


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv))
