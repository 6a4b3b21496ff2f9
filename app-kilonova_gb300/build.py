"""Build libknc_gpu.so for GB300 (sm_103a) in-tree with nvcc.

Each translation unit compiles in parallel to app-kilonova_gb300/_build/*.o
and links into app-kilonova_gb300/_build/libknc_gpu.so. The FP64 stage
(knc_f64.cu) is compiled with --fmad=false so that its arithmetic rounds like
the CPU reference implementation; every other unit keeps FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
INCLUDE = HERE.parent / "include"
LIB = OUT / "libknc_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          # host-side geometry and time bookkeeping round like the CPU reference
          # implementation on x86-64 and aarch64 alike (gcc contracts by default)
          "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", f"-I{INCLUDE}"]
PER_FILE = {
    "knc_f64.cu": ["--fmad=false"],
    "knc_noalloc.cu": ["--fmad=false"],
    "knc_mixed.cu": ["-prec-div=false", "-prec-sqrt=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, headers) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = _headers()
    cc = nvcc()
    stamp = OUT / "flags.txt"
    flags = repr((ARCH, COMMON, PER_FILE, cc))
    force = not stamp.exists() or stamp.read_text() != flags
    jobs = []
    for src in _sources():
        obj = OUT / (src.stem + ".o")
        if force or _stale(obj, src, headers) or ptxas_info:
            cmd = [cc, *ARCH, *COMMON, *PER_FILE.get(src.name, []), "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    failed = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src, cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append((src, r.stdout + r.stderr))
    if failed:
        msg = "\n".join(f"--- {s.name}\n{log}" for s, log in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    stamp.write_text(flags)
    objs = [str(OUT / (s.stem + ".o")) for s in _sources()]
    if jobs or not LIB.exists():
        cmd = [cc, *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
