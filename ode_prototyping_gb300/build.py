"""Builds libgbode.so in-tree (ode_prototyping_gb300/_build/) for sm_103a.

Each CUDA translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a) and linked into one shared
library with the CUDA runtime linked statically, so the library has no
runtime dependency beyond the driver.  Also builds the C++ drop-in test
program (tests/cpp) against the C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libgbode.so")
# throughput probe of the force kernel's roofline (a standalone program, not
# part of the library; bench.py --workload pipes and the headline line run it)
PROBE_SRC = os.path.join(CSRC, "probe", "pipes.cu")
PROBE = os.path.join(BUILD, "probe_pipes")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]
SOURCES = ["rk.cu", "nbody.cu", "integrator.cu", "mlp.cu", "batched.cu", "energy.cu", "ic.cu",
           "noalloc.cu", "trajectory.cu",
           "leapfrog.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "gbode.h"))
    return hs


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    headers = _headers()
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append((s, cmd))
    if os.path.exists(PROBE_SRC) and (force or _stale(PROBE, [PROBE_SRC])):
        jobs.append(("probe/pipes.cu", [cc, *ARCH, "-O3", "-std=c++17", PROBE_SRC, "-o", PROBE]))
    outputs = {}
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): s for s, cmd in jobs}
        for f in cf.as_completed(futs):
            r = f.result()
            outputs[futs[f]] = r
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError(f"nvcc failed on {futs[f]}")
            if verbose or ptxas_info:
                sys.stderr.write(f"== {futs[f]}\n{r.stderr}")
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in srcs]
    if force or any(name.endswith(".cu") and "/" not in name for name, _ in jobs) or \
            _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv, force="-f" in sys.argv)
    print(LIB)
