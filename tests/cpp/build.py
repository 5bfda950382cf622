"""Builds the C++ drop-in test programs into tests/_build/:
test_dropin (nvcc, sm_103a: generic kernels through Gb300Executor) and
test_dropin_host (g++ only: the header needs no CUDA headers)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "tests", "_build")
LIBDIR = os.path.join(ROOT, "ode_prototyping_gb300", "_build")
INC = os.path.join(ROOT, "include")
RPATH = "-Wl,-rpath,$ORIGIN/../../ode_prototyping_gb300/_build"


def stale(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target)
                                             for d in deps)


def main():
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in os.listdir(HERE)] + [
        os.path.join(INC, "gbode.h"), os.path.join(INC, "gbode", "gbode.hpp"),
        os.path.join(LIBDIR, "libgbode.so")]
    host = os.path.join(OUT, "test_dropin_host")
    if stale(host, deps):
        subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", f"-I{INC}", f"-I{HERE}",
                        os.path.join(HERE, "test_dropin_host.cpp"), "-o", host, f"-L{LIBDIR}",
                        "-lgbode", RPATH], check=True)
    dev = os.path.join(OUT, "test_dropin")
    if stale(dev, deps):
        nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "-O2",
                        "--expt-relaxed-constexpr", f"-I{INC}", f"-I{HERE}",
                        os.path.join(HERE, "test_dropin.cu"), "-o", dev, f"-L{LIBDIR}", "-lgbode",
                        "-Xlinker", "-rpath,$ORIGIN/../../ode_prototyping_gb300/_build"],
                       check=True)


if __name__ == "__main__":
    main()
    sys.exit(0)
