"""Builds the oracle's compiled parts into oracle/_build/ (TEST
INFRASTRUCTURE: only tests and the benchmark's CPU-baseline and accuracy legs
load them):
- libtfqg_cpuref.so from cpu_ref.cc: the reference's expectation + adjoint
  loops restated in C++, the timed CPU baseline;
- libtfqg_sv128.so from sv128.c: complex128 matrix application for the
  oracle's large-state and density-matrix checks.

Host flags are portable (-O3, no -march=native): the same sources build on
x86-64 and on the aarch64 GPU hosts, where gcc's default target already has
the 128-bit Advanced SIMD unit that -O3 vectorizes for."""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
TARGETS = {
    "cpuref": (os.path.join(HERE, "cpu_ref.cc"), os.path.join(OUT_DIR, "libtfqg_cpuref.so"),
               ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp"]),
    "sv128": (os.path.join(HERE, "sv128.c"), os.path.join(OUT_DIR, "libtfqg_sv128.so"),
              ["gcc", "-O3", "-std=c11", "-fcx-limited-range", "-fPIC", "-shared",
               "-fopenmp"]),
}
# kept for callers that name the baseline library directly
SRC, OUT = TARGETS["cpuref"][0], TARGETS["cpuref"][1]


def build_one(name, force=False):
    src, out, cc = TARGETS[name]
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= os.path.getmtime(src)):
        return out
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = cc + [src, "-o", out + ".tmp"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(out + ".tmp", out)
    return out


def build(force=False):
    """Build every compiled part; return the CPU-baseline library's path."""
    for name in TARGETS:
        build_one(name, force)
    return OUT


if __name__ == "__main__":
    for name in TARGETS:
        print(build_one(name, force=True))
