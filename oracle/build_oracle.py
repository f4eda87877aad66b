"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/hyperball_oracle.cpp (HyperBall), oracle/visits_oracle.cpp
(breadth-first visits) and oracle/sum_sweep_oracle.cpp (ExactSumSweep) into oracle/_build/libhb_oracle.so with g++. The reference crate itself is Rust and cannot be built in this image (no
cargo/rustc), so there is no oracle/_ref: the oracle is this C++ restatement.
The seeded graph generators (webgraph-algo-rs_gb300/csrc/graph_gen.cpp, plain
C++) are compiled in too, so a process that only runs the oracle can build the
benchmark graphs without loading the product library.

-ffp-contract=off keeps every f64 multiply and add separately rounded, as Rust
computes them; without it gcc on aarch64 fuses a*b+c into fmadd and the
per-node sums would drift from the reference's arithmetic.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhb_oracle.so")
GEN_DIR = os.path.join(os.path.dirname(HERE), "webgraph-algo-rs_gb300", "csrc")
SOURCES = [os.path.join(HERE, "hyperball_oracle.cpp"), os.path.join(HERE, "visits_oracle.cpp"),
           os.path.join(HERE, "sum_sweep_oracle.cpp"), os.path.join(GEN_DIR, "graph_gen.cpp")]
HEADERS = [os.path.join(HERE, "hll_oracle.hpp"), os.path.join(HERE, "par_fair.hpp"),
           os.path.join(GEN_DIR, "graph_gen.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS)


def command():
    return [
        "g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread",
        "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-I" + GEN_DIR,
        "-o", LIB, *SOURCES,
    ]


def build(force=False, wait=True):
    """Compile the oracle library; returns the Popen when wait=False."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale():
        return None
    p = subprocess.Popen(command())
    if wait:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed")
        return None
    return p


if __name__ == "__main__":
    build(force=True)
    print(LIB)
