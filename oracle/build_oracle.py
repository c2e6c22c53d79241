"""Build recipe of the CPU oracle (test infrastructure, never the product).

  oracle/_build/liboracle.so   the restatement of the reference's CPU path
                               (scd_oracle.cpp), loaded by oracle.py
  oracle/_ref/*                the reference's own CPU binaries, compiled from
                               its unmodified sources by build_ref.sh, only where
                               those sources exist (the development container);
                               a machine without them builds the restatement only

Usage: python oracle/build_oracle.py [reference source directory]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(ref_src=None):
    """Compiles the oracle; ref_src (default: build_ref.sh's own default) names
    the reference's source directory for oracle/_ref."""
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "liboracle.so")
    src = [os.path.join(HERE, "scd_oracle.cpp"), os.path.join(HERE, "scd_oracle.h")]
    procs = []
    if not _newer(so, src):
        procs.append(subprocess.Popen(["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
                                       src[0], "-o", so], stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    # the reference's own binaries: build_ref.sh builds nothing where its sources are absent
    args = ["sh", os.path.join(HERE, "build_ref.sh")] + ([ref_src] if ref_src else [])
    procs.append(subprocess.Popen(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    for p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build step failed:\n" + " ".join(p.args) + "\n" + out.decode())
    return so


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else None)
    print("built", OUT)
