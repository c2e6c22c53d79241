"""Build recipe of the SCD engine and its tools (no cmake; parallel nvcc/g++).

Outputs (all under het-scd_gb300/_build/, git-ignored):
  libscd_gb300.so   CUDA kernels + the C ABI of include/scd_gb300.h (sm_103a only)
  convert, main-gpu, main   the reference's command lines on top of the C ABI
  libscdgen.so      seeded synthetic graph generators
The CPU oracle (test infrastructure) has its own recipe, oracle/build_oracle.py.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["engine.cu", "preprocess.cu", "csr.cu", "text.cu", "triangles.cu", "partition.cu", "refine.cu",
              "improve.cu", "resident.cu", "wcc_static.cu"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps_cuda():
    csrc = os.path.join(HERE, "csrc")
    hdrs = [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(ROOT, "include", "scd_gb300.h"))
    return hdrs


def nvcc_flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                   "-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "csrc")] + list(extra)


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    jobs = jobs or max(4, os.cpu_count() or 4)
    hdrs = _deps_cuda()
    objs = []
    tasks = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for src in CU_SOURCES:
            s = os.path.join(HERE, "csrc", src)
            o = os.path.join(OUT, src.replace(".cu", ".o"))
            objs.append(o)
            if not _newer(o, [s] + hdrs):
                tasks.append(ex.submit(_run, ["nvcc"] + nvcc_flags(["-Xptxas", "-v"] if verbose else []) +
                                       ["-c", s, "-o", o]))
        gen_so = os.path.join(OUT, "libscdgen.so")
        gen_src = os.path.join(HERE, "gen", "scdgen.c")
        if not _newer(gen_so, [gen_src]):
            tasks.append(ex.submit(_run, ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                                          "-Wall", gen_src, "-o", gen_so]))
        logs = [t.result() for t in tasks]
    lib = os.path.join(OUT, "libscd_gb300.so")
    if not _newer(lib, objs):
        _run(["nvcc"] + ARCH + ["-shared", "-o", lib] + objs)
    # command-line tools over the C ABI
    host = os.path.join(HERE, "host")
    common = [os.path.join(host, "graph_io.cpp")]
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = []
        for tool, src in (("convert", "convert.cpp"), ("main-gpu", "main_gpu.cpp"), ("main", "main.cpp")):
            exe = os.path.join(OUT, tool)
            deps = [os.path.join(host, src), lib] + common + [os.path.join(host, "graph_io.hpp"),
                                                              os.path.join(ROOT, "include", "scd_gb300.h")]
            if not _newer(exe, deps):
                futs.append(ex.submit(_run, ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"),
                                             os.path.join(host, src)] + common +
                                      ["-o", exe, "-L", OUT, "-lscd_gb300", "-Wl,-rpath,$ORIGIN"]))
        logs += [f.result() for f in futs]
    if verbose:
        print("\n".join(l for l in logs if l))
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", OUT)
