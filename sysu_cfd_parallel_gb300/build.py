"""Build recipe of libcycasgpu.so (in-tree, sm_103a only).

Translation units:
  host_case.cpp  g++  -- param.in / gmsh reader, face discovery, initial fields
  assembly.cu    nvcc -fmad=false -- FP64 face/cell kernels, rounded exactly as the
                 reference's source orders each product and sum
  krylov.cu      nvcc -- persistent GMRES, reductions
  capi.cu        nvcc -- C ABI and iteration schedule
  mesh_tables.cpp g++ -- CSR pattern, slots and face orders of a mesh (host threads)
  result_io.cpp  g++ -ffp-contract=off -- result files in the reference's formats
Objects are compiled in parallel and linked with nvcc into
``sysu_cfd_parallel_gb300/_build/libcycasgpu.so``.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcycasgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")

UNITS = [
    ("host_case.cpp", "cxx", []),
    ("assembly.cu", "nvcc", ["-fmad=false"]),
    ("krylov.cu", "nvcc", []),
    ("gmres.cu", "nvcc", []),
    ("amg.cu", "nvcc", []),
    ("amg_setup.cpp", "cxx", []),
    ("capi.cu", "nvcc", []),
    ("noalloc.cu", "nvcc", []),
    ("server.cpp", "cxx", []),
    ("mesh_tables.cpp", "cxx", []),
    ("union_mesh.cpp", "cxx", []),
    ("batch_schedule.cpp", "cxx", []),
    ("result_io.cpp", "cxx", ["-ffp-contract=off"]),
]
# bench-only: the FP64/FP32 FMA-rate probe bench.py uses for the FP64 roofline of the channel
# workload, built as its own library so that the product library does not carry it
PROBE_SRC = "rate_probe.cu"
PROBE_LIB = os.path.join(BUILD, "libcycas_rate_probe.so")


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home:
        return home
    import shutil
    nvcc = shutil.which(NVCC)
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _sources_digest() -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)):  # the product units and the bench-only probe
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode())
            h.update(f.read())
    with open(os.path.join(INCLUDE, "cycasgpu.h"), "rb") as f:
        h.update(f.read())
    with open(__file__, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp.txt")
    digest = _sources_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    procs = []
    objs = []
    for src, kind, extra in UNITS:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        path = os.path.join(CSRC, src)
        if kind == "cxx":
            cmd = [CXX, "-O2", "-std=c++17", "-fPIC", "-Wall", *extra, "-c", path, "-o", obj, "-I", INCLUDE,
                   "-I", os.path.join(_cuda_home(), "include")]
        else:
            cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                   *extra, "-c", path, "-o", obj, "-I", INCLUDE]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("compilation failed:\n" + "\n".join(failed))
    link = [NVCC, *ARCH, "-shared", "-o", LIB, *objs]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    probe = [NVCC, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", os.path.join(CSRC, PROBE_SRC), "-o",
             PROBE_LIB]
    r = subprocess.run(probe, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("rate probe build failed:\n" + r.stdout.decode(errors="replace"))
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
