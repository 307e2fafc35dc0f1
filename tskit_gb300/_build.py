"""Compile the package's native code in place.

* ``libtskit_gb300.so`` -- the CUDA kernels and the C ABI (nvcc, sm_103a only);
* ``_smc_sim.so``       -- the host-side synthetic tree-sequence generator (gcc).

Objects go to ``tskit_gb300/_build/`` and are compiled in parallel; nothing is
installed outside the source tree.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")

CUDA_SOURCES = [
    "tsg_treeseq.cu",
    "tsg_plan.cu",
    "tsg_stats.cu",
    "tsg_batch.cu",
    "tsg_eval_f32_pol.cu",
    "tsg_eval_f32_unpol.cu",
    "tsg_eval_f64_pol.cu",
    "tsg_eval_f64_unpol.cu",
    "tsg_afs.cu",
    "tsg_matvec.cu",
    "tsg_gram.cu",
    "tsg_grm.cu",
    "tsg_general.cu",
    "tsg_kastore.cu",
    "tsg_index.cu",
    "tsg_gnn.cu",
    "tsg_callback.cu",
    "tsg_cplan.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIB_NAME = "libtskit_gb300.so"
SIM_NAME = "_smc_sim.so"


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_sim(force=False):
    src = os.path.join(CSRC, "smc_sim.c")
    out = os.path.join(PKG, SIM_NAME)
    if force or _stale(out, [src]):
        _run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", src, "-lm", "-o", out])
    return out


def build_cuda(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = nvcc_path()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    flags = ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
        "-I", INCLUDE, "-I", CSRC,
    ]
    if verbose:
        flags += ["-Xptxas", "-v"]
    objs = []
    jobs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    logs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    lib = os.path.join(PKG, LIB_NAME)
    if force or jobs or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib, logs


def build_all(force=False):
    build_sim(force)
    return build_cuda(force)
