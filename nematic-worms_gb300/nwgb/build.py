"""In-tree build of the GB300 engine (libnwgb.so) and of the test oracle.

Everything is compiled for sm_103a only, one nvcc per translation unit in
parallel, then linked into nematic-worms_gb300/lib/libnwgb.so.  The oracle
(plain C, test infrastructure) goes to oracle/_build/, and, where the
reference tree is present, the CPU emulation of the reference kernels goes to
oracle/_ref/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from .abi import LIB_DIR, LIB_PATH, PKG_ROOT, REPO_ROOT

CSRC = PKG_ROOT / "csrc"
COMPAT = PKG_ROOT / "compat"
BUILD_DIR = PKG_ROOT / "_build"
ORACLE_DIR = REPO_ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libnworacle.so"
REF_DIR = ORACLE_DIR / "_ref"
REF_CUDA_HOST = ORACLE_DIR / "_build" / "libnwref_cuda.so"


def reference_tree() -> Path | None:
    """The reference checkout the oracle recipes compile from: $NW_REFERENCE_TREE,
    else a checkout named ``reference`` beside this repository; None if absent
    (on a host without it the prebuilt oracle/_ref files are used as they are)."""
    env = os.environ.get("NW_REFERENCE_TREE")
    for cand in ([Path(env)] if env else []) + [REPO_ROOT.parent / "reference"]:
        if (cand / "simulation" / "particles_kernel_impl.cuh").exists():
            return cand
    return None

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]

CU_SOURCES = ["nw_kernels.cu", "nw_fused.cu", "nw_fused_planar.cu", "nw_engine.cu", "nw_legacy.cu", "nw_sort.cu", "nw_noalloc.cu", "nw_batch.cu", "nw_adjoint.cu", "nw_writer.cu", "nw_defects.cu", "nw_observables.cu"]
CPP_SOURCES = ["nw_config.cpp"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and Path(cand, "bin", "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps if Path(d).exists())


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout)
    return r.stdout


def _headers():
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((REPO_ROOT / "include").glob("*.h"))
    hs += list(COMPAT.glob("*.h")) + list(COMPAT.glob("*.cuh"))
    return hs


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA / C++ source for sm_103a and link libnwgb.so."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        sp = CSRC / src
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        if force or _newer(obj, [sp] + headers):
            if src.endswith(".cu"):
                cmd = [nvcc] + NVCC_FLAGS + ["-c", str(sp), "-o", str(obj)]
            else:
                cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", f"-I{cuda / 'include'}", f"-I{COMPAT}",
                       "-c", str(sp), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or _newer(LIB_PATH, objs):
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", str(LIB_PATH)] + [str(o) for o in objs]
             + ["-lcudart"])
    return LIB_PATH


def build_oracle(force: bool = False) -> Path:
    """Compile the plain-C oracle (test infrastructure) with OpenMP."""
    out = ORACLE_LIB
    out.parent.mkdir(exist_ok=True)
    srcs = [ORACLE_DIR / "nw_oracle.c", ORACLE_DIR / "nw_oracle_impl.h", ORACLE_DIR / "nw_oracle.h",
            REPO_ROOT / "include" / "nwgb.h"]
    if force or _newer(out, srcs):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
              "-o", str(out), str(ORACLE_DIR / "nw_oracle.c"), "-lm"])
    return out


def build_reference_emulation(force: bool = False):
    """Compile the reference's own kernel source for the CPU (only where the
    reference tree exists; nothing at run time depends on it)."""
    tree = reference_tree()
    if tree is None or shutil.which("make") is None:
        return None
    args = ["make", "-s", "-C", str(ORACLE_DIR / "ref_emu"), f"REF={tree}", f"OUT={REF_DIR}",
            f"CUDA_HOME={_cuda_home()}"]
    if force:
        args.insert(1, "-B")
    _run(args)
    return REF_DIR


def build_reference_cuda(force: bool = False):
    """The reference CUDA build used as checker and speed denominator (test
    infrastructure): its device code as an sm_103a fatbin, compiled from the
    reference tree where that exists (oracle/ref_cuda/Makefile; the fatbin then
    travels with the repository), and the host harness that loads it
    (oracle/ref_cuda/nwref_host.cu), compiled on every host."""
    tree = reference_tree()
    if tree is not None and shutil.which("make") is not None:
        args = ["make", "-s", "-C", str(ORACLE_DIR / "ref_cuda"), f"REF={tree}", f"OUT={REF_DIR}",
                f"CUDA_HOME={_cuda_home()}"]
        if force:
            args.insert(1, "-B")
        _run(args)
    cuda = _cuda_home()
    src = ORACLE_DIR / "ref_cuda" / "nwref_host.cu"
    deps = [src, COMPAT / "particles_kernel.cuh"]
    REF_CUDA_HOST.parent.mkdir(exist_ok=True)
    if force or _newer(REF_CUDA_HOST, deps):
        _run([str(cuda / "bin" / "nvcc")] + ARCH + ["-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
              "-o", str(REF_CUDA_HOST), str(src), f"-L{cuda / 'lib64' / 'stubs'}", "-lcuda", "-lcurand"])
    return REF_CUDA_HOST


def build_all(force: bool = False, verbose: bool = False):
    with ThreadPoolExecutor(max_workers=4) as ex:
        f_lib = ex.submit(build_library, force, verbose)
        f_or = ex.submit(build_oracle, force)
        f_ref = ex.submit(build_reference_emulation, force)
        f_rc = ex.submit(build_reference_cuda, force)
        return f_lib.result(), f_or.result(), f_ref.result(), f_rc.result()
