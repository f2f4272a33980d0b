"""In-tree build of libcdx.so (CUDA kernels for sm_103a + C++ host engine + C ABI).

Translation units compile in parallel; the FP64 plain-method kernels are compiled with
--fmad=false so their arithmetic is rounded exactly as written (bit-reproducible against the
CPU oracle). Host C++ uses -ffp-contract=off for the same reason (the GPU machine's aarch64 gcc
contracts by default).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcdx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("CUDA toolkit not found")


def _stamp(cmd: list[str], deps: list[str]) -> str:
    """Digest of what an output is built from: the command, the machine and every input's bytes."""
    h = hashlib.sha256()
    h.update(" ".join(cmd).encode())
    h.update(platform.machine().encode())
    for d in sorted(deps):
        h.update(d.encode())
        with open(d, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _needs(out: str, stamp: str) -> bool:
    """An output is rebuilt unless it exists with a stamp equal to its inputs' digest (file times
    are not trusted: a copied tree may carry objects newer than their sources, or built for
    another machine)."""
    if not os.path.exists(out) or not os.path.exists(out + ".stamp"):
        return True
    with open(out + ".stamp") as f:
        return f.read().strip() != stamp


def _mark(out: str, stamp: str) -> None:
    with open(out + ".stamp", "w") as f:
        f.write(stamp + "\n")


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = _cuda_home()
    os.makedirs(OBJ, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 "-Xptxas", "-warn-spills"] + ARCH
        if os.path.basename(src).startswith(("k_fp64", "k_csr", "noalloc", "k_adjoint")):
            flags += ["--fmad=false"]
        cmd = [os.path.join(cuda, "bin", "nvcc"), *flags, "-I", CSRC, "-c", src, "-o", obj]
        jobs.append((obj, [src] + headers, cmd))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-I", os.path.join(cuda, "include"), "-I", CSRC, "-c", src, "-o", obj]
        jobs.append((obj, [src] + headers, cmd))

    def run(job):
        obj, deps, cmd = job
        stamp = _stamp(cmd, deps)
        if not force and not _needs(obj, stamp):
            return obj, ""
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        _mark(obj, stamp)
        return obj, p.stderr

    objs = []
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for obj, log in ex.map(run, jobs):
            objs.append(obj)
            if verbose and log.strip():
                print(log, file=sys.stderr)
    libdir = os.path.join(cuda, "lib64")
    link = ["g++", "-shared", "-o", LIB, *objs, "-L", libdir, "-lcudart_static", "-ldl", "-lrt", "-lpthread",
            "-Wl,--no-undefined"]
    lstamp = _stamp(link, objs)
    if force or _needs(LIB, lstamp):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [tmp if c == LIB else c for c in link]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, LIB)
        _mark(LIB, lstamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
