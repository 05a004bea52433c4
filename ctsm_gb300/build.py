"""In-tree build of libctsm_gpu.so for sm_103a (nvcc, one -gencode, parallel TUs)."""
import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libctsm_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# extra nvcc flags for tuning builds (e.g. -DCTSMG_PIPE_CHUNKS=8)
NVFLAGS += os.environ.get("CTSMG_NVCC_EXTRA", "").split()


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctsm_gpu.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


STAMP = os.path.join(BUILD, "stamp")


def _digest():
    """Hash of every source and header, the flags and the host architecture:
    the library is rebuilt whenever any of them differs from the last build."""
    h = hashlib.sha256()
    deps = sources() + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    deps.append(os.path.join(ROOT, "include", "ctsm_gpu.h"))
    for d in deps:
        h.update(os.path.basename(d).encode())
        with open(d, "rb") as f:
            h.update(f.read())
    h.update(" ".join(ARCH + NVFLAGS).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _stale():
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        return f.read().strip() != _digest()


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nv] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources()))) as ex:
        results = list(ex.map(compile_one, sources()))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    r = subprocess.run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_digest() + "\n")
    with open(os.path.join(BUILD, "build.log"), "w") as f:
        f.write(" ".join([nv] + ARCH + NVFLAGS) + "\n")
        for src, (_, log) in zip(sources(), results):
            f.write("%s\n%s" % (os.path.basename(src), log))
    if verbose:
        for _, log in results:
            print(log)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
    print(LIB)
