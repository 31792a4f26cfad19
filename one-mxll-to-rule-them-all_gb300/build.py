"""Build libomx_gpu.so (sm_103a) in-tree.

The FP64 kernels and every FP64 sparse kernel are compiled with -fmad=false so that their
rounding matches the reference's FP64 arithmetic; the FP32 stencil kernels keep FMA
contraction.  Host set-up code is compiled with -ffp-contract=off for the same reason.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libomx_gpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include():
    nvcc = _nvcc()
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _jobs():
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
    inc = ["-I", CSRC]
    jobs = [
        [nvcc] + ARCH + common + ["-fmad=false"] + inc + ["-c", os.path.join(CSRC, "omx_kernels_exact.cu"),
                                                           "-o", os.path.join(BUILD, "exact.o")],
        [nvcc] + ARCH + common + inc + ["-c", os.path.join(CSRC, "omx_kernels_fast.cu"),
                                        "-o", os.path.join(BUILD, "fast.o")],
        [nvcc] + ARCH + common + ["-fmad=false"] + inc + ["-c", os.path.join(CSRC, "omx_noalloc.cu"),
                                                           "-o", os.path.join(BUILD, "noalloc.o")],
        [nvcc] + ARCH + common + inc + ["-c", os.path.join(CSRC, "omx_closure.cu"),
                                        "-o", os.path.join(BUILD, "closure.o")],
        [nvcc] + ARCH + common + ["-fmad=false"] + inc + ["-c", os.path.join(CSRC, "omx_fd.cu"),
                                                           "-o", os.path.join(BUILD, "fd.o")],
    ]
    for name in ("omx_capi", "omx_host"):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", _cuda_include(), "-I", CSRC,
                     "-c", os.path.join(CSRC, name + ".cpp"), "-o", os.path.join(BUILD, name + ".o")])
    return jobs


def _newest_source_mtime():
    t = 0.0
    for root in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(root):
            t = max(t, os.path.getmtime(os.path.join(root, f)))
    return t


def build(force=False, verbose=False):
    """Compile the library if any source is newer than the .so; return its path."""
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= _newest_source_mtime():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    jobs = _jobs()

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    objs = [os.path.join(BUILD, n) for n in ("exact.o", "fast.o", "noalloc.o", "closure.o", "fd.o", "omx_capi.o",
                                              "omx_host.o")]
    tmp = OUT + ".tmp"
    run([_nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
