"""Builds the in-tree shared library mypbr_gb300/_lib/libmypbr_gb300.so.

Every translation unit is compiled by nvcc for sm_103a only (one -gencode),
in parallel, then linked with the static CUDA runtime so the library loads on a
machine without a GPU (calls that need one then return MYPBR_ERR_NO_DEVICE).
The C ABI the library exports is include/mypbr_gpu.h.
"""
import concurrent.futures
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libmypbr_gb300.so")
OBJ_DIR = os.path.join(OUT_DIR, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]
CU_FLAGS = ARCH + COMMON + ["-lineinfo", "--use_fast_math", "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]
CPP_FLAGS = ARCH + COMMON + ["-Xcompiler", "-Wall"]
# Sources whose FP64 arithmetic must round like the reference's (no fused multiply-add)
NO_FMA = {"post.cu"}


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "device", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    return cu, cpp


def _headers_digest():
    h = hashlib.sha1()
    for path in sorted(glob.glob(os.path.join(CSRC, "**", "*.h*"), recursive=True)) + [
            os.path.join(ROOT, "include", "mypbr_gpu.h")]:
        with open(path, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _compile(args):
    src, obj, flags, extra = args
    cmd = [nvcc(), *flags, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose=False, extra_flags=()):
    """Compiles and links the library if any source changed; returns its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    cu, cpp = sources()
    digest = _headers_digest() + "|" + " ".join(extra_flags)
    stamp = os.path.join(OBJ_DIR, "headers.sha1")
    headers_changed = not os.path.exists(stamp) or open(stamp).read() != digest
    jobs = []
    for src in cu + cpp:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        flags = CU_FLAGS if src.endswith(".cu") else CPP_FLAGS
        if os.path.basename(src) in NO_FMA:
            flags = flags + ["-fmad=false"]
        if headers_changed or not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src):
            jobs.append((src, obj, flags, list(extra_flags)))
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(workers) as ex:
            for err in ex.map(_compile, jobs):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    objs = [os.path.join(OBJ_DIR, os.path.basename(s) + ".o") for s in cu + cpp]
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


def build_oracle():
    """Builds the FP64 checker (oracle/_build/libmypbr_oracle.so) and, where the
    reference checkout exists, its golden-vector harness (oracle/_ref)."""
    oracle = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-C", oracle], check=True)
    subprocess.run(["make", "-s", "-C", oracle, "ref-if-present"], check=True)


def reference_dir():
    """The reference checkout's folder as oracle/Makefile knows it (the
    REFERENCE variable there), or None where it is absent."""
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(ROOT, "oracle"), "reference-dir"],
                       capture_output=True, text=True)
    path = r.stdout.strip()
    return path if r.returncode == 0 and path else None


if __name__ == "__main__":
    print(build(verbose=True))
    build_oracle()
