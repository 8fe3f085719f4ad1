"""Build recipe for libbemgpu.so (sm_103a only).

Compiles each translation unit under bemuse_gb300/csrc with nvcc in parallel
and links them into bemuse_gb300/_lib/libbemgpu.so.  Invoked by
__graft_entry__.build() and by `python -m bemuse_gb300.build`.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB = os.path.join(OUT_DIR, "libbemgpu.so")

SOURCES = ["host_api.cpp", "host_mesh.cpp", "host_io.cpp", "host_batch.cpp", "k_influence.cu", "k_lu.cu", "k_tc_gemm.cu", "k_gmres.cu", "noalloc.cu", "k_mlp.cu", "k_mlp_tc.cu", "k_lu_piv.cu", "host_cusolver.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, verbose=False):
    obj = os.path.join(OBJ_DIR, src + ".o")
    cmd = [nvcc(), "-c", os.path.join(SRC, src), "-o", obj, "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fno-fast-math"]
    if src.endswith(".cu"):
        cmd += ARCH + ["-lineinfo"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "cu"] + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, force=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in SOURCES]
    hdrs = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(HERE, "..", "include", "bemgpu.h"))
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) < t for p in srcs + hdrs) and not verbose:
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    objs = [o for o, _ in results]
    cmd = [nvcc(), "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
