"""Build recipe of libaenet_gb300.so (sm_103a only, in-tree).

Each translation unit under ``csrc/`` is compiled in parallel by nvcc into
``_build/*.o`` and linked into ``aenet_gb300/libaenet_gb300.so`` with the
CUDA runtime linked statically, so the library has no dependency on the
PyTorch installation.  ``capi.cpp`` is compiled with ``-ffp-contract=off``
(unfused reciprocal-lattice arithmetic, see its header).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaenet_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["k_neighbors.cu", "k_cheb_order.cu", "k_atom.cu", "k_cheb_f32.cu", "k_cheb_mom.cu", "k_cheb_f64.cu", "k_behler.cu", "k_mlp.cu", "k_mlp_tc.cu",
           "k_cheb_tangent.cu", "k_cheb_jac.cu", "k_train.cu", "k_md.cu", "capi.cpp", "noalloc.cu"]


def _nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime():
    t = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(src, force, verbose):
    nvcc = _nvcc()
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src.rsplit(".", 1)[0] + ".o")
    if (not force and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(path), _headers_mtime())):
        return obj
    xc = "-fPIC,-fvisibility=hidden"
    if src.endswith(".cpp"):
        xc += ",-ffp-contract=off"
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", xc,
           "-Xptxas", "-warn-spills", "-c", path, "-o", obj + ".tmp"]
    if src.endswith(".cpp"):
        cmd.insert(1, "-x")
        cmd.insert(2, "cu")
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
