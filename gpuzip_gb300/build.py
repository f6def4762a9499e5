"""Builds libgpuinflate.so in place (sm_103a), with nvcc directly: one object per source file,
compiled in parallel, linked with the CUDA runtime statically (the library needs only the
driver, like the one it replaces)."""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libgpuinflate.so")
SOURCES = ["gi_find.cu", "gi_decode.cu", "gi_resolve.cu", "gi_engine.cu", "gi_noalloc.cu", "gi_server.cu", "gi_rescue.cu",
           "gi_tarindex.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(verbose=False, ptxas_info=False):
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    cc = nvcc()
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-O2", "-I", os.path.join(ROOT, "include"),
             "-I", CSRC] + ARCH
    if ptxas_info:
        flags += ["-Xptxas", "-v"]

    def one(src):
        obj = os.path.join(bdir, src.replace(".cu", ".o"))
        srcp = os.path.join(CSRC, src)
        deps = [srcp, os.path.join(ROOT, "include", "gpuinflate.h"), os.path.join(ROOT, "include", "gzrescue_gb300.h")] + [
            os.path.join(CSRC, h) for h in ("gi_common.cuh", "gi_internal.h", "gi_arena.h", "gi_find_cl.h", "gi_tar.h", "gi_model.h", "gi_parallel.h")]
        if not ptxas_info and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
            return obj, ""
        r = subprocess.run([cc, "-c", srcp, "-o", obj] + flags, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(one, SOURCES))
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    objs = [o for o, _ in results]
    link = ["-cudart", "static", "-Xcompiler", "-fPIC", "-Xlinker", "--version-script=" + os.path.join(CSRC, "exports.map")]
    r = subprocess.run([cc, "-shared", "-o", OUT] + objs + ARCH + link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
