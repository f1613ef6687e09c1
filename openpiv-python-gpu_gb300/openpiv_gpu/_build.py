"""Builds libpiv_gb300.so from csrc/ with nvcc for sm_103a (in-tree, into _lib/)."""

import concurrent.futures
import os
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libpiv_gb300.so")
# The checked build (index checks in the tensor-core and refinement kernels,
# see piv_bounds_check): a test and debugging aid, built only on request.
CHECKED_PATH = os.path.join(LIB_DIR, "checked", "libpiv_gb300_checked.so")
SOURCES = ["piv_correlate.cu", "piv_correlate_f64.cu", "piv_tensor.cu", "piv_refine.cu", "piv_deform.cu", "piv_validate.cu", "piv_smoothn.cu", "piv_abi.cu"]
NVCC_FLAGS = ["-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
              "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(path=LIB_PATH):
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h")) and os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    inc = os.path.join(os.path.dirname(ROOT), "include")
    if os.path.isdir(inc):
        for f in os.listdir(inc):
            if os.path.getmtime(os.path.join(inc, f)) > t:
                return True
    return False


def build(force=False, verbose=False, checked=False):
    """Compiles every translation unit in parallel and links the shared
    library (``checked``: the checked build, with -DPIV_BOUNDS_CHECK)."""
    path = CHECKED_PATH if checked else LIB_PATH
    if not force and not _stale(path):
        return path
    out_dir = os.path.dirname(path)
    os.makedirs(out_dir, exist_ok=True)
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + (["-DPIV_BOUNDS_CHECK"] if checked else [])

    def compile_one(src):
        obj = os.path.join(obj_dir, src.replace(".cu", ".o"))
        cmd = [nvcc] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = path + ".tmp"
    cmd = [nvcc, "-shared", "--cudart", "static", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, path)
    return path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
