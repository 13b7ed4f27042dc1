"""Builds the engine's shared library in-tree with nvcc for sm_103a.

    fast-rbd-gradients_gb300/csrc/*.cu, *.cpp  ->  fast-rbd-gradients_gb300/frg/libfrg.so

Translation units compile in parallel into fast-rbd-gradients_gb300/_build/;
the link uses the shared CUDA runtime so that the library and PyTorch share one
runtime (and one primary context) when both are loaded.

The robot is compiled in: the iiwa_14 by default, another 7-joint serial arm
from a tables header written by frg/urdf.py when FRG_MODEL_TABLES names it
(in-tree build), or build_model(tables, out_dir) for a library of its own.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
HOST_SRC = os.path.join(PKG_ROOT, "host")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(PKG_ROOT, "frg", "libfrg.so")
BIN_DIR = os.path.join(PKG_ROOT, "frg", "bin")
INCLUDE = os.path.join(REPO_ROOT, "include")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfrg.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _model_flags(tables):
    return [f'-DFRG_MODEL_TABLES="{os.path.abspath(tables)}"'] if tables else []


def build(force=False, verbose=False, ptxas_info=False):
    """Compile and link libfrg.so if any source or header changed; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    tables = os.environ.get("FRG_MODEL_TABLES") or None
    stamp = os.path.join(BUILD_DIR, "model.txt")
    model_id = os.path.abspath(tables) if tables else "default"
    if not os.path.exists(stamp) or open(stamp).read() != model_id:
        force = True  # another robot: every translation unit changes
    hdrs = _headers() + ([tables] if tables else [])
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        if force or _stale(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if (ptxas_info and src.endswith(".cu")) else []
            jobs.append((src, obj, [nvcc] + ARCH_FLAGS + COMMON + _model_flags(tables) + extra +
                         ["-c", src, "-o", obj]))

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return src, r.stderr

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for src, log in ex.map(run, jobs):
                if ptxas_info and log:
                    print(log)
    objs = [os.path.join(BUILD_DIR, os.path.basename(s) + ".o") for s in sources()]
    if force or jobs or _stale(LIB_PATH, objs):
        cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-cudart", "shared", "-o", LIB_PATH] + objs + [
            "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libfrg.so failed:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(model_id)
    build_host_tools(nvcc, force, verbose)
    return LIB_PATH


def build_model(tables, out_dir, verbose=False):
    """libfrg.so for the robot of a tables header (frg/urdf.py) in out_dir,
    beside the in-tree library; returns its path."""
    nvcc = _nvcc()
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    jobs = [(src, os.path.join(obj_dir, os.path.basename(src) + ".o")) for src in sources()]

    def run(job):
        src, obj = job
        cmd = [nvcc] + ARCH_FLAGS + COMMON + _model_flags(tables) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(run, jobs))
    lib = os.path.join(out_dir, "libfrg.so")
    cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-cudart", "shared", "-o", lib] + [o for _, o in jobs] + [
        "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {lib} failed:\n{r.stdout}\n{r.stderr}")
    return lib


def build_host_tools(nvcc, force=False, verbose=False):
    """C++ host code over the C ABI, linked to libfrg.so: host/lib<name>.cpp ->
    frg/lib<name>.so (libraries bench.py drives), other host/*.cpp ->
    frg/bin/<name> (executables); host/*.cu -> frg/bin/<name>, standalone
    CUDA tools (sm_103a) that do not link libfrg.so."""
    if not os.path.isdir(HOST_SRC):
        return
    os.makedirs(BIN_DIR, exist_ok=True)
    for f in sorted(os.listdir(HOST_SRC)):
        if f.endswith(".cu"):
            src, out = os.path.join(HOST_SRC, f), os.path.join(BIN_DIR, f[:-3])
            if force or _stale(out, [src]):
                cmd = [nvcc] + ARCH_FLAGS + ["-O3", "-std=c++17", "-lineinfo", src, "-o", out]
                if verbose:
                    print(" ".join(cmd), flush=True)
                r = subprocess.run(cmd, capture_output=True, text=True)
                if r.returncode != 0:
                    raise RuntimeError(f"build of {f} failed:\n{r.stdout}\n{r.stderr}")
            continue
        if not f.endswith(".cpp"):
            continue
        src = os.path.join(HOST_SRC, f)
        shared = f.startswith("lib")
        out = os.path.join(os.path.dirname(LIB_PATH), f[:-4] + ".so") if shared else os.path.join(BIN_DIR, f[:-4])
        if not force and not _stale(out, [src, LIB_PATH, os.path.join(INCLUDE, "frg.h")]):
            continue
        rpath = "-rpath,$ORIGIN" if shared else "-rpath,$ORIGIN/.."
        cmd = [nvcc, "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", out, "-L", os.path.dirname(LIB_PATH), "-lfrg",
               "-cudart", "shared", "-Xlinker", rpath, "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        if shared:
            cmd[1:1] = ["-shared", "-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of {f} failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
