"""Compile every native part of the project in-tree (no cmake, no setup.py).

Outputs (all git-ignored):
  ceres-raytracer_gb300/libcrt_gpu.so      CUDA kernels for sm_103a + the C ABI (include/crt_gpu.h)
  ceres-raytracer_gb300/_crt<ext>          pybind11 module with the reference `_crt` surface
  ceres-raytracer_gb300/libcrt_scene.so    synthetic scene generators (host C++)
  oracle/libcrt_oracle.so                  CPU oracle (test infrastructure)

Translation units compile in parallel; objects are rebuilt only when a source or header is
newer than the object.  nvcc gets exactly one -gencode (arch=compute_103a,code=sm_103a).
"""
import glob
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # ceres-raytracer_gb300/
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJDIR = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")
ORACLE = os.path.join(REPO, "oracle")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
CUDA_HOME = os.path.dirname(os.path.dirname(NVCC)) if os.path.isabs(NVCC) else "/usr/local/cuda"
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC] + GENCODE
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I" + INCLUDE, "-I" + CSRC]

LIB_GPU = os.path.join(PKG, "libcrt_gpu.so")
LIB_SCENE = os.path.join(PKG, "libcrt_scene.so")
LIB_ORACLE = os.path.join(ORACLE, "libcrt_oracle.so")
EXT = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
MOD_CRT = os.path.join(PKG, "_crt" + EXT)


def _pybind_include():
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        import torch
        return os.path.join(os.path.dirname(torch.__file__), "include")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return r


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def build(verbose=False, jobs=None):
    os.makedirs(OBJDIR, exist_ok=True)
    hdrs = _headers()
    cu_srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    host_srcs = [os.path.join(CSRC, "mesh.cpp")]
    compile_jobs = []
    gpu_objs = []
    for src in cu_srcs:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        gpu_objs.append(obj)
        if _newer(obj, [src] + hdrs):
            compile_jobs.append(([NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj], obj))
    for src in host_srcs:
        if not os.path.exists(src):
            continue
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        gpu_objs.append(obj)
        if _newer(obj, [src] + hdrs):
            compile_jobs.append((["g++"] + CXX_FLAGS + ["-fopenmp", "-c", src, "-o", obj], obj))
    # host-only libraries: single command each
    scene_src = os.path.join(CSRC, "scenes.cpp")
    oracle_src = os.path.join(ORACLE, "crt_oracle.c")
    link_jobs_independent = []
    if _newer(LIB_SCENE, [scene_src]):
        link_jobs_independent.append(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                                      scene_src, "-o", LIB_SCENE])
    if _newer(LIB_ORACLE, [oracle_src, os.path.join(ORACLE, "crt_oracle.h")]):
        link_jobs_independent.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                                      oracle_src, "-o", LIB_ORACLE, "-lm"])
    njobs = jobs or max(2, min(16, os.cpu_count() or 4))
    with ThreadPoolExecutor(njobs) as ex:
        futs = [ex.submit(_run, c, verbose) for c, _ in compile_jobs]
        futs += [ex.submit(_run, c, verbose) for c in link_jobs_independent]
        for f in futs:
            f.result()
    if gpu_objs and _newer(LIB_GPU, gpu_objs):
        _run([NVCC] + GENCODE + ["-shared", "-o", LIB_GPU] + gpu_objs +
             ["-Xcompiler", "-fopenmp", "-lgomp", "-Xlinker", "-rpath,$ORIGIN"], verbose)
    mod_src = os.path.join(CSRC, "crt_module.cpp")
    if os.path.exists(mod_src) and _newer(MOD_CRT, [mod_src, LIB_GPU] + hdrs):
        py_inc = sysconfig.get_paths()["include"]
        _run(["g++"] + CXX_FLAGS + ["-shared", "-fvisibility=hidden", "-I" + py_inc, "-I" + _pybind_include(),
                                    mod_src, "-o", MOD_CRT, "-L" + PKG, "-l:libcrt_gpu.so",
                                    "-Wl,-rpath,$ORIGIN"], verbose)
    return {"gpu": LIB_GPU, "scene": LIB_SCENE, "oracle": LIB_ORACLE, "module": MOD_CRT}


if __name__ == "__main__":
    print(build(verbose=True))
