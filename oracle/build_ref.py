"""Build the reference implementation into oracle/_ref/ (TEST INFRASTRUCTURE ONLY).

Compiles the unmodified ceres-raytracer sources where they lie (the directory given as the first
argument, or in CRT_REFERENCE_DIR) with g++ directly, as the reference's own setup.py/CMake
would, into:

  oracle/_ref/golden/_crt<ext>         the reference pybind11 module (src/pybind.cpp +
                                        lib/lodepng/lodepng.cpp), deterministic flags
  oracle/_ref/golden/libref_driver.so  oracle/ref_driver.cpp against the same headers, with the
                                        random_device shim oracle/ref_shim.h force-included
  oracle/_ref/perf/_crt<ext>           the reference module with its CMake release flags
                                        (CMakeLists.txt:15-16) for CPU timing on this host

The golden build uses -O2 -ffp-contract=off (no -march=native) so that its arithmetic rounds
as written; the oracle restatement in crt_oracle.c is compiled the same way.  Nothing here is
shipped: oracle/_ref/ is git-ignored and only read by tests/golden/make_golden.py.
"""
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("CRT_REFERENCE_DIR", "")
OUT = os.path.join(HERE, "_ref")

# CMakeLists.txt:15-16 (release flags of the reference)
CMAKE_RELEASE = ["-O3", "-march=native", "-fno-math-errno", "-fno-signed-zeros", "-fno-trapping-math",
                 "-freciprocal-math", "-fno-rounding-math", "-fno-signaling-nans", "-fexcess-precision=fast"]


def pybind_includes():
    try:
        import pybind11
        return [pybind11.get_include()]
    except ImportError:
        import torch
        return [os.path.join(os.path.dirname(torch.__file__), "include")]


def available(ref=None):
    ref = REF if ref is None else ref
    return bool(ref) and os.path.isfile(os.path.join(ref, "src", "pybind.cpp"))


def _sources(ref):
    return [os.path.join(ref, "src", "pybind.cpp"), os.path.join(ref, "lib", "lodepng", "lodepng.cpp"),
            os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_shim.h")]


def up_to_date(ref):
    """The three outputs exist and are newer than the recipe's own sources (the reference is read-only)."""
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    outs = [os.path.join(OUT, "golden", "_crt" + ext), os.path.join(OUT, "golden", "libref_driver.so"),
            os.path.join(OUT, "perf", "_crt" + ext)]
    if not all(os.path.exists(o) for o in outs):
        return False
    t = min(os.path.getmtime(o) for o in outs)
    return all(os.path.getmtime(s) <= t for s in _sources(ref) + [os.path.abspath(__file__)] if os.path.exists(s))


def build(verbose=False, ref=None):
    global REF
    REF = REF if ref is None else ref
    if not available():
        raise FileNotFoundError("reference sources not found: pass their directory as the first argument or set "
                                "CRT_REFERENCE_DIR")
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]
    incs = ["-I" + os.path.join(REF, "lib"), "-I" + os.path.join(REF, "src"), "-I" + os.path.join(REF, "src", "crt"),
            "-I" + py_inc] + ["-I" + p for p in pybind_includes()]
    common = ["g++", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-include", "iostream", "-w"] + incs
    srcs = [os.path.join(REF, "src", "pybind.cpp"), os.path.join(REF, "lib", "lodepng", "lodepng.cpp")]
    os.makedirs(os.path.join(OUT, "golden"), exist_ok=True)
    os.makedirs(os.path.join(OUT, "perf"), exist_ok=True)
    det = ["-O2", "-ffp-contract=off"]
    jobs = [
        common + det + srcs + ["-o", os.path.join(OUT, "golden", "_crt" + ext)],
        common + det + ["-include", os.path.join(HERE, "ref_shim.h"), os.path.join(HERE, "ref_driver.cpp"),
                        os.path.join(REF, "lib", "lodepng", "lodepng.cpp"),
                        "-o", os.path.join(OUT, "golden", "libref_driver.so")],
        common + CMAKE_RELEASE + srcs + ["-o", os.path.join(OUT, "perf", "_crt" + ext)],
    ]

    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)

    with ThreadPoolExecutor(3) as ex:
        list(ex.map(run, jobs))


if __name__ == "__main__":
    build(verbose=True, ref=sys.argv[1] if len(sys.argv) > 1 else None)
    print("built", OUT)
    sys.exit(0)
