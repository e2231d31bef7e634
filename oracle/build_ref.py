"""ORACLE build recipe — test infrastructure only.

Compiles SQUANDER's own C++ sources for the decomposition path, where they lie in the
reference tree, into ``oracle/_ref/libsqg_ref.so`` together with ``oracle/ref_driver.cpp``
(a C interface over the reference's classes).  Nothing from the reference tree is copied:
the sources are compiled in place, and the objects and the library are written under
``oracle/_ref/`` only (git-ignored).

The reference's CMake build is not used.  Its three outside interfaces get test-only
stand-ins, none of which computes anything the decomposition path's results depend on
except the BLAS routines, which stay OpenBLAS:

* ``oracle/ref_shim/tbb/`` — a serial oneTBB stand-in (threading only; every parallel loop
  runs in index order on the calling thread);
* ``oracle/ref_shim/Config.h`` — the CMake-generated configuration header, with no vendor
  BLAS selected (the reference's ``BLAS==0`` branches);
* ``oracle/ref_shim/blas_shim.cpp`` — ``cblas_zgemm``/``cblas_cgemm``/``cblas_dznrm2`` and
  ``LAPACKE_zgesdd``/``cgesdd`` forwarded to the OpenBLAS build bundled with numpy.

Kernels are the reference's portable ones (no ``USE_AVX``), so the same recipe works on
x86-64 and arm64.  The reference tree is found at ``$SQG_REFERENCE_ROOT`` or
``/root/reference``; without it ``build()`` returns None and the tests that need the
library skip.

Usage: ``python oracle/build_ref.py`` (or ``build()`` from the tests).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_PATH = os.path.join(OUT_DIR, "libsqg_ref.so")
SHIM = os.path.join(HERE, "ref_shim")
DRIVER = os.path.join(HERE, "ref_driver.cpp")

# Sources of the path: matrices and helpers, every gate class (Gates_block creates any of
# them), the portable kernels, the decomposition classes and the optimisation engines
# (Optimization_Interface dispatches to all of them).  numpy_interface / MPI / DFE / Groq
# glue is left out: it belongs to the Python extension and the accelerator back ends.
_EXCLUDE = ("numpy_interface", "mpi_base", "common_DFE", "common_GROQ")
_SUBDIRS_INC = ("common", "decomposition", "gates", "gates/kernels", "optimization_engines",
                "random_unitary", "nn")


def reference_root():
    root = os.environ.get("SQG_REFERENCE_ROOT", "/root/reference")
    src = os.path.join(root, "squander", "src-cpp")
    return src if os.path.isdir(src) else None


def _sources(src):
    files = []
    for f in sorted(glob.glob(os.path.join(src, "common", "*.cpp"))):
        if not any(x in os.path.basename(f) for x in _EXCLUDE):
            files.append(f)
    files += sorted(glob.glob(os.path.join(src, "gates", "*.cpp")))
    files += [f for f in sorted(glob.glob(os.path.join(src, "gates", "kernels", "*.cpp"))) if "AVX" not in f]
    for d in ("decomposition", "optimization_engines", "random_unitary", "nn"):
        files += sorted(glob.glob(os.path.join(src, d, "*.cpp")))
    return files


def _openblas():
    import numpy

    libs = glob.glob(os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "libscipy_openblas*.so*"))
    if not libs:
        raise RuntimeError("numpy's bundled OpenBLAS was not found")
    return os.path.realpath(libs[0])


def _flags(src):
    inc = ["-I" + SHIM] + ["-I" + os.path.join(src, d, "include") for d in _SUBDIRS_INC]
    # -include climits: Optimization_Interface.cpp uses INT_MAX without including <climits>
    return ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-w", "-include", "climits"] + inc


def _compile(args):
    f, obj, flags = args
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(f):
        return None
    r = subprocess.run(["g++"] + flags + ["-c", f, "-o", obj], capture_output=True, text=True)
    return None if r.returncode == 0 else (f, r.stderr[-2000:])


def build(force=False, verbose=False):
    """Build oracle/_ref/libsqg_ref.so; returns its path, or None without the reference tree."""
    src = reference_root()
    if src is None:
        return None
    deps = [DRIVER, os.path.join(SHIM, "blas_shim.cpp"), __file__] + glob.glob(os.path.join(SHIM, "tbb", "*.h"))
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    flags = _flags(src)
    jobs = []
    for f in _sources(src) + [DRIVER, os.path.join(SHIM, "blas_shim.cpp")]:
        tag = os.path.relpath(f, src).replace(os.sep, "_") if f.startswith(src) else "local_" + os.path.basename(f)
        jobs.append((f, os.path.join(OBJ_DIR, tag[:-4] + ".o"), flags))
    if force:
        for _, obj, _ in jobs:
            if os.path.exists(obj):
                os.remove(obj)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        errors = [e for e in ex.map(_compile, jobs) if e]
    if errors:
        raise RuntimeError("reference build failed:\n" + "\n".join("%s\n%s" % e for e in errors))
    blas = _openblas()
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp] + [o for _, o, _ in jobs]
                          + [blas, "-Wl,-rpath," + os.path.dirname(blas), "-Wl,--no-undefined"])
    os.replace(tmp, LIB_PATH)
    if verbose:
        print("built", LIB_PATH, "from", len(jobs), "translation units")
    return LIB_PATH


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True)
    if path is None:
        sys.exit("reference tree not found (set SQG_REFERENCE_ROOT)")
