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
x86-64 and arm64.  ``build(avx=True)`` (x86-64 only) builds a second library,
``oracle/_ref/libsqg_ref_avx.so``, with the reference's AVX kernels and ``-O3 -mavx2 -mfma``,
as its own CMake build does on x86; it serves timing comparisons, not parity.  The reference tree is found at ``$SQG_REFERENCE_ROOT`` or
``/root/reference``; without it ``build()`` returns None and the tests that need the
library skip.

Usage: ``python oracle/build_ref.py`` (or ``build()`` from the tests).
"""
import concurrent.futures as cf
import glob
import os
import platform
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


def _sources(src, avx=False):
    files = []
    for f in sorted(glob.glob(os.path.join(src, "common", "*.cpp"))):
        if not any(x in os.path.basename(f) for x in _EXCLUDE):
            files.append(f)
    files += sorted(glob.glob(os.path.join(src, "gates", "*.cpp")))
    files += [f for f in sorted(glob.glob(os.path.join(src, "gates", "kernels", "*.cpp"))) if avx or "AVX" not in f]
    for d in ("decomposition", "optimization_engines", "random_unitary", "nn"):
        files += sorted(glob.glob(os.path.join(src, d, "*.cpp")))
    return files


def _openblas():
    import numpy

    libs = glob.glob(os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs", "libscipy_openblas*.so*"))
    if not libs:
        raise RuntimeError("numpy's bundled OpenBLAS was not found")
    return os.path.realpath(libs[0])


def _flags(src, avx=False):
    inc = ["-I" + SHIM] + ["-I" + os.path.join(src, d, "include") for d in _SUBDIRS_INC]
    # -include climits: Optimization_Interface.cpp uses INT_MAX without including <climits>
    opt = ["-O3", "-DUSE_AVX", "-mavx2", "-mfma"] if avx else ["-O2"]
    return ["-std=c++17", "-fPIC", "-fopenmp", "-w", "-include", "climits"] + opt + inc


def _compile(args):
    f, obj, flags = args
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(f):
        return None
    r = subprocess.run(["g++"] + flags + ["-c", f, "-o", obj], capture_output=True, text=True)
    return None if r.returncode == 0 else (f, r.stderr[-2000:])


def build(force=False, verbose=False, avx=False):
    """Build oracle/_ref/libsqg_ref.so (libsqg_ref_avx.so with avx=True); returns its path, or
    None without the reference tree (or, for avx, on a host that is not x86-64)."""
    src = reference_root()
    if src is None or (avx and platform.machine() not in ("x86_64", "AMD64")):
        return None
    lib_path = LIB_PATH.replace(".so", "_avx.so") if avx else LIB_PATH
    obj_dir = OBJ_DIR + "_avx" if avx else OBJ_DIR
    deps = [DRIVER, os.path.join(SHIM, "blas_shim.cpp"), __file__] + glob.glob(os.path.join(SHIM, "tbb", "*.h"))
    if (not force and os.path.exists(lib_path)
            and os.path.getmtime(lib_path) >= max(os.path.getmtime(d) for d in deps)):
        return lib_path
    os.makedirs(obj_dir, exist_ok=True)
    flags = _flags(src, avx)
    jobs = []
    for f in _sources(src, avx) + [DRIVER, os.path.join(SHIM, "blas_shim.cpp")]:
        tag = os.path.relpath(f, src).replace(os.sep, "_") if f.startswith(src) else "local_" + os.path.basename(f)
        jobs.append((f, os.path.join(obj_dir, tag[:-4] + ".o"), flags))
    if force:
        for _, obj, _ in jobs:
            if os.path.exists(obj):
                os.remove(obj)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        errors = [e for e in ex.map(_compile, jobs) if e]
    if errors:
        raise RuntimeError("reference build failed:\n" + "\n".join("%s\n%s" % e for e in errors))
    blas = _openblas()
    tmp = lib_path + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp] + [o for _, o, _ in jobs]
                          + [blas, "-Wl,-rpath," + os.path.dirname(blas), "-Wl,--no-undefined"])
    os.replace(tmp, lib_path)
    if verbose:
        print("built", lib_path, "from", len(jobs), "translation units")
    return lib_path


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True, avx="--avx" in sys.argv)
    if path is None:
        sys.exit("reference tree not found (set SQG_REFERENCE_ROOT)")
