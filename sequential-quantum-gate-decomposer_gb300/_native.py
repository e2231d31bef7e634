"""Loader and ctypes bindings of the engine's C ABI (include/sqg.h).

The shared library ``libsqg.so`` is built in-tree by :func:`build` with nvcc for
sm_103a.  There is no CPU fallback: every entry point of this package raises if the
library or a CUDA device is missing.
"""
import ctypes
import os
import subprocess
import sys
import threading

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
LIB_PATH = os.path.join(PKG_DIR, "libsqg.so")
BUILD_DIR = os.path.join(PKG_DIR, "_build")

CU_SOURCES = ["engine.cu", "decompose.cu", "loop.cu", "probe.cu", "mlp.cu", "ragged.cu", "gemm_tc.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]

# status codes and limits (sqg.h)
SQG_OK = 0
SQG_ERR_INVALID_ARGUMENT = 1
SQG_ERR_UNSUPPORTED = 2
SQG_ERR_WORKSPACE = 3
SQG_NOALLOC_SCRATCH_BYTES = 32 << 20
STATUS_TEXT = {0: "ok", 1: "invalid argument", 2: "unsupported configuration", 3: "workspace too small",
               4: "CUDA error", 5: "wrong number of parameters"}


class SQGError(RuntimeError):
    """Error reported by the engine through a non-zero status code."""


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES]


def _deps():
    deps = _sources() + [os.path.join(INCLUDE, "sqg.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return deps


def needs_build():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False):
    """Compile every CUDA translation unit for sm_103a (in parallel) and link libsqg.so."""
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc] + NVCC_FLAGS + ["-I", INCLUDE, "-c", "-o", obj, src]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + [
        "-lcudart"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None
_lock = threading.Lock()


def _declare(lib):
    c_int, c_ll, c_sz, vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_size_t, ctypes.c_void_p
    lib.sqg_status_string.restype = ctypes.c_char_p
    lib.sqg_status_string.argtypes = [c_int]
    lib.sqg_last_error.restype = ctypes.c_char_p
    lib.sqg_last_error.argtypes = []
    lib.sqg_circuit_create.argtypes = [c_int, vp, c_int, ctypes.POINTER(vp)]
    lib.sqg_circuit_destroy.argtypes = [vp]
    for f in ("sqg_circuit_param_num", "sqg_circuit_qbit_num", "sqg_circuit_gate_num"):
        getattr(lib, f).argtypes = [vp]
    lib.sqg_cost_grad_workspace_bytes.restype = c_sz
    lib.sqg_cost_grad_workspace_bytes.argtypes = [vp, c_int, c_int, c_int]
    lib.sqg_cost_grad_checkpoint_workspace_bytes.restype = c_sz
    lib.sqg_cost_grad_checkpoint_workspace_bytes.argtypes = [vp, c_int, c_int, c_int]
    lib.sqg_cost_grad.argtypes = [vp, vp, c_int, vp, c_int, c_ll, c_int, c_int, vp, vp, c_int, vp, c_sz, vp]
    lib.sqg_cost_grad_noalloc.argtypes = [vp, vp, c_int, vp, c_int, c_ll, c_int, c_int, vp, vp, c_int, vp]
    lib.sqg_ragged_create.argtypes = [vp, vp, c_int, c_int, vp, ctypes.POINTER(vp)]
    lib.sqg_ragged_destroy.argtypes = [vp]
    lib.sqg_ragged_workspace_bytes.restype = c_sz
    lib.sqg_ragged_workspace_bytes.argtypes = [vp]
    lib.sqg_ragged_layout.argtypes = [vp, vp, vp]
    lib.sqg_ragged_cost_grad.argtypes = [vp, vp, vp, c_int, vp, vp, vp, c_sz, vp]
    lib.sqg_apply_workspace_bytes.restype = c_sz
    lib.sqg_apply_workspace_bytes.argtypes = [vp, c_int]
    lib.sqg_apply.argtypes = [vp, vp, c_int, vp, c_int, c_ll, c_ll, c_int, vp, c_sz, vp]
    lib.sqg_apply_from_right.argtypes = [vp, vp, vp, c_int, c_ll, vp, c_sz, vp]
    lib.sqg_combined_unitary.argtypes = [vp, vp, vp, c_int, vp, vp, c_sz, vp]
    lib.sqg_probe_fp64_scratch_bytes.restype = c_sz
    lib.sqg_probe_fp64_scratch_bytes.argtypes = []
    lib.sqg_probe_fp64_tflops.argtypes = [ctypes.POINTER(ctypes.c_double), c_int, vp, c_sz, vp]
    lib.sqg_decompose_workspace_bytes.restype = c_sz
    lib.sqg_decompose_workspace_bytes.argtypes = [vp, c_int, c_int]
    lib.sqg_state_workspace_bytes.restype = c_sz
    lib.sqg_state_workspace_bytes.argtypes = [vp, c_int]
    lib.sqg_state_block_count.argtypes = [vp]
    lib.sqg_circuit_set_partitions.argtypes = [vp, vp, c_int]
    lib.sqg_apply_state.argtypes = [vp, vp, c_int, vp, c_ll, c_int, vp, c_sz, vp]
    lib.sqg_decompose_batched_adam.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, vp, vp, ctypes.c_double,
                                               c_int, ctypes.c_double, c_int, c_int, c_ll, c_int, ctypes.c_uint64, vp]
    lib.sqg_adam_loop_workspace_bytes.restype = c_sz
    lib.sqg_adam_loop_workspace_bytes.argtypes = [vp, c_int]
    lib.sqg_decompose_adam_loop.argtypes = [vp, vp, c_int, c_int, c_int, vp, vp, vp, vp, ctypes.c_double, c_int,
                                            ctypes.c_double, c_int, c_int, c_ll, c_int, ctypes.c_double,
                                            ctypes.c_uint64, vp, c_sz, vp]
    lib.sqg_bfgs_loop_workspace_bytes.restype = c_sz
    lib.sqg_bfgs_loop_workspace_bytes.argtypes = [vp, c_int]
    lib.sqg_decompose_bfgs_loop.argtypes = [vp, vp, c_int, c_int, c_int, vp, vp, vp, vp, ctypes.c_double, c_int, c_int,
                                            c_int, c_int, ctypes.c_ulonglong, vp, c_sz, vp]
    lib.sqg_decompose_structures_workspace_bytes.restype = c_sz
    lib.sqg_decompose_structures_workspace_bytes.argtypes = [vp, c_int, c_int]
    lib.sqg_decompose_structures.argtypes = [vp, vp, vp, c_ll, c_int, c_int, c_int, c_int, vp, vp, vp, vp,
                                             ctypes.c_double, c_int, c_int, c_int, c_int, ctypes.c_ulonglong, vp, c_sz,
                                             vp]
    lib.sqg_decompose_batched.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, vp, vp, ctypes.c_double,
                                          c_int, c_int, c_int, c_int, ctypes.c_ulonglong, vp, c_sz, vp]
    lib.sqg_decompose_structures_adam_workspace_bytes.restype = c_sz
    lib.sqg_decompose_structures_adam_workspace_bytes.argtypes = [vp, c_int]
    lib.sqg_decompose_structures_adam.argtypes = [vp, vp, vp, c_ll, c_int, c_int, c_int, c_int, vp, vp, vp, vp,
                                                  ctypes.c_double, c_int, ctypes.c_double, c_int, c_int, c_ll, c_int,
                                                  ctypes.c_ulonglong, vp, c_sz, vp]


def lib():
    """The loaded engine library (built on first use if absent)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if needs_build():
                    build()
                l = ctypes.CDLL(LIB_PATH)
                _declare(l)
                _lib = l
    return _lib


def probe_fp64_tflops(active_lanes=32):
    """Live FP64 FMA peak of the current CUDA device (TFLOP/s)."""
    from . import _device as dev

    dev.require_cuda()
    l = lib()
    nbytes = l.sqg_probe_fp64_scratch_bytes()
    buf = dev.torch.empty(nbytes, dtype=dev.torch.uint8, device="cuda")
    out = ctypes.c_double()
    check(l.sqg_probe_fp64_tflops(ctypes.byref(out), int(active_lanes), buf.data_ptr(), nbytes, dev.stream_ptr()),
          "sqg_probe_fp64_tflops")
    return out.value


def check(status, what=""):
    if status != SQG_OK:
        msg = lib().sqg_last_error().decode(errors="replace")
        raise SQGError("%s: %s (%s)" % (what, STATUS_TEXT.get(status, "status %d" % status), msg))


EXPORTED_SYMBOLS = [
    "sqg_status_string", "sqg_last_error", "sqg_circuit_create", "sqg_circuit_destroy", "sqg_circuit_param_num",
    "sqg_circuit_qbit_num", "sqg_circuit_gate_num", "sqg_cost_grad_workspace_bytes",
    "sqg_cost_grad_checkpoint_workspace_bytes", "sqg_cost_grad", "sqg_cost_grad_noalloc", "sqg_apply_workspace_bytes",
    "sqg_apply",
    "sqg_apply_from_right", "sqg_combined_unitary", "sqg_decompose_workspace_bytes", "sqg_decompose_batched", "sqg_decompose_batched_adam",
    "sqg_adam_loop_workspace_bytes", "sqg_decompose_adam_loop", "sqg_decompose_structures_workspace_bytes",
    "sqg_bfgs_loop_workspace_bytes", "sqg_decompose_bfgs_loop",
    "sqg_decompose_structures", "sqg_decompose_structures_adam_workspace_bytes", "sqg_decompose_structures_adam",
    "sqg_state_workspace_bytes", "sqg_state_block_count", "sqg_apply_state", "sqg_circuit_set_partitions",
    "sqg_probe_fp64_scratch_bytes", "sqg_probe_fp64_tflops",
    "sqg_mlp_gemm_bf16", "sqg_mlp_to_bf16", "sqg_mlp_relu_backward", "sqg_mlp_col_sum", "sqg_mlp_adam",
    "sqg_mlp_angle_head", "sqg_mlp_features",
    "sqg_ragged_create", "sqg_ragged_destroy", "sqg_ragged_workspace_bytes", "sqg_ragged_layout",
    "sqg_ragged_cost_grad", "sqg_mlp_gemm_tc", "sqg_mlp_transpose_bf16",
]
