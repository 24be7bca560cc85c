"""ctypes binding of libqflex_gb300.so (the C ABI in include/qflex_gb300.h).

The shared library is the product: there is no Python or CPU fallback.
Loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

LIB_PATH = Path(__file__).resolve().parent / "libqflex_gb300.so"

OK, ERR_INPUT, ERR_CUDA, ERR_ARG = 0, 1, 2, 3
FP32, TF32X3, BF16X3, FP16X3, FP64, FP64_FF = 0, 1, 2, 3, 4, 5
PRECISIONS = {"fp32": FP32, "tf32x3": TF32X3, "bf16x3": BF16X3, "fp16x3": FP16X3, "fp64": FP64,
              "fp64ff": FP64_FF}

# Every symbol include/qflex_gb300.h declares.
EXPORTS = (
    "qflex_gb300_create", "qflex_gb300_destroy", "qflex_gb300_last_error",
    "qflex_gb300_set_precision", "qflex_gb300_set_stream", "qflex_gb300_evaluate",
    "qflex_gb300_evaluate_many", "qflex_gb300_result_count", "qflex_gb300_result_state",
    "qflex_gb300_result_amplitude", "qflex_gb300_result_initial_state",
    "qflex_gb300_result_final_state", "qflex_gb300_last_stats", "qflex_gb300_last_shapes",
    "qflex_gb300_last_gemms", "qflex_gb300_set_profiling", "qflex_gb300_last_ops",
    "qflex_gb300_set_option", "qflex_gb300_get_option", "qflex_gb300_set_tc_variant",
    "qflex_gb300_permute", "qflex_gb300_check_permute",
    "qflex_gb300_reorder",
    "qflex_gb300_multiply", "qflex_gb300_synchronize", "qflex_gb300_mlp_param_count",
    "qflex_gb300_mlp_work_floats", "qflex_gb300_mlp_forward", "qflex_gb300_mlp_loss_grad",
    "qflex_gb300_mlp_adam", "qflex_gb300_multiply_skinny_noalloc",
    "qflex_gb300_circuit_load", "qflex_gb300_circuit_free", "qflex_gb300_circuit_num_active_qubits",
    "qflex_gb300_circuit_depth", "qflex_gb300_circuit_gate_count", "qflex_gb300_circuit_gate",
    "qflex_gb300_grid_load", "qflex_gb300_ordering_load",
)


class QflexGb300Error(RuntimeError):
    """An error reported through the C ABI. ``code`` is one of ERR_*."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class Stats(C.Structure):
    _fields_ = [
        ("device_ms", C.c_double),
        ("gemm_flop", C.c_double),
        ("permute_bytes", C.c_double),
        ("arena_bytes", C.c_double),
        ("reference_bytes", C.c_double),
        ("n_ops", C.c_size_t),
        ("n_leaves", C.c_size_t),
        ("batch", C.c_size_t),
        ("launches", C.c_size_t),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
_lock = threading.Lock()


def load_library(path: Optional[Path] = None) -> C.CDLL:
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"{p} is missing: build it with `python -m qflex_gb300.build` "
                "(qflex_gb300 has no fallback path)")
        lib = C.CDLL(str(p))
        vp, cp, sz, dbl, i = C.c_void_p, C.c_char_p, C.c_size_t, C.c_double, C.c_int
        sig = {
            "qflex_gb300_create": (i, [i, i, C.POINTER(vp)]),
            "qflex_gb300_destroy": (None, [vp]),
            "qflex_gb300_last_error": (cp, [vp]),
            "qflex_gb300_set_precision": (i, [vp, i]),
            "qflex_gb300_set_stream": (i, [vp, vp]),
            "qflex_gb300_evaluate": (i, [vp, cp, cp, cp, cp, cp, dbl]),
            "qflex_gb300_evaluate_many": (i, [vp, cp, cp, cp, cp, C.POINTER(cp), sz, dbl]),
            "qflex_gb300_result_count": (sz, [vp]),
            "qflex_gb300_result_state": (cp, [vp, sz]),
            "qflex_gb300_result_amplitude": (i, [vp, sz, C.POINTER(dbl), C.POINTER(dbl)]),
            "qflex_gb300_result_initial_state": (cp, [vp]),
            "qflex_gb300_result_final_state": (cp, [vp, sz]),
            "qflex_gb300_last_stats": (i, [vp, C.POINTER(Stats)]),
            "qflex_gb300_last_shapes": (sz, [vp, C.POINTER(sz), sz]),
            "qflex_gb300_last_gemms": (sz, [vp, C.POINTER(sz), sz]),
            "qflex_gb300_set_profiling": (i, [vp, i]),
            "qflex_gb300_set_option": (i, [vp, C.c_char_p, dbl]),
            "qflex_gb300_get_option": (i, [vp, C.c_char_p, C.POINTER(dbl)]),
            "qflex_gb300_set_tc_variant": (i, [vp, sz, sz, sz, i]),
            "qflex_gb300_last_ops": (sz, [vp, C.POINTER(dbl), sz]),
            "qflex_gb300_permute": (i, [vp, vp, vp, sz, C.POINTER(sz), C.POINTER(sz), sz, sz]),
            "qflex_gb300_check_permute": (i, [sz, C.POINTER(sz), C.POINTER(sz), vp, vp]),
            "qflex_gb300_reorder": (i, [vp, vp, vp, sz, C.POINTER(sz), C.POINTER(sz)]),
            "qflex_gb300_multiply": (i, [vp, vp, vp, vp, sz, sz, sz, sz, sz]),
            "qflex_gb300_synchronize": (i, [vp]),
            "qflex_gb300_multiply_skinny_noalloc": (i, [vp, vp, vp, sz, sz, sz, vp, C.c_char_p, sz]),
            "qflex_gb300_mlp_param_count": (sz, [i, i]),
            "qflex_gb300_mlp_work_floats": (sz, [sz, i]),
            "qflex_gb300_mlp_forward": (i, [vp, vp, vp, sz, i, i, vp, vp]),
            "qflex_gb300_mlp_loss_grad": (i, [vp, vp, vp, vp, sz, i, i, vp, vp, vp]),
            "qflex_gb300_mlp_adam": (i, [vp, vp, vp, vp, vp, sz, i, C.c_float]),
            "qflex_gb300_circuit_load": (i, [cp, C.POINTER(vp), cp, sz]),
            "qflex_gb300_circuit_free": (None, [vp]),
            "qflex_gb300_circuit_num_active_qubits": (sz, [vp]),
            "qflex_gb300_circuit_depth": (sz, [vp]),
            "qflex_gb300_circuit_gate_count": (sz, [vp]),
            "qflex_gb300_circuit_gate": (i, [vp, sz, C.POINTER(cp), C.POINTER(cp), C.POINTER(sz), C.POINTER(sz), sz,
                                             C.POINTER(sz), C.POINTER(dbl), sz, C.POINTER(sz)]),
            "qflex_gb300_grid_load": (i, [cp, C.POINTER(sz), C.POINTER(sz), C.POINTER(sz), sz, C.POINTER(sz), cp,
                                          sz]),
            "qflex_gb300_ordering_load": (i, [cp, cp, sz, C.POINTER(sz), C.POINTER(sz), cp, sz]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def check_permute(src, dims: Sequence[int], new_order: Sequence[int]):
    """Runs the permutation kernel's index schedule on a host numpy array
    (complex64) and returns the permuted copy."""
    import numpy as np
    lib = load_library()
    a = np.ascontiguousarray(src, dtype=np.complex64).reshape(-1)
    out = np.zeros_like(a)
    rc = lib.qflex_gb300_check_permute(len(dims), _sizes(dims), _sizes(new_order),
                                       a.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    if rc != OK:
        raise QflexGb300Error(rc, "permutation schedule check failed")
    return out


def multiply_skinny_noalloc(A: int, B: int, Cp: int, m: int, n: int, k: int, stream: int = 0) -> None:
    """C[m,n] = A[m,k] * B[k,n] for at most 64 outputs, without allocating
    device memory (see qflex_gb300_multiply_skinny_noalloc). Pointers are
    CUDA device addresses; `stream` a cudaStream_t handle (0: legacy)."""
    lib = load_library()
    err = C.create_string_buffer(512)
    rc = lib.qflex_gb300_multiply_skinny_noalloc(C.c_void_p(A), C.c_void_p(B), C.c_void_p(Cp), m, n, k,
                                                 C.c_void_p(stream or None), err, len(err))
    if rc != OK:
        raise QflexGb300Error(rc, err.value.decode())


def _b(s: Optional[str]) -> bytes:
    return (s or "").encode()


def _sizes(vals: Sequence[int]):
    arr = (C.c_size_t * max(len(vals), 1))(*vals)
    return arr


class Context:
    """One engine context: a CUDA device (or -1 for planning only), a stream,
    a planned HBM arena and the results of the last evaluation."""

    def __init__(self, device: int = 0, precision: int = FP32):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.qflex_gb300_create(device, precision, C.byref(h))
        self._h = h
        if rc != OK:
            msg = self._lib.qflex_gb300_last_error(h).decode() if h else "create failed"
            self._lib.qflex_gb300_destroy(h)
            self._h = None
            raise QflexGb300Error(rc, msg)
        self.device = device
        self.precision = precision

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.qflex_gb300_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != OK:
            raise QflexGb300Error(rc, self._lib.qflex_gb300_last_error(self._h).decode())

    def set_precision(self, precision) -> None:
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        self._check(self._lib.qflex_gb300_set_precision(self._h, precision))
        self.precision = precision

    def set_stream(self, stream: int) -> None:
        self._check(self._lib.qflex_gb300_set_stream(self._h, C.c_void_p(stream or None)))

    def evaluate(self, circuit: str, ordering: str, grid: str, initial_state: str = "",
                 final_state: str = "", memory_limit: float = 0) -> List[Tuple[str, complex]]:
        self._check(self._lib.qflex_gb300_evaluate(
            self._h, _b(circuit), _b(ordering), _b(grid), _b(initial_state), _b(final_state),
            float(memory_limit)))
        return self.results()

    def evaluate_many(self, circuit: str, ordering: str, grid: str, initial_state: str,
                      final_states: Sequence[str], memory_limit: float = 0) -> List[Tuple[str, complex]]:
        arr = (C.c_char_p * max(len(final_states), 1))(*[_b(f) for f in final_states])
        self._check(self._lib.qflex_gb300_evaluate_many(
            self._h, _b(circuit), _b(ordering), _b(grid), _b(initial_state), arr,
            len(final_states), float(memory_limit)))
        return self.results()

    def results(self) -> List[Tuple[str, complex]]:
        n = self._lib.qflex_gb300_result_count(self._h)
        out = []
        re, im = C.c_double(), C.c_double()
        for i in range(n):
            s = self._lib.qflex_gb300_result_state(self._h, i).decode()
            self._check(self._lib.qflex_gb300_result_amplitude(self._h, i, C.byref(re), C.byref(im)))
            out.append((s, complex(re.value, im.value)))
        return out

    def initial_state(self) -> str:
        return self._lib.qflex_gb300_result_initial_state(self._h).decode()

    def final_state(self, which: int = 0) -> str:
        r = self._lib.qflex_gb300_result_final_state(self._h, which)
        return r.decode() if r is not None else ""

    def stats(self) -> dict:
        s = Stats()
        self._check(self._lib.qflex_gb300_last_stats(self._h, C.byref(s)))
        return s.as_dict()

    def shapes(self) -> List[Tuple[int, int, int, int]]:
        n = self._lib.qflex_gb300_last_shapes(self._h, None, 0)
        buf = (C.c_size_t * (4 * max(n, 1)))()
        self._lib.qflex_gb300_last_shapes(self._h, buf, n)
        return [tuple(buf[4 * i:4 * i + 4]) for i in range(n)]

    def gemms(self) -> List[Tuple[int, int, int]]:
        n = self._lib.qflex_gb300_last_gemms(self._h, None, 0)
        buf = (C.c_size_t * (3 * max(n, 1)))()
        self._lib.qflex_gb300_last_gemms(self._h, buf, n)
        return [tuple(buf[3 * i:3 * i + 3]) for i in range(n)]

    def set_profiling(self, on: bool) -> None:
        self._check(self._lib.qflex_gb300_set_profiling(self._h, 1 if on else 0))

    def set_option(self, name: str, value: float) -> None:
        """Tuning option: tc_chunk, tc_pair, graphs or max_batch."""
        self._check(self._lib.qflex_gb300_set_option(self._h, name.encode(), float(value)))

    def get_option(self, name: str) -> float:
        v = C.c_double()
        rc = self._lib.qflex_gb300_get_option(self._h, name.encode(), C.byref(v))
        if rc != 0:
            raise QflexGb300Error(rc, f"unknown option {name!r}")
        return v.value

    def set_tc_variant(self, m: int, n: int, k: int, variant: int) -> None:
        """Tensor-core kernel for products of shape (m, n, k): 0 single CTA,
        1 CTA pair, -1 no override."""
        self._check(self._lib.qflex_gb300_set_tc_variant(self._h, m, n, k, int(variant)))

    def ops(self):
        """Device ops of the last plan as a (n_ops, 8) numpy array: kind, m,
        n, k, flop, bytes, batch, milliseconds (-1 unless profiled)."""
        import numpy as np
        n = self._lib.qflex_gb300_last_ops(self._h, None, 0)
        buf = (C.c_double * (8 * max(n, 1)))()
        self._lib.qflex_gb300_last_ops(self._h, buf, n)
        return np.frombuffer(buf, dtype=np.float64)[:8 * n].reshape(n, 8).copy()

    # ---- tensor-level device operations (pointers are CUDA addresses) ----
    def permute(self, src: int, dst: int, dims: Sequence[int], new_order: Sequence[int],
                batch: int = 1, batch_stride: int = 0) -> None:
        self._check(self._lib.qflex_gb300_permute(
            self._h, C.c_void_p(src), C.c_void_p(dst), len(dims), _sizes(dims), _sizes(new_order),
            batch, batch_stride))

    def reorder(self, data: int, scratch: int, dims: Sequence[int], new_order: Sequence[int]) -> None:
        self._check(self._lib.qflex_gb300_reorder(
            self._h, C.c_void_p(data), C.c_void_p(scratch), len(dims), _sizes(dims),
            _sizes(new_order)))

    def multiply(self, A: int, B: int, Cp: int, m: int, n: int, k: int, batch: int = 1,
                 batch_stride: int = 0) -> None:
        self._check(self._lib.qflex_gb300_multiply(
            self._h, C.c_void_p(A), C.c_void_p(B), C.c_void_p(Cp), m, n, k, batch, batch_stride))

    def synchronize(self) -> None:
        self._check(self._lib.qflex_gb300_synchronize(self._h))
