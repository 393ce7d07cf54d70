"""ctypes binding of ``libpcvl_gb300.so``: the only way the package reaches the GPU.

There is no CPU fallback: when the library is missing or CUDA is unavailable every
entry point raises ``RuntimeError``.  Tensors passed in must be CUDA tensors on the
current device, contiguous, of the documented dtype; outputs are written in place.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np
import torch

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libpcvl_gb300.so"
_lib = None

SYMBOLS = {
    "pcvl_version": (ctypes.c_char_p, []),
    "pcvl_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "pcvl_release_workspace": (ctypes.c_int, []),
    "pcvl_permanent_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                            ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pcvl_permanent_batch_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                    ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                                    ctypes.c_int32, ctypes.c_void_p]),
    "pcvl_permanent_estimate_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64,
                                                     ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p]),
    "pcvl_perm_set_tuning": (ctypes.c_int, [ctypes.c_int32] * 5),
    "pcvl_perm_get_tuning": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "pcvl_perm_plan_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "pcvl_perm_plan_execute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_perm_plan_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "pcvl_perm_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pcvl_slos_plan_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_void_p,
                                             ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "pcvl_slos_plan_create_multi": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                                   ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.c_int32]),
    "pcvl_slos_plan_create_masked": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                                     ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint32,
                                                     ctypes.c_int32, ctypes.c_int32]),
    "pcvl_slos_output_ranks": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_slos_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pcvl_fock_mask_ranks": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                             ctypes.POINTER(ctypes.c_int64)]),
    "pcvl_slap_output_count": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "pcvl_slap_probabilities": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "pcvl_slap_amplitudes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p]),
    "pcvl_slos_forward_shared": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_slos_output_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "pcvl_slos_plan_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "pcvl_slos_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_slos_probabilities": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_slos_forward_probabilities": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.c_void_p]),
    "pcvl_slos_amplitudes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_slos_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_cc2017_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "pcvl_cc2017_sample_multi": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_gemm_bf16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int32] * 7 +
                       [ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "pcvl_mlp_elementwise": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_colsum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "pcvl_softmax_xent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_bag_embed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_void_p]),
    "pcvl_bag_embed_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                               ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                 ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int32,
                                 ctypes.c_void_p, ctypes.c_void_p]),
    "pcvl_sample_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_void_p]),
}


def library_path() -> Path:
    return Path(os.environ.get("PCVL_GB300_LIB", _LIB_PATH))


def load(require_cuda: bool = True):
    """Load the library (once).  Raises RuntimeError if it or CUDA is unavailable."""
    global _lib
    if require_cuda and not torch.cuda.is_available():
        raise RuntimeError("perceval_gb300 needs a CUDA GPU: torch.cuda.is_available() is False")
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it with perceval_gb300._build.build()")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SYMBOLS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        if require_cuda:
            # launch shapes tuned earlier on this GPU and build, if a cached table exists
            try:
                from . import autotune
                autotune.load()
            except (OSError, ValueError, KeyError, RuntimeError):
                pass
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load(require_cuda=False).pcvl_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, what: str):
    if status != 0:
        raise RuntimeError(f"{what} failed (status {status}): {last_error()}")


# precision codes of the C ABI (PCVL_PREC_*)
PREC_FLOAT_FLOAT, PREC_FP32, PREC_FP64, PREC_FP64_DADD = 0, 1, 2, 3
_PREC_NAMES = {"fp64": PREC_FP64, "float64": PREC_FP64, "float-float": PREC_FLOAT_FLOAT,
               "ff": PREC_FLOAT_FLOAT, "fp32": PREC_FP32, "fp64-dadd": PREC_FP64_DADD}


def precision_code(precision) -> int:
    """ABI code of a precision given as a code or a name.  "fp64" (the default
    everywhere): FP64 precision, no step rounding more coarsely than an FP64 operation
    (permanents and the sampler take exact fixed-point sums and run part of their products
    in 64-bit block floating point on the integer pipes); "float-float": pairs of FP32
    numbers, about 48 significant bits, faster; "fp32": the sampler's FP32 mode;
    "fp64-dadd" (permanents): every row sum and product an FP64 operation."""
    if isinstance(precision, str):
        try:
            return _PREC_NAMES[precision.lower()]
        except KeyError:
            raise ValueError(f"unknown precision {precision!r}: use 'fp64' or 'float-float'") from None
    return int(precision)


def _stream_ptr(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _dev_tensor(t: torch.Tensor, dtype, name: str) -> torch.Tensor:
    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t


# ------------------------------------------------------------------ permanents
def permanent_batch(mats: torch.Tensor, offsets: np.ndarray, sizes: np.ndarray, out: torch.Tensor,
                    method: int = 0, stream=None, precision="fp64") -> torch.Tensor:
    """Permanents of packed square complex128 matrices (see pcvl_permanent_batch); FP64
    arithmetic unless ``precision="float-float"``."""
    lib = load()
    _dev_tensor(mats, torch.complex128, "mats")
    _dev_tensor(out, torch.complex128, "out")
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    count = int(sizes.shape[0])
    if offsets.shape[0] != count or out.numel() < count:
        raise ValueError("offsets, sizes and out must describe the same number of matrices")
    if count and int((offsets + sizes.astype(np.int64) ** 2).max()) > mats.numel():
        raise ValueError("a matrix extends beyond the end of mats")
    check(lib.pcvl_permanent_batch(mats.data_ptr(), offsets.ctypes.data, sizes.ctypes.data, count,
                                   out.data_ptr(), int(method), precision_code(precision), _stream_ptr(stream)),
          "pcvl_permanent_batch")
    return out


def permanent_batch_noalloc(mats: torch.Tensor, offsets: np.ndarray, sizes: np.ndarray, out: torch.Tensor,
                            method: int = 0, stream=None, precision="fp64") -> torch.Tensor:
    """Same as ``permanent_batch`` through the allocation-free entry point: the library
    allocates no device memory for the call (fixed per-call limits, see the header)."""
    lib = load()
    _dev_tensor(mats, torch.complex128, "mats")
    _dev_tensor(out, torch.complex128, "out")
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    count = int(sizes.shape[0])
    if offsets.shape[0] != count or out.numel() < count:
        raise ValueError("offsets, sizes and out must describe the same number of matrices")
    if count and int((offsets + sizes.astype(np.int64) ** 2).max()) > mats.numel():
        raise ValueError("a matrix extends beyond the end of mats")
    check(lib.pcvl_permanent_batch_noalloc(mats.data_ptr(), offsets.ctypes.data, sizes.ctypes.data, count,
                                           out.data_ptr(), int(method), precision_code(precision),
                                           _stream_ptr(stream)),
          "pcvl_permanent_batch_noalloc")
    return out


def permanent_estimate_batch(mats: torch.Tensor, offsets: np.ndarray, sizes: np.ndarray, out: torch.Tensor,
                             err: torch.Tensor, iterations: int, seed: int, first_sample: int = 0,
                             stream=None) -> tuple[torch.Tensor, torch.Tensor]:
    """Gurvits estimates of packed permanents and their 99% error bounds
    (see pcvl_permanent_estimate_batch)."""
    lib = load()
    _dev_tensor(mats, torch.complex128, "mats")
    _dev_tensor(out, torch.complex128, "out")
    _dev_tensor(err, torch.float64, "err")
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    count = int(sizes.shape[0])
    if offsets.shape[0] != count or out.numel() < count or err.numel() < count:
        raise ValueError("offsets, sizes, out and err must describe the same number of matrices")
    if count and int((offsets + sizes.astype(np.int64) ** 2).max()) > mats.numel():
        raise ValueError("a matrix extends beyond the end of mats")
    check(lib.pcvl_permanent_estimate_batch(mats.data_ptr(), offsets.ctypes.data, sizes.ctypes.data, count,
                                            int(iterations), int(seed) & (2**64 - 1), int(first_sample),
                                            out.data_ptr(), err.data_ptr(), _stream_ptr(stream)),
          "pcvl_permanent_estimate_batch")
    return out, err


def set_perm_tuning(method: int, n: int, lo_bits: int = -1, ctas_per_sm: int = 0, precision="fp64"):
    """Launch shape of the size-n permanent bin of one arithmetic (-1 / 0: built-in
    choice).  Host-only."""
    check(load(require_cuda=False).pcvl_perm_set_tuning(int(method), precision_code(precision), int(n),
                                                        int(lo_bits), int(ctas_per_sm)), "pcvl_perm_set_tuning")


def get_perm_tuning(method: int, n: int, precision="fp64") -> tuple[int, int]:
    """Effective (lo_bits, ctas_per_sm) of the size-n permanent bin of one arithmetic."""
    lo, ct = ctypes.c_int32(), ctypes.c_int32()
    check(load(require_cuda=False).pcvl_perm_get_tuning(int(method), precision_code(precision), int(n),
                                                        ctypes.byref(lo), ctypes.byref(ct)), "pcvl_perm_get_tuning")
    return lo.value, ct.value


class PermPlan:
    """Owner of a ``pcvl_perm_plan``: permanents of a fixed batch shape, executed as one
    CUDA graph per call (see pcvl_perm_plan_create)."""

    def __init__(self, offsets: np.ndarray, sizes: np.ndarray, method: int = 0, precision="fp64"):
        self._lib = load()
        self.precision = precision_code(precision)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.count = int(self.sizes.shape[0])
        if self.offsets.shape[0] != self.count or self.count < 1:
            raise ValueError("offsets and sizes must describe the same (non-zero) number of matrices")
        self.span = int((self.offsets + self.sizes.astype(np.int64) ** 2).max())
        h = ctypes.c_void_p()
        check(self._lib.pcvl_perm_plan_create(ctypes.byref(h), self.offsets.ctypes.data, self.sizes.ctypes.data,
                                              self.count, int(method), self.precision), "pcvl_perm_plan_create")
        self._h = h

    @property
    def nbytes(self) -> int:
        v = ctypes.c_int64()
        check(self._lib.pcvl_perm_plan_bytes(self._h, ctypes.byref(v)), "pcvl_perm_plan_bytes")
        return v.value

    def __call__(self, mats: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        _dev_tensor(mats, torch.complex128, "mats")
        if mats.numel() < self.span:
            raise ValueError("a matrix extends beyond the end of mats")
        if out is None:
            out = torch.empty(self.count, dtype=torch.complex128, device=mats.device)
        _dev_tensor(out, torch.complex128, "out")
        if out.numel() < self.count:
            raise ValueError("out is smaller than the plan's matrix count")
        check(self._lib.pcvl_perm_plan_execute(self._h, mats.data_ptr(), out.data_ptr(), _stream_ptr(stream)),
              "pcvl_perm_plan_execute")
        return out

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pcvl_perm_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ SLOS
class SlosPlan:
    """Owner of a ``pcvl_slos_plan``: fixed (m, input state(s), batch).

    ``input_state`` is one state shared by the ``batch`` entries, or a (batch x m)
    array of per-entry states with one photon count (``pcvl_slos_plan_create_multi``).
    ``mask`` (an ``FSMask``) restricts every layer to the states the mask can still
    accept (``pcvl_slos_plan_create_masked``): the outputs are then the accepted states,
    ``output_ranks()`` gives their ranks in the full n-photon space.  ``precision``:
    "fp64" (native FP64, the reference's arithmetic) or "float-float".
    """

    def __init__(self, m: int, input_state, batch: int = 1, keep_layers: bool = False, mask=None,
                 precision="fp64"):
        self._lib = load()
        self.precision = precision_code(precision)
        prec = self.precision
        inp = np.ascontiguousarray(input_state, dtype=np.int32)
        h = ctypes.c_void_p()
        self.masked = mask is not None
        if mask is not None:
            if inp.ndim == 1:
                if inp.shape != (m,):
                    raise ValueError("input_state must have m entries")
                self.input_state = tuple(int(v) for v in inp)
                inp = np.ascontiguousarray(np.tile(inp, (int(batch), 1)))
            elif inp.ndim != 2 or inp.shape[1] != m or inp.shape[0] < 1:
                raise ValueError("input states must form a (batch x m) array")
            else:
                self.input_state = [tuple(int(v) for v in row) for row in inp]
            batch = inp.shape[0]
            digits, at_least, mask_n = mask.device_spec()
            if digits.shape[1] != m:
                raise ValueError("mask and input state lengths differ")
            check(self._lib.pcvl_slos_plan_create_masked(ctypes.byref(h), int(m), inp.ctypes.data, int(batch),
                                                         1 if keep_layers else 0, int(digits.shape[0]),
                                                         digits.ctypes.data, int(at_least), int(mask_n), prec),
                  "pcvl_slos_plan_create_masked")
        elif inp.ndim == 2:
            if inp.shape[1] != m or inp.shape[0] < 1:
                raise ValueError("input states must form a (batch x m) array")
            batch = inp.shape[0]
            check(self._lib.pcvl_slos_plan_create_multi(ctypes.byref(h), int(m), inp.ctypes.data, int(batch),
                                                        1 if keep_layers else 0, prec),
                  "pcvl_slos_plan_create_multi")
            self.input_state = [tuple(int(v) for v in row) for row in inp]
        else:
            if inp.shape != (m,):
                raise ValueError("input_state must have m entries")
            check(self._lib.pcvl_slos_plan_create(ctypes.byref(h), int(m), inp.ctypes.data, int(batch),
                                                  1 if keep_layers else 0, prec), "pcvl_slos_plan_create")
            self.input_state = tuple(int(v) for v in inp)
        self._h = h
        self.m, self.batch, self.keep_layers = m, batch, keep_layers
        c = ctypes.c_int64()
        check(self._lib.pcvl_slos_output_count(h, ctypes.byref(c)), "pcvl_slos_output_count")
        self.count = int(c.value)

    def output_ranks(self) -> np.ndarray:
        """Ranks of the plan's outputs in the full n-photon space (descending
        lexicographic order), ascending; 0 .. count-1 without a mask."""
        out = np.empty(self.count, dtype=np.uint64)
        check(self._lib.pcvl_slos_output_ranks(self._h, out.ctypes.data), "pcvl_slos_output_ranks")
        return out

    @property
    def device_bytes(self) -> int:
        b = ctypes.c_int64()
        check(self._lib.pcvl_slos_plan_bytes(self._h, ctypes.byref(b)), "pcvl_slos_plan_bytes")
        return int(b.value)

    def forward(self, u: torch.Tensor, stream=None):
        """Propagate: ``u`` holds batch x m x m unitaries, or one m x m unitary shared by
        every entry."""
        _dev_tensor(u, torch.complex128, "u")
        if u.numel() == self.batch * self.m * self.m:
            check(self._lib.pcvl_slos_forward(self._h, u.data_ptr(), _stream_ptr(stream)), "pcvl_slos_forward")
        elif u.numel() == self.m * self.m:
            check(self._lib.pcvl_slos_forward_shared(self._h, u.data_ptr(), _stream_ptr(stream)),
                  "pcvl_slos_forward_shared")
        else:
            raise ValueError("u must hold batch x m x m or m x m elements")

    def forward_probabilities(self, u: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """``forward`` then ``probabilities`` in one call; with one circuit the last layer
        writes the probabilities directly (its coefficients are not kept: ``amplitudes``
        and ``backward`` need a ``forward`` first).  ``u``: batch x m x m unitaries."""
        _dev_tensor(u, torch.complex128, "u")
        if u.numel() != self.batch * self.m * self.m:
            raise ValueError("u must hold batch x m x m elements")
        if out is None:
            out = torch.empty(self.count * self.batch, dtype=torch.float64, device="cuda")
        if self.count == 0:
            return out
        _dev_tensor(out, torch.float64, "out")
        check(self._lib.pcvl_slos_forward_probabilities(self._h, u.data_ptr(), out.data_ptr(), _stream_ptr(stream)),
              "pcvl_slos_forward_probabilities")
        return out

    def probabilities(self, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        if out is None:
            out = torch.empty(self.count * self.batch, dtype=torch.float64, device="cuda")
        if self.count == 0:  # a mask that accepts no output
            return out
        _dev_tensor(out, torch.float64, "out")
        check(self._lib.pcvl_slos_probabilities(self._h, out.data_ptr(), _stream_ptr(stream)),
              "pcvl_slos_probabilities")
        return out

    def amplitudes(self, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        if out is None:
            out = torch.empty(self.count * self.batch, dtype=torch.complex128, device="cuda")
        if self.count == 0:
            return out
        _dev_tensor(out, torch.complex128, "out")
        check(self._lib.pcvl_slos_amplitudes(self._h, out.data_ptr(), _stream_ptr(stream)),
              "pcvl_slos_amplitudes")
        return out

    def backward(self, weights: torch.Tensor, grad_u: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        _dev_tensor(weights, torch.float64, "weights")
        if weights.numel() != self.count * self.batch:
            raise ValueError("weights must hold count x batch elements (state-major)")
        if grad_u is None:
            grad_u = torch.empty(self.batch * self.m * self.m, dtype=torch.complex128, device="cuda")
        if self.count == 0:  # L is identically zero
            return grad_u.zero_()
        _dev_tensor(grad_u, torch.complex128, "grad_u")
        check(self._lib.pcvl_slos_backward(self._h, weights.data_ptr(), grad_u.data_ptr(), _stream_ptr(stream)),
              "pcvl_slos_backward")
        return grad_u

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pcvl_slos_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ SLAP
def slap_output_count(m: int, input_state) -> int:
    lib = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    if inp.shape != (m,):
        raise ValueError("input_state must have m entries")
    c = ctypes.c_int64()
    check(lib.pcvl_slap_output_count(int(m), inp.ctypes.data, ctypes.byref(c)), "pcvl_slap_output_count")
    return int(c.value)


def slap_all(u: torch.Tensor, input_state, amplitudes: bool = False, out: torch.Tensor | None = None,
             stream=None) -> torch.Tensor:
    """Every output probability (float64) or amplitude (complex128) of one input state,
    in descending-lexicographic order, by the SLAP walk (``pcvl_slap_probabilities`` /
    ``pcvl_slap_amplitudes``)."""
    lib = load()
    _dev_tensor(u, torch.complex128, "u")
    m = u.shape[-1]
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    count = slap_output_count(m, inp)
    dt = torch.complex128 if amplitudes else torch.float64
    if out is None:
        out = torch.empty(count, dtype=dt, device="cuda")
    _dev_tensor(out, dt, "out")
    if out.numel() < count:
        raise ValueError("out holds fewer than the output count")
    fn = lib.pcvl_slap_amplitudes if amplitudes else lib.pcvl_slap_probabilities
    check(fn(u.data_ptr(), int(m), inp.ctypes.data, out.data_ptr(), _stream_ptr(stream)),
          "pcvl_slap_amplitudes" if amplitudes else "pcvl_slap_probabilities")
    return out


def fock_mask_ranks(m: int, n: int, mask) -> torch.Tensor:
    """Ranks (int64 CUDA tensor, ascending) of the n-photon states on m modes that the
    ``FSMask`` keeps (``pcvl_fock_mask_ranks``)."""
    lib = load()
    digits, _, mask_n = mask.device_spec()
    if digits.shape[1] != m:
        raise ValueError("mask and state lengths differ")
    atl = np.zeros(m, dtype=np.uint8)
    for i in mask.at_least_modes:
        if 0 <= i < m:
            atl[i] = 1
    kept = ctypes.c_int64()
    args = (int(m), int(n), int(digits.shape[0]), digits.ctypes.data, atl.ctypes.data, int(mask_n))
    check(lib.pcvl_fock_mask_ranks(*args, None, 0, ctypes.byref(kept)), "pcvl_fock_mask_ranks")
    out = torch.empty(max(kept.value, 1), dtype=torch.int64, device="cuda")
    if kept.value:
        check(lib.pcvl_fock_mask_ranks(*args, out.data_ptr(), int(kept.value), ctypes.byref(kept)),
              "pcvl_fock_mask_ranks")
    return out[:kept.value]


# ------------------------------------------------------------------ sampling
def cc2017_sample(u: torch.Tensor, input_state, count: int, seed: int, first_sample: int = 0,
                  precision: int = 0, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """Exact boson samples (Clifford & Clifford 2018); returns int32 counts (count, m)."""
    lib = load()
    _dev_tensor(u, torch.complex128, "u")
    m = u.shape[-1]
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    if inp.shape != (m,):
        raise ValueError("input_state must have m entries")
    if out is None:
        out = torch.empty((count, m), dtype=torch.int32, device="cuda")
    if count == 0:
        return out
    _dev_tensor(out, torch.int32, "out")
    check(lib.pcvl_cc2017_sample(u.data_ptr(), int(m), inp.ctypes.data, int(count), int(seed) & (2**64 - 1),
                                 int(first_sample), int(precision), out.data_ptr(), _stream_ptr(stream)),
          "pcvl_cc2017_sample")
    return out


def cc2017_sample_multi(u: torch.Tensor, input_states, counts, seed: int, first_sample: int = 0,
                        precision: int = 0, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """Samples of several input states of one photon count in one wavefront
    (``pcvl_cc2017_sample_multi``): int32 (sum(counts), m), state b's samples after those of
    the states before it."""
    lib = load()
    _dev_tensor(u, torch.complex128, "u")
    m = u.shape[-1]
    states = np.ascontiguousarray(input_states, dtype=np.int32)
    cnt = np.ascontiguousarray(counts, dtype=np.int64)
    if states.ndim != 2 or states.shape[1] != m or states.shape[0] != cnt.shape[0] or states.shape[0] < 1:
        raise ValueError("input_states must be (nstates x m) with one count per state")
    total = int(cnt.sum())
    if out is None:
        out = torch.empty((total, m), dtype=torch.int32, device="cuda")
    if total == 0:
        return out
    _dev_tensor(out, torch.int32, "out")
    check(lib.pcvl_cc2017_sample_multi(u.data_ptr(), int(m), int(states.shape[0]), states.ctypes.data,
                                       cnt.ctypes.data, int(seed) & (2**64 - 1), int(first_sample), int(precision),
                                       out.data_ptr(), _stream_ptr(stream)), "pcvl_cc2017_sample_multi")
    return out


# ------------------------------------------------------------------ learned proposal kernels
def _ptr(t):
    return 0 if t is None else t.data_ptr()


def gemm_bf16(A, B, M, N, K, lda, ldb, transA=0, transB=0, alpha=1.0, beta=0.0, bias=None, epilogue=0, C=None,
              Cb=None, Cpre=None, ldc=None, stream=None):
    """BF16 tensor-core GEMM with FP32 accumulation (see pcvl_gemm_bf16)."""
    lib = load()
    check(lib.pcvl_gemm_bf16(_ptr(A), _ptr(B), M, N, K, lda, ldb, transA, transB, alpha, beta, _ptr(bias),
                             epilogue, _ptr(C), _ptr(Cb), _ptr(Cpre), N if ldc is None else ldc,
                             _stream_ptr(stream)), "pcvl_gemm_bf16")


def gelu_backward(dy, pre, out=None, outb=None, stream=None):
    lib = load()
    check(lib.pcvl_mlp_elementwise(0, _ptr(dy), _ptr(pre), dy.numel(), _ptr(out), _ptr(outb), _stream_ptr(stream)),
          "pcvl_mlp_elementwise")


def to_bf16(x, out, stream=None):
    lib = load()
    check(lib.pcvl_mlp_elementwise(1, _ptr(x), 0, x.numel(), _ptr(out), 0, _stream_ptr(stream)), "pcvl_mlp_elementwise")


def colsum(x, M, N, ld, out, stream=None):
    check(load().pcvl_colsum(_ptr(x), M, N, ld, _ptr(out), _stream_ptr(stream)), "pcvl_colsum")


def softmax_xent(logits, R, N, target=None, scale=1.0, logp_target=None, grad=None, gradb=None, all_logp=None,
                 stream=None):
    check(load().pcvl_softmax_xent(_ptr(logits), R, N, _ptr(target), scale, _ptr(logp_target), _ptr(grad),
                                   _ptr(gradb), _ptr(all_logp), _stream_ptr(stream)), "pcvl_softmax_xent")


def bag_embed(seq, S, n, step, mode_emb, pos_emb, D, h, stream=None):
    check(load().pcvl_bag_embed(_ptr(seq), S, n, step, _ptr(mode_emb), _ptr(pos_emb), D, _ptr(h),
                                _stream_ptr(stream)), "pcvl_bag_embed")


def bag_embed_backward(seq, S, n, dh, D, dmode, dpos, stream=None):
    check(load().pcvl_bag_embed_backward(_ptr(seq), S, n, _ptr(dh), D, _ptr(dmode), _ptr(dpos), _stream_ptr(stream)),
          "pcvl_bag_embed_backward")


def adam(w, g, m1, m2, lr, b1, b2, eps, step, wb=None, stream=None):
    check(load().pcvl_adam(_ptr(w), _ptr(g), _ptr(m1), _ptr(m2), w.numel(), lr, b1, b2, eps, step, _ptr(wb),
                           _stream_ptr(stream)), "pcvl_adam")


def sample_step(logits, S, N, step, seed, chain0, seq, n, logq, stream=None):
    check(load().pcvl_sample_step(_ptr(logits), S, N, step, int(seed) & (2**64 - 1), int(chain0), _ptr(seq), n,
                                  _ptr(logq), _stream_ptr(stream)), "pcvl_sample_step")
