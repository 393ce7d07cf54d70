"""Python side of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs use
this module, to check results and to time the CPU baseline: nothing in ``perceval_gb300``
imports it.

Two layers:
* ``liboracle.so`` (``pcvl_oracle.c``): FP64 restatements of the reference's
  permanent, SLOS and Clifford & Clifford paths, multi-threaded with OpenMP;
* pure numpy/Python brute force (``perm_brute``, ``slos_brute``) for tiny cases,
  used to pin the C oracle itself.
"""
from __future__ import annotations

import ctypes
import itertools
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    """Compile ``liboracle.so`` with the committed Makefile (gcc, OpenMP)."""
    src = HERE / "pcvl_oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        res = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        vp, i32, i64, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64
        L.oracle_fock_count.restype = u64
        L.oracle_fock_count.argtypes = [i32, i32]
        L.oracle_fock_rank.restype = u64
        L.oracle_fock_rank.argtypes = [i32, vp]
        L.oracle_fock_unrank.argtypes = [i32, i32, u64, vp]
        L.oracle_perm_glynn.argtypes = [i32, vp, vp]
        L.oracle_perm_ryser.argtypes = [i32, vp, vp]
        L.oracle_perm_batch.argtypes = [vp, vp, vp, i32, i32, vp]
        L.oracle_perm_batch_fast.argtypes = [vp, vp, vp, i32, vp]
        L.oracle_cc2017_fast.argtypes = [vp, i32, vp, i64, u64, u64, vp]
        L.oracle_slos_order.restype = i32
        L.oracle_slos_order.argtypes = [i32, vp, vp]
        L.oracle_slos_coefs.restype = i32
        L.oracle_slos_coefs.argtypes = [i32, vp, vp, vp]
        L.oracle_slos.restype = i32
        L.oracle_slos.argtypes = [i32, vp, vp, vp, vp]
        L.oracle_slos_grad.restype = i32
        L.oracle_slos_grad.argtypes = [i32, vp, vp, vp, vp]
        L.oracle_slos_fast.restype = i32
        L.oracle_slos_fast.argtypes = [i32, vp, vp, vp, vp]
        L.oracle_slos_grad_fast.restype = i32
        L.oracle_slos_grad_fast.argtypes = [i32, vp, vp, vp, vp]
        L.oracle_philox.argtypes = [ctypes.c_uint32] * 6 + [vp]
        L.oracle_cc2017.argtypes = [vp, i32, vp, i64, u64, u64, vp]
        L.oracle_glynn_term.argtypes = [i32, vp, vp, vp]
        L.oracle_gurvits.argtypes = [i32, vp, i64, u64, u64, vp]
        L.oracle_gurvits_batch_fast.argtypes = [vp, vp, vp, i32, i64, u64, vp, vp]
        L.oracle_num_threads.restype = i32
        L.oracle_set_threads.argtypes = [i32]
        _lib = L
    return _lib


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_threads(t: int):
    lib().oracle_set_threads(int(t))


def perm(a, method: str = "glynn") -> complex:
    a = _c128(a)
    n = a.shape[0]
    out = np.zeros(2)
    fn = lib().oracle_perm_glynn if method == "glynn" else lib().oracle_perm_ryser
    fn(n, a.ctypes.data, out.ctypes.data)
    return complex(out[0], out[1])


def perm_batch(mats: np.ndarray, offsets, sizes, method: str = "glynn") -> np.ndarray:
    mats = _c128(mats)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = _i32(sizes)
    out = np.zeros(len(sizes), dtype=np.complex128)
    lib().oracle_perm_batch(mats.ctypes.data, offsets.ctypes.data, sizes.ctypes.data, len(sizes),
                            1 if method == "ryser" else 0, out.ctypes.data)
    return out


def perm_batch_fast(mats: np.ndarray, offsets, sizes) -> np.ndarray:
    """Glynn permanents of a packed batch by the host-tuned path (the CPU baseline):
    sixteen consecutive Gray-code steps at once in vector lanes, one OpenMP task per
    2^12-step chunk of every matrix, chunks added in order with compensation (FP64)."""
    mats = _c128(mats)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    sizes = _i32(sizes)
    out = np.zeros(len(sizes), dtype=np.complex128)
    lib().oracle_perm_batch_fast(mats.ctypes.data, offsets.ctypes.data, sizes.ctypes.data, len(sizes),
                                 out.ctypes.data)
    return out


def cc2017_fast(U, input_state, count: int, seed: int, first: int = 0) -> np.ndarray:
    """Clifford & Clifford samples drawn in parallel over samples, the k sub-permanents of
    a step from one Glynn sum over sixteen Gray-code steps at once in vector lanes (the CPU
    baseline; same Philox stream and draws as cc2017)."""
    U = _c128(U)
    m = U.shape[0]
    inp = _i32(input_state)
    out = np.zeros((count, m), dtype=np.int32)
    lib().oracle_cc2017_fast(U.ctypes.data, m, inp.ctypes.data, int(count), int(seed) & (2**64 - 1), int(first),
                             out.ctypes.data)
    return out


def fock_rank(state) -> int:
    s = _i32(state)
    return int(lib().oracle_fock_rank(len(s), s.ctypes.data))


def fock_unrank(m: int, n: int, rank: int) -> tuple:
    s = np.zeros(m, dtype=np.int32)
    lib().oracle_fock_unrank(m, n, rank, s.ctypes.data)
    return tuple(int(v) for v in s)


def slos_order(input_state) -> list[int]:
    s = _i32(input_state)
    out = np.zeros(int(s.sum()) + 1, dtype=np.int32)
    k = lib().oracle_slos_order(len(s), s.ctypes.data, out.ctypes.data)
    return [int(v) for v in out[:k]]


def slos_coefs(U, input_state) -> np.ndarray:
    U = _c128(U)
    s = _i32(input_state)
    m, n = len(s), int(s.sum())
    out = np.zeros(math.comb(m + n - 1, n), dtype=np.complex128)
    if lib().oracle_slos_coefs(m, s.ctypes.data, U.ctypes.data, out.ctypes.data):
        raise MemoryError("oracle SLOS allocation failed")
    return out


def slos(U, input_state) -> tuple[np.ndarray, np.ndarray]:
    """(probabilities, amplitudes) over all outputs in descending-lex order."""
    U = _c128(U)
    s = _i32(input_state)
    m, n = len(s), int(s.sum())
    N = math.comb(m + n - 1, n)
    probs = np.zeros(N)
    amps = np.zeros(N, dtype=np.complex128)
    if lib().oracle_slos(m, s.ctypes.data, U.ctypes.data, probs.ctypes.data, amps.ctypes.data):
        raise MemoryError("oracle SLOS allocation failed")
    return probs, amps


def slos_grad(U, input_state, w) -> np.ndarray:
    """dL/dU (dL/dRe + i dL/dIm) of L = sum_r w_r p_r."""
    U = _c128(U)
    s = _i32(input_state)
    w = np.ascontiguousarray(w, dtype=np.float64)
    g = np.zeros_like(U)
    lib().oracle_slos_grad(len(s), s.ctypes.data, U.ctypes.data, w.ctypes.data, g.ctypes.data)
    return g


def slos_fast(U, input_state) -> tuple[np.ndarray, np.ndarray]:
    """(probabilities, amplitudes) like slos, by the host-tuned path (the CPU baseline):
    layers parallel over contiguous rank ranges, parent ranks from one O(m) pass per state."""
    U = _c128(U)
    s = _i32(input_state)
    m, n = len(s), int(s.sum())
    N = math.comb(m + n - 1, n)
    probs = np.zeros(N)
    amps = np.zeros(N, dtype=np.complex128)
    if lib().oracle_slos_fast(m, s.ctypes.data, U.ctypes.data, probs.ctypes.data, amps.ctypes.data):
        raise ValueError("oracle SLOS: more than 63 photons")
    return probs, amps


def slos_grad_fast(U, input_state, w) -> np.ndarray:
    """dL/dU like slos_grad, by the host-tuned path (parallel reverse sweep)."""
    U = _c128(U)
    s = _i32(input_state)
    w = np.ascontiguousarray(w, dtype=np.float64)
    g = np.zeros_like(U)
    if lib().oracle_slos_grad_fast(len(s), s.ctypes.data, U.ctypes.data, w.ctypes.data, g.ctypes.data):
        raise ValueError("oracle SLOS: more than 63 photons")
    return g


def philox(counter, key) -> tuple:
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox(*[int(c) for c in counter], *[int(k) for k in key], out.ctypes.data)
    return tuple(int(v) for v in out)


def cc2017(U, input_state, count: int, seed: int, first: int = 0) -> np.ndarray:
    U = _c128(U)
    s = _i32(input_state)
    out = np.zeros((count, len(s)), dtype=np.int32)
    lib().oracle_cc2017(U.ctypes.data, len(s), s.ctypes.data, int(count), int(seed) & (2**64 - 1), int(first),
                        out.ctypes.data)
    return out


def glynn_term(a, x_bits: int) -> complex:
    """One Gurvits draw X(x) for the sign vector whose set bits are the -1 entries."""
    a = _c128(a)
    w = np.array([x_bits & 0xffffffff, (x_bits >> 32) & 0xffffffff], dtype=np.uint32)
    out = np.zeros(2)
    lib().oracle_glynn_term(a.shape[0], a.ctypes.data, w.ctypes.data, out.ctypes.data)
    return complex(out[0], out[1])


def gurvits(a, iterations: int, seed: int, first: int = 0) -> complex:
    """Mean of `iterations` draws with the GPU estimator's Philox stream (draw k has
    global index first + k)."""
    a = _c128(a)
    out = np.zeros(2)
    lib().oracle_gurvits(a.shape[0], a.ctypes.data, int(iterations), int(seed) & (2**64 - 1), int(first),
                         out.ctypes.data)
    return complex(out[0], out[1])


def gurvits_batch_fast(mats, iterations: int, seed: int, firsts) -> np.ndarray:
    """gurvits for each matrix of a list (matrix b's draws start at index firsts[b]) by the
    host-tuned path (the CPU baseline): OpenMP over (matrix, 256 draws) on all threads."""
    mats = [_c128(a) for a in mats]
    sizes = np.array([a.shape[0] for a in mats], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum([a.size for a in mats])[:-1]]).astype(np.int64)
    flat = np.ascontiguousarray(np.concatenate([a.reshape(-1) for a in mats]))
    firsts = np.ascontiguousarray(firsts, dtype=np.uint64)
    out = np.zeros(len(mats), dtype=np.complex128)
    lib().oracle_gurvits_batch_fast(flat.ctypes.data, offs.ctypes.data, sizes.ctypes.data, len(mats),
                                    int(iterations), int(seed) & (2**64 - 1), firsts.ctypes.data, out.ctypes.data)
    return out


# ---------------------------------------------------------------- brute force
def perm_brute(a) -> complex:
    """Permanent by the sum over all permutations (n <= 8)."""
    a = np.asarray(a, dtype=np.complex128)
    n = a.shape[0]
    tot = 0j
    for p in itertools.permutations(range(n)):
        v = 1 + 0j
        for i in range(n):
            v *= a[i, p[i]]
        tot += v
    return tot


def fock_states(m: int, n: int) -> list[tuple]:
    """All n-photon states on m modes, descending-lex order (recursive definition)."""
    if m == 1:
        return [(n,)]
    out = []
    for a in range(n, -1, -1):
        out.extend((a,) + t for t in fock_states(m - 1, n - a))
    return out


def submatrix(U, input_state, output_state) -> np.ndarray:
    """Rows repeat output modes, columns repeat input modes (perceval/backends/_naive.py:51-68)."""
    rows = [j for j, v in enumerate(output_state) for _ in range(v)]
    cols = [i for i, v in enumerate(input_state) for _ in range(v)]
    return np.asarray(U)[np.ix_(rows, cols)]


def amplitude_brute(U, input_state, output_state) -> complex:
    if sum(input_state) != sum(output_state):
        return 0j
    f = math.prod(math.factorial(v) for v in input_state) * math.prod(math.factorial(v) for v in output_state)
    return perm_brute(submatrix(U, input_state, output_state)) / math.sqrt(f)


def slos_brute(U, input_state) -> tuple[np.ndarray, np.ndarray]:
    """(probabilities, amplitudes) by one brute-force permanent per output."""
    m, n = len(input_state), sum(input_state)
    amps = np.array([amplitude_brute(U, input_state, s) for s in fock_states(m, n)])
    return np.abs(amps) ** 2, amps
