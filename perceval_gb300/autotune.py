"""Autotuner for the launch shape of the permanent kernels.

The size-n bin kernel splits the 2^F sign patterns of Glynn's formula (F = n - 1; Ryser:
the 2^n subsets, F = n) into lo bits, which every thread enumerates from a shared-memory
table of row-sum parts, and hi bits spread over threads and CTAs; the target number of
CTAs per SM over a bin sets how many hi patterns each thread takes.  Both trade table
size and occupancy against per-pattern work, and the best pair depends on n and on the
GPU.  For every size the tuner times each candidate pair on a synthetic batch of Haar
submatrices with CUDA events (best of ``reps`` runs after one warm-up), installs the
fastest through ``pcvl_perm_set_tuning`` and records the table.  Tables are cached as
JSON keyed by device name, SM count and library version; ``load`` ignores a table made
on another device or build.

Each arithmetic (FP64, float-float) has its own table: their kernels differ in register
and shared-memory footprint.  Results do not depend on the tuning beyond rounding: every
candidate computes the same sign-vector sum, only split differently (the tuner checks this
on each candidate).
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np
import torch

from . import _native

_KMAX_SMEM = 227 * 1024
_CTAS = (4, 8, 16, 32)


def default_cache_path() -> Path:
    env = os.environ.get("PCVL_GB300_TUNING")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent / "lib" / "tuning.json"


def device_key() -> dict:
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    lib = _native.load()
    return {"device": props.name, "sms": int(props.multi_processor_count),
            "library": lib.pcvl_version().decode()}


def glynn_flops(n: int) -> float:
    return 2.0 ** (n - 1) * (8 * n - 4)


def candidates(n: int, method: int = 0) -> list[tuple[int, int]]:
    """(lo_bits, ctas_per_sm) pairs tried for size n: lo bits around the built-in choice
    whose shared-memory table fits, times the CTA targets."""
    F = n if method else n - 1
    base = min(7, max(0, F - 7))
    out = []
    for lo in range(max(0, base - 2), min(F, base + 2) + 1):
        if (n * n + (1 << lo) * n) * 16 > _KMAX_SMEM:
            continue
        for c in _CTAS:
            out.append((lo, c))
    return out


def _batch(n: int, count: int, seed: int):
    from .utils.matrix import random_unitary
    U = random_unitary(max(64, 2 * n), seed=seed)
    rng = np.random.default_rng(seed)
    mats = np.empty((count, n, n), dtype=np.complex128)
    for i in range(count):
        r = rng.choice(U.shape[0], n, replace=False)
        c = rng.choice(U.shape[0], n, replace=False)
        mats[i] = U[np.ix_(r, c)]
    offsets = np.arange(count, dtype=np.int64) * n * n
    sizes = np.full(count, n, dtype=np.int32)
    return torch.from_numpy(mats.reshape(-1)).cuda(), offsets, sizes


def _time_ms(fn, reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    best = math.inf
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return best


def tune_permanents(sizes=range(8, 27), method: int = 0, target_ms: float = 20.0, reps: int = 3,
                    seed: int = 0, rate_flops: float | None = None, log=None, precision="fp64") -> dict:
    """Tunes every size in ``sizes`` for one arithmetic and installs the winners; returns
    the table {"key": device_key(), "method": method, "precision": name, "entries": {n: {...}}}."""
    code = _native.precision_code(precision)
    name = _prec_name(code)
    if rate_flops is None:  # work per candidate run: about target_ms at the expected rate
        rate_flops = 3.5e12 if code == _native.PREC_FLOAT_FLOAT else 0.7e12
    entries = {}
    for n in sizes:
        n = int(n)
        count = int(min(8192, max(1, math.ceil(target_ms * 1e-3 * rate_flops / glynn_flops(n)))))
        mats, offsets, sizes_a = _batch(n, count, seed + n)
        out = torch.empty(count, dtype=torch.complex128, device=mats.device)

        def run():
            _native.permanent_batch(mats, offsets, sizes_a, out, method, precision=code)

        _native.set_perm_tuning(method, n, precision=code)  # built-in shape first: reference values and time
        t_default = _time_ms(run, reps)
        ref = out.clone()
        best = (t_default, -1, 0)
        tol = 1e-8 if method == 0 else 1e-4  # Ryser's cancellation leaves more rounding
        for lo, c in candidates(n, method):
            _native.set_perm_tuning(method, n, lo, c, precision=code)
            t = _time_ms(run, reps)
            rel = float(((out - ref).abs() / ref.abs().clamp_min(1e-300)).max())
            if rel > tol:
                raise RuntimeError(f"tuning n={n} lo={lo} ctas={c} changed results by {rel:.2e}")
            if t < best[0]:
                best = (t, lo, c)
        t, lo, c = best
        _native.set_perm_tuning(method, n, lo, c, precision=code)
        eff_lo, eff_c = _native.get_perm_tuning(method, n, precision=code)
        entries[str(n)] = {"lo_bits": eff_lo, "ctas_per_sm": eff_c, "ms": t, "default_ms": t_default,
                           "matrices": count}
        if log:
            log(f"{name} n={n}: lo={eff_lo} ctas/SM={eff_c} {t:.3f} ms (built-in {t_default:.3f} ms, "
                f"{count} matrices)")
    return {"key": device_key(), "method": method, "precision": name, "entries": entries}


def _prec_name(code: int) -> str:
    return {_native.PREC_FP64: "fp64", _native.PREC_FP64_DADD: "fp64-dadd"}.get(code, "float-float")


def _tables(doc: dict) -> list[dict]:
    """The tables of a cache document (one table per method and arithmetic)."""
    if "tables" in doc:
        return list(doc["tables"])
    if "entries" in doc:  # a document holding one table
        return [doc]
    return []


def apply(table: dict) -> int:
    """Installs a table's entries (a table, or a cache document of several); returns how
    many were set."""
    k = 0
    for t in _tables(table):
        method = int(t.get("method", 0))
        prec = t.get("precision", "float-float")
        for n, e in t.get("entries", {}).items():
            _native.set_perm_tuning(method, int(n), int(e["lo_bits"]), int(e["ctas_per_sm"]), precision=prec)
            k += 1
    return k


def save(table: dict, path: Path | None = None) -> Path:
    """Adds (or replaces) a table in the cache document for this device and build."""
    path = Path(path) if path else default_cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    doc = {"key": table["key"], "tables": []}
    try:
        old = json.loads(path.read_text())
        if old.get("key") == table["key"]:
            doc["tables"] = [t for t in _tables(old)
                             if (t.get("method", 0), t.get("precision", "float-float")) !=
                             (table.get("method", 0), table.get("precision", "float-float"))]
    except (OSError, ValueError):
        pass
    doc["tables"].append({k: v for k, v in table.items() if k != "key"})
    tmp = path.with_name(f"{path.name}.{os.getpid()}.tmp")
    tmp.write_text(json.dumps(doc, indent=1, sort_keys=True))
    os.replace(tmp, path)  # atomic: concurrent processes never read a partial table
    return path


def _cached(path: Path, key: dict) -> list[dict]:
    if not path.exists():
        return []
    try:
        doc = json.loads(path.read_text())
    except (OSError, ValueError):
        return []
    if doc.get("key") != key:
        return []
    return _tables(doc)


def load(path: Path | None = None, key: dict | None = None) -> bool:
    """Applies the cached tables if they exist and were made for this device and build."""
    path = Path(path) if path else default_cache_path()
    tables = _cached(path, key if key is not None else device_key())
    return sum(apply(t) for t in tables) > 0


def ensure_tuned(sizes=range(8, 27), method: int = 0, path: Path | None = None, log=None,
                 precision="fp64") -> dict | None:
    """Loads the cached table of (method, arithmetic) for this device, or tunes ``sizes``
    and caches the result."""
    path = Path(path) if path else default_cache_path()
    name = _prec_name(_native.precision_code(precision))
    tables = _cached(path, device_key())
    for t in tables:
        if int(t.get("method", 0)) == method and t.get("precision", "float-float") == name:
            apply(t)
            return None
    table = tune_permanents(sizes, method, log=log, precision=precision)
    save(table, path)
    return table
