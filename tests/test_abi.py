"""The C-ABI library loads and exports every function include/pcvl_gb300.h declares
(no compute calls: no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared():
    text = (ROOT / "include" / "pcvl_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pcvl_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from perceval_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared()
    for must in ("pcvl_permanent_batch", "pcvl_slos_forward", "pcvl_slos_backward", "pcvl_cc2017_sample",
                 "pcvl_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_without_gpu(lib):
    lib.pcvl_version.restype = ctypes.c_char_p
    assert lib.pcvl_version().startswith(b"pcvl_gb300")
    buf = ctypes.create_string_buffer(64)
    assert lib.pcvl_last_error(buf, 64) == 0
    assert lib.pcvl_last_error(None, 0) != 0


def test_argument_errors_are_reported_without_device_work(lib):
    from perceval_gb300 import _native
    L = _native.load(require_cuda=False)
    import numpy as np
    sizes = np.array([50], dtype=np.int32)
    offs = np.array([0], dtype=np.int64)
    # size 50 exceeds the kernel's limit: refused on the host before any CUDA call
    rc = L.pcvl_permanent_batch(ctypes.c_void_p(16), offs.ctypes.data, sizes.ctypes.data, 1, ctypes.c_void_p(16), 0,
                                2, None)
    assert rc == 1 and "outside" in _native.last_error()
    rc = L.pcvl_permanent_batch(None, None, None, -1, None, 0, 2, None)
    assert rc == 1
    # an unknown arithmetic is refused (FP32 serves the sampler only)
    sizes = np.array([3], dtype=np.int32)
    rc = L.pcvl_permanent_batch(ctypes.c_void_p(16), offs.ctypes.data, sizes.ctypes.data, 1, ctypes.c_void_p(16), 0,
                                1, None)
    assert rc == 1 and "precision" in _native.last_error()
    # overlapping matrices are refused before any device work (identical entries are allowed)
    sizes = np.array([3, 3, 2], dtype=np.int32)
    offs = np.array([0, 0, 4], dtype=np.int64)
    rc = L.pcvl_permanent_batch(ctypes.c_void_p(16), offs.ctypes.data, sizes.ctypes.data, 3, ctypes.c_void_p(16), 0,
                                2, None)
    assert rc == 1 and "overlap" in _native.last_error()
    h = ctypes.c_void_p()
    inp = np.array([1] * 40, dtype=np.int32)
    rc = L.pcvl_slos_plan_create(ctypes.byref(h), 40, inp.ctypes.data, 1, 0, 2)
    assert rc == 1 and "outside" in _native.last_error()
    inp = np.array([1] * 4, dtype=np.int32)
    rc = L.pcvl_slos_plan_create(ctypes.byref(h), 4, inp.ctypes.data, 1, 0, 1)
    assert rc == 1 and "precision" in _native.last_error()


def test_masked_slap_and_mask_ranks_refuse_bad_arguments(lib):
    """New entry points check their arguments on the host, before any device work; the
    SLAP output count is host-only: C(m + n - 1, n)."""
    import math

    import numpy as np
    from perceval_gb300 import _native
    L = _native.load(require_cuda=False)
    h = ctypes.c_void_p()
    inp = np.array([1, 1, 0, 0], dtype=np.int32)
    digits = np.array([[-1, -1, 0, 0]], dtype=np.int8)
    assert L.pcvl_slos_plan_create_masked(ctypes.byref(h), 4, inp.ctypes.data, 1, 0, 0, digits.ctypes.data, 0, 2,
                                          2) == 1
    assert "n_masks" in _native.last_error()
    bad = np.array([[-1, -2, 0, 0]], dtype=np.int8)
    assert L.pcvl_slos_plan_create_masked(ctypes.byref(h), 4, inp.ctypes.data, 1, 0, 1, bad.ctypes.data, 0, 2,
                                          2) == 1
    assert "digit" in _native.last_error()
    two = np.array([1, 1, 0, 0, 1, 0, 0, 0], dtype=np.int32)
    assert L.pcvl_slos_plan_create_masked(ctypes.byref(h), 4, two.ctypes.data, 2, 0, 1, digits.ctypes.data, 0, 2,
                                          2) == 1
    assert "photon count" in _native.last_error()
    kept = ctypes.c_int64()
    assert L.pcvl_fock_mask_ranks(0, 2, 1, digits.ctypes.data, None, 2, None, 0, ctypes.byref(kept)) == 1
    assert L.pcvl_fock_mask_ranks(4, 2, 1, bad.ctypes.data, None, 2, None, 0, ctypes.byref(kept)) == 1
    c = ctypes.c_int64()
    for m, n in [(4, 2), (64, 6), (1024, 3), (3, 12)]:
        state = np.zeros(m, dtype=np.int32)
        state[0] = n
        assert L.pcvl_slap_output_count(m, state.ctypes.data, ctypes.byref(c)) == 0
        assert c.value == math.comb(m + n - 1, n)
    state = np.zeros(4, dtype=np.int32)
    state[0] = 13
    assert L.pcvl_slap_output_count(4, state.ctypes.data, ctypes.byref(c)) == 1
    assert "photons" in _native.last_error()


def test_product_path_has_no_cpu_fallback():
    import torch
    from perceval_gb300 import _native
    if torch.cuda.is_available():
        pytest.skip("only meaningful without a GPU")
    with pytest.raises(RuntimeError, match="CUDA"):
        _native.load()
