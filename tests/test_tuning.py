"""Host-side logic of the permanent tuning table (no GPU): set/get round trips, the
refusals of impossible shapes, and the JSON cache's device check."""
import json

import pytest

from perceval_gb300 import _native


@pytest.fixture(autouse=True)
def reset_table():
    yield
    for method in (0, 1):
        for n in range(1, 41):
            _native.set_perm_tuning(method, n)


def test_defaults_and_round_trip():
    assert _native.get_perm_tuning(0, 24) == (7, 8)   # built-in: min(7, F - 7), 8 CTAs/SM
    assert _native.get_perm_tuning(0, 10) == (2, 8)
    assert _native.get_perm_tuning(1, 10) == (3, 8)
    _native.set_perm_tuning(0, 24, 5, 16)
    assert _native.get_perm_tuning(0, 24) == (5, 16)
    assert _native.get_perm_tuning(1, 24) == (7, 8)    # per method
    _native.set_perm_tuning(0, 3, 9, 4)                # clamped to the free bits
    assert _native.get_perm_tuning(0, 3) == (2, 4)
    _native.set_perm_tuning(0, 24)
    assert _native.get_perm_tuning(0, 24) == (7, 8)


@pytest.mark.parametrize("args", [(2, 10, 3, 8), (0, 0, 3, 8), (0, 41, 3, 8), (0, 10, -2, 8), (0, 10, 3, 65),
                                  (0, 36, 10, 8)])
def test_refusals(args):
    with pytest.raises(RuntimeError):
        _native.set_perm_tuning(*args)


def test_cache_applies_only_to_its_device(tmp_path):
    from perceval_gb300 import autotune
    key = {"device": "GB300-test", "sms": 152, "library": "x"}
    table = {"key": key, "method": 0, "entries": {"20": {"lo_bits": 6, "ctas_per_sm": 16, "ms": 1.0}}}
    path = tmp_path / "t.json"
    path.write_text(json.dumps(table))
    assert not autotune.load(path, key={"device": "other", "sms": 152, "library": "x"})
    assert _native.get_perm_tuning(0, 20) == (7, 8)
    assert autotune.load(path, key=key)
    assert _native.get_perm_tuning(0, 20) == (6, 16)
    assert not autotune.load(tmp_path / "missing.json", key=key)


def test_candidates_fit_shared_memory():
    from perceval_gb300 import autotune
    for n in range(2, 41):
        for lo, c in autotune.candidates(n):
            assert (n * n + (1 << lo) * n) * 16 <= 227 * 1024 and c in (4, 8, 16, 32)
