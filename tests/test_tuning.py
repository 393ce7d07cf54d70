"""Host-side logic of the permanent tuning table (no GPU): set/get round trips, the
refusals of impossible shapes, and the JSON cache's device check."""
import json

import pytest

from perceval_gb300 import _native


@pytest.fixture(autouse=True)
def reset_table():
    yield
    for prec in ("fp64", "float-float"):
        for method in (0, 1):
            for n in range(1, 41):
                _native.set_perm_tuning(method, n, precision=prec)


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
    # one table per arithmetic
    _native.set_perm_tuning(0, 20, 6, 32, precision="float-float")
    assert _native.get_perm_tuning(0, 20, precision="float-float") == (6, 32)
    assert _native.get_perm_tuning(0, 20) == (7, 8)
    with pytest.raises(ValueError):
        _native.get_perm_tuning(0, 20, precision="fp16")


@pytest.mark.parametrize("args", [(2, 10, 3, 8), (0, 0, 3, 8), (0, 41, 3, 8), (0, 10, -2, 8), (0, 10, 3, 65),
                                  (0, 36, 10, 8)])
def test_refusals(args):
    with pytest.raises(RuntimeError):
        _native.set_perm_tuning(*args)


def test_cache_applies_only_to_its_device(tmp_path):
    from perceval_gb300 import autotune
    key = {"device": "GB300-test", "sms": 152, "library": "x"}
    table = {"key": key, "tables": [{"method": 0, "precision": "fp64",
                                     "entries": {"20": {"lo_bits": 6, "ctas_per_sm": 16, "ms": 1.0}}},
                                    {"method": 0, "precision": "float-float",
                                     "entries": {"20": {"lo_bits": 5, "ctas_per_sm": 4, "ms": 1.0}}}]}
    path = tmp_path / "t.json"
    path.write_text(json.dumps(table))
    assert not autotune.load(path, key={"device": "other", "sms": 152, "library": "x"})
    assert _native.get_perm_tuning(0, 20) == (7, 8)
    assert autotune.load(path, key=key)
    assert _native.get_perm_tuning(0, 20) == (6, 16)
    assert _native.get_perm_tuning(0, 20, precision="float-float") == (5, 4)
    assert not autotune.load(tmp_path / "missing.json", key=key)


def test_cache_keeps_one_table_per_method_and_arithmetic(tmp_path, monkeypatch):
    from perceval_gb300 import autotune
    key = {"device": "GB300-test", "sms": 152, "library": "x"}
    path = tmp_path / "t.json"
    for prec, lo in (("fp64", 6), ("float-float", 5), ("fp64", 4)):
        autotune.save({"key": key, "method": 0, "precision": prec,
                       "entries": {"18": {"lo_bits": lo, "ctas_per_sm": 8, "ms": 1.0}}}, path)
    doc = json.loads(path.read_text())
    assert sorted((t["precision"], t["entries"]["18"]["lo_bits"]) for t in doc["tables"]) == \
        [("float-float", 5), ("fp64", 4)]
    # a table made on another device is dropped, not merged
    autotune.save({"key": dict(key, device="other"), "method": 1, "precision": "fp64", "entries": {}}, path)
    assert len(json.loads(path.read_text())["tables"]) == 1


def test_candidates_fit_shared_memory():
    from perceval_gb300 import autotune
    for n in range(2, 41):
        for lo, c in autotune.candidates(n):
            assert (n * n + (1 << lo) * n) * 16 <= 227 * 1024 and c in (4, 8, 16, 32)
