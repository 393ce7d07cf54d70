"""Permanent plans (one CUDA graph per execution) and tuned launch shapes: a plan
returns exactly what pcvl_permanent_batch returns (same kernels, same shapes) and keeps
doing so when the input and output buffers change; tuned shapes stay within 1e-10
relative of the oracle; the autotuner installs and caches a table."""
import numpy as np
import pytest
import torch

from test_permanent_gpu import haar_submatrices, pack

pytestmark = pytest.mark.gpu
RTOL = 1e-10


@pytest.fixture(autouse=True)
def reset_table():
    yield
    from perceval_gb300 import _native
    for prec in ("fp64", "float-float"):
        for method in (0, 1):
            for n in range(1, 41):
                _native.set_perm_tuning(method, n, precision=prec)


def _mixed(seed):
    mats = haar_submatrices(300, 1, 20, seed=seed)
    mats.insert(5, np.zeros((0, 0), complex))
    return mats


@pytest.mark.parametrize("prec", ["fp64", "float-float"])
@pytest.mark.parametrize("method", [0, 1])
def test_plan_equals_batch_call(native, method, prec):
    mats = _mixed(1)
    flat, offs, sizes = pack(mats)
    dev = torch.from_numpy(flat).cuda()
    ref = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    native.permanent_batch(dev, offs, sizes, ref, method, precision=prec)
    plan = native.PermPlan(offs, sizes, method, precision=prec)
    got = plan(dev)
    assert torch.equal(got, ref)
    assert got[5].item() == 1.0
    # new input and output buffers: the graph's pointers follow
    rng = np.random.default_rng(2)
    mats2 = [0.7 * m + 0.05 * (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)) for m in mats]
    flat2 = np.concatenate([m.reshape(-1) for m in mats2])
    dev2 = torch.from_numpy(flat2).cuda()
    ref2 = torch.empty_like(ref)
    native.permanent_batch(dev2, offs, sizes, ref2, method, precision=prec)
    out2 = torch.empty_like(ref)
    for _ in range(3):
        plan(dev2, out2)
    assert torch.equal(out2, ref2)
    assert torch.equal(plan(dev), ref)
    assert plan.nbytes > 0
    plan.close()


def test_plan_against_oracle(native, oracle):
    mats = haar_submatrices(64, 1, 12, seed=3)
    flat, offs, sizes = pack(mats)
    got = native.PermPlan(offs, sizes)(torch.from_numpy(flat).cuda()).cpu().numpy()
    ref = oracle.perm_batch(flat, offs, sizes)
    assert np.all(np.abs(got - ref) <= RTOL * np.abs(ref))


def test_plan_on_side_stream(native):
    mats = haar_submatrices(40, 8, 16, seed=4)
    flat, offs, sizes = pack(mats)
    dev = torch.from_numpy(flat).cuda()
    ref = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    native.permanent_batch(dev, offs, sizes, ref)
    s = torch.cuda.Stream()
    plan = native.PermPlan(offs, sizes)
    out = torch.empty_like(ref)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan(dev, out, stream=s)
    s.synchronize()
    assert torch.equal(out, ref)


@pytest.mark.parametrize("prec", ["fp64", "float-float"])
@pytest.mark.parametrize("n,lo,ctas", [(14, 3, 4), (18, 9, 32), (20, 8, 16), (22, 4, 2)])
def test_tuned_shapes_keep_parity(native, oracle, n, lo, ctas, prec):
    mats = haar_submatrices(6, n, n, seed=n)
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    native.set_perm_tuning(0, n, lo, ctas, precision=prec)
    dev = torch.from_numpy(flat).cuda()
    out = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    native.permanent_batch(dev, offs, sizes, out, precision=prec)
    assert np.all(np.abs(out.cpu().numpy() - ref) <= RTOL * np.abs(ref))
    plan_out = native.PermPlan(offs, sizes, precision=prec)(dev).cpu().numpy()
    assert np.array_equal(plan_out, out.cpu().numpy())


def test_autotuner_installs_and_caches(native, tmp_path):
    from perceval_gb300 import autotune
    table = autotune.tune_permanents(sizes=[9, 13], target_ms=1.0, reps=1)
    assert table["precision"] == "fp64"
    assert set(table["entries"]) == {"9", "13"}
    for n, e in table["entries"].items():
        assert native.get_perm_tuning(0, int(n)) == (e["lo_bits"], e["ctas_per_sm"])
        assert e["ms"] <= e["default_ms"]
    path = autotune.save(table, tmp_path / "tuning.json")
    ff = autotune.tune_permanents(sizes=[11], target_ms=1.0, reps=1, precision="float-float")
    autotune.save(ff, path)
    for n in (9, 13):
        native.set_perm_tuning(0, n)
    native.set_perm_tuning(0, 11, precision="float-float")
    assert autotune.load(path)
    for n, e in table["entries"].items():
        assert native.get_perm_tuning(0, int(n)) == (e["lo_bits"], e["ctas_per_sm"])
    e = ff["entries"]["11"]
    assert native.get_perm_tuning(0, 11, precision="float-float") == (e["lo_bits"], e["ctas_per_sm"])
