"""GPU SLOS against the FP64 oracle (1e-10 relative to the largest amplitude, and
1e-10 relative elementwise where |p| >= 1e-6 max p), plus sum rules at full size, in
both arithmetics (native FP64, the default, and float-float)."""
import math

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary
from perceval_gb300.utils.states import fock_rank

pytestmark = pytest.mark.gpu
RTOL = 1e-10
PRECS = ["fp64", "float-float"]


def run(native, U, inp, batch=1, prec="fp64"):
    plan = native.SlosPlan(len(inp), inp, batch=batch, precision=prec)
    plan.forward(torch.from_numpy(np.ascontiguousarray(U)).cuda())
    p = plan.probabilities().cpu().numpy()
    a = plan.amplitudes().cpu().numpy()
    return p, a


def check(got_p, got_a, ref_p, ref_a):
    scale = np.abs(ref_a).max()
    assert np.abs(got_a - ref_a).max() <= RTOL * scale
    big = ref_p >= 1e-6 * ref_p.max()
    assert (np.abs(got_p - ref_p)[big] / ref_p[big]).max() <= RTOL
    assert np.abs(got_p - ref_p).max() <= RTOL * ref_p.max()


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("inp", [(1, 1, 1, 0, 0), (2, 0, 1, 0, 0), (0, 3, 0, 0, 1), (0, 0, 0, 0, 0), (0, 0, 0, 0, 5)])
def test_small_vs_oracle(native, oracle, inp, prec):
    U = random_unitary(5, seed=3)
    check(*run(native, U, inp, prec=prec), *oracle.slos(U, inp))


@pytest.mark.parametrize("prec", PRECS)
def test_golden_vectors(native, golden, prec):
    for case in golden["slos"]:
        m = case["m"]
        U = np.array([complex(*v) for v in case["unitary"]]).reshape(m, m)
        ref = np.array([complex(float(a), float(b)) for a, b in case["amplitudes"]])
        _, a = run(native, U, case["input"], prec=prec)
        assert np.abs(a - ref).max() <= RTOL * np.abs(ref).max()


@pytest.mark.parametrize("prec", PRECS)
def test_config_m12_n6(native, oracle, prec):
    U = random_unitary(12, seed=0)
    inp = [1] * 6 + [0] * 6
    p, a = run(native, U, inp, prec=prec)
    assert len(p) == 12376
    check(p, a, *oracle.slos(U, inp))
    assert abs(p.sum() - 1) < 1e-12


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("m,inp_seed", [(8, 1), (16, 2), (24, 3), (32, 4)])
def test_random_inputs_with_collisions(native, oracle, m, inp_seed, prec):
    rng = np.random.default_rng(inp_seed)
    n = {8: 6, 16: 5, 24: 4, 32: 4}[m]
    inp = np.bincount(rng.integers(0, m, n), minlength=m)
    U = random_unitary(m, seed=inp_seed)
    check(*run(native, U, inp, prec=prec), *oracle.slos(U, inp))


@pytest.mark.parametrize("prec", PRECS)
def test_batched_matches_single(native, oracle, prec):
    m, B = 6, 37
    inp = (1, 0, 2, 0, 1, 0)
    Us = np.stack([random_unitary(m, seed=100 + b) for b in range(B)])
    p, a = run(native, Us, inp, batch=B, prec=prec)
    count = len(p) // B
    p = p.reshape(count, B)
    a = a.reshape(count, B)
    for b in (0, 5, 31, 32, 36):
        check(p[:, b], a[:, b], *oracle.slos(Us[b], inp))


@pytest.mark.parametrize("prec", PRECS)
def test_m16_n8_batch_sum_rule(native, prec):
    B = 64
    Us = np.stack([random_unitary(16, seed=b) for b in range(B)])
    p, _ = run(native, Us, [1] * 8 + [0] * 8, batch=B, prec=prec)
    s = p.reshape(-1, B).sum(axis=0)
    assert np.abs(s - 1).max() < 1e-11


@pytest.mark.parametrize("prec", PRECS)
def test_large_m24_n12_properties(native, oracle, prec):
    # the scale-up workload: C(35,12) = 834,451,800 outputs (13.4 GB per layer);
    # checked by the unitarity sum rule and by spot amplitudes against the oracle's
    # FP64 permanents (rows = output modes repeated by count, columns = input modes)
    m, n = 24, 12
    U = random_unitary(m, seed=0)
    inp = [1] * n + [0] * (m - n)
    plan = native.SlosPlan(m, inp, precision=prec)
    Ud = torch.from_numpy(U).cuda()
    plan.forward(Ud)
    probs = plan.probabilities()
    assert probs.numel() == math.comb(35, 12)
    assert abs(float(probs.sum()) - 1) < 1e-10
    amps = plan.amplitudes()
    rng = np.random.default_rng(0)
    outs = []
    for _ in range(16):
        o = np.bincount(rng.integers(0, m, n), minlength=m)
        outs.append(o)
    rows = [np.repeat(np.arange(m), o) for o in outs]
    cols = np.arange(n)
    mats = [np.ascontiguousarray(U[np.ix_(r, cols)]) for r in rows]
    flat = np.concatenate([x.reshape(-1) for x in mats])
    offs = np.arange(len(mats), dtype=np.int64) * n * n
    perms = oracle.perm_batch(flat, offs, np.full(len(mats), n, dtype=np.int32))
    for o, pm in zip(outs, perms):
        amp = complex(amps[fock_rank(o)].item())
        ref = pm / math.sqrt(math.prod(math.factorial(int(v)) for v in o))
        assert abs(amp - ref) <= 1e-10 * max(abs(ref), 1e-6)
    del plan, probs, amps
    torch.cuda.empty_cache()


def test_plan_errors(native):
    with pytest.raises(RuntimeError, match="outside"):
        native.SlosPlan(33, [0] * 33)
    with pytest.raises(RuntimeError, match="more than 2"):
        native.SlosPlan(32, [1] * 20 + [0] * 12)
    plan = native.SlosPlan(3, [1, 1, 0])
    with pytest.raises(RuntimeError, match="forward"):
        plan.probabilities()
    with pytest.raises(RuntimeError, match="keep_layers"):
        plan.forward(torch.from_numpy(random_unitary(3, seed=1)).cuda())
        plan.backward(torch.zeros(plan.count, dtype=torch.float64, device="cuda"))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("m,n", [(6, 3), (12, 6), (16, 8), (20, 10), (24, 8), (9, 0)])
def test_fused_probabilities_equal_two_pass(native, m, n, prec):
    """forward_probabilities (the last layer writes probabilities, one circuit) gives
    exactly the forward + probabilities results, over the large-tile and the grouped
    small-tile paths; afterwards the plan refuses amplitudes until a plain forward."""
    inp = [1] * n + [0] * (m - n)
    U = torch.from_numpy(random_unitary(m, seed=m + n)).cuda()
    plan = native.SlosPlan(m, inp, precision=prec)
    plan.forward(U)
    ref = plan.probabilities().clone()
    got = plan.forward_probabilities(U)
    assert torch.equal(got, ref)
    if n > 0:
        with pytest.raises(RuntimeError):
            plan.amplitudes()
    plan.forward(U)
    assert torch.equal(plan.probabilities(), ref)


def test_fused_probabilities_batched_and_masked(native):
    from perceval_gb300.utils import FSMask
    m, inp = 8, [1, 1, 0, 1, 0, 0, 1, 0]
    Us = torch.from_numpy(np.stack([random_unitary(m, seed=40 + b) for b in range(5)])).cuda()
    plan = native.SlosPlan(m, inp, batch=5)
    plan.forward(Us)
    ref = plan.probabilities().clone()
    assert torch.equal(plan.forward_probabilities(Us), ref)
    mplan = native.SlosPlan(m, inp, mask=FSMask(m, 4, ["******00"]))
    mplan.forward(Us[0])
    mref = mplan.probabilities().clone()
    assert torch.equal(mplan.forward_probabilities(Us[0].contiguous()), mref)


def test_fp64_and_float_float_agree_m20_n10(native):
    """The two arithmetics on the same 20,030,010 outputs: probabilities within 1e-10 of
    the largest one (float-float carries ~48 significant bits)."""
    m, n = 20, 10
    U = torch.from_numpy(random_unitary(m, seed=7)).cuda()
    inp = [1] * n + [0] * (m - n)
    p64 = native.SlosPlan(m, inp).forward_probabilities(U)
    pff = native.SlosPlan(m, inp, precision="float-float").forward_probabilities(U)
    assert float((p64 - pff).abs().max()) <= 1e-10 * float(p64.max())
    assert abs(float(p64.sum()) - 1) < 1e-12
