"""Concurrent calls on two streams from two host threads: every plan-free entry point
takes its scratch from a stream-ordered pool per call, so two backends running side by
side (as the reference runs simulations on LocalJob threads) get exactly the results of
the same calls made one after the other."""
import threading

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary
from test_permanent_gpu import haar_submatrices, pack

pytestmark = pytest.mark.gpu


def _inputs(seed):
    """Host inputs of one worker, made before any thread starts (numpy's LAPACK calls are
    not meant to run concurrently from several threads)."""
    mats = haar_submatrices(200, 6, 18, seed=seed)
    flat, offs, sizes = pack(mats)
    return flat, offs, sizes, random_unitary(40, seed=seed)


def _work(native, inputs, seed, stream, results, key, reps):
    flat, offs, sizes, U = inputs
    inp = [1] * 6 + [0] * 34
    with torch.cuda.stream(stream):
        dev = torch.from_numpy(flat).cuda()
        Ud = torch.from_numpy(U).cuda()
        outs = []
        for r in range(reps):
            out = torch.empty(len(sizes), dtype=torch.complex128, device="cuda")
            native.permanent_batch(dev, offs, sizes, out, precision="fp64" if r % 2 == 0 else "float-float",
                                   stream=stream)
            samples = native.cc2017_sample(Ud, inp, 256, seed=seed, first_sample=256 * r, stream=stream)
            probs = native.slap_all(Ud, inp, stream=stream)
            outs.append((out, samples, probs))
        stream.synchronize()
    results[key] = [(o.cpu().numpy(), s.cpu().numpy(), p.cpu().numpy()) for o, s, p in outs]


def test_two_threads_two_streams_match_serial_calls(native, oracle):
    reps = 6
    ins = {"a": _inputs(1), "b": _inputs(2)}
    serial = {}
    s0 = torch.cuda.Stream()
    _work(native, ins["a"], 1, s0, serial, "a", reps)
    _work(native, ins["b"], 2, s0, serial, "b", reps)
    conc = {}
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    ta = threading.Thread(target=_work, args=(native, ins["a"], 1, sa, conc, "a", reps))
    tb = threading.Thread(target=_work, args=(native, ins["b"], 2, sb, conc, "b", reps))
    ta.start()
    tb.start()
    ta.join()
    tb.join()
    again = {}
    _work(native, ins["a"], 1, s0, again, "a", reps)
    for key in ("a", "b"):
        assert len(conc[key]) == reps
        for r, ((po, so, qo), (pc, sc, qc)) in enumerate(zip(serial[key], conc[key])):
            if key == "a":
                assert np.array_equal(po, again["a"][r][0]), ("serial calls differ", r)
            bad = np.nonzero(po != pc)[0]
            assert bad.size == 0, (key, r, bad[:8], np.abs(po - pc)[bad[:8]] / np.abs(po[bad[:8]]))
            assert np.array_equal(so, sc), (key, r, "samples")
            assert np.array_equal(qo, qc), (key, r, "slap")
    # and the permanents are the oracle's
    flat, offs, sizes, _ = ins["a"]
    ref = oracle.perm_batch(flat, offs, sizes)
    got = conc["a"][0][0]
    assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-10
