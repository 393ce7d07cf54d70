"""Exact boson sampling on the GPU (restating perceval/backends/_clifford2017.py:36-61).

``samples(count)`` draws all samples in one ``pcvl_cc2017_sample`` call (Clifford &
Clifford 2018 algorithm B): up to 32768 samples advance together photon by photon, two
kernels per photon over all of them (the sub-permanents, spread over lane groups and
CTAs, then the weights and the draw).  Randomness comes from
Philox4x32-10 keyed by the seed of ``perceval_gb300.utils.random_seed``; every
sample has its own counter, so a fixed seed gives the same samples however the
launch is scheduled, and successive calls continue the stream.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native
from ..utils import _random
from ..utils.states import BSSamples, FockState
from ._abstract_backends import ASamplingBackend


class Clifford2017Backend(ASamplingBackend):
    def __init__(self, precision: str = "double"):
        super().__init__()
        names = {"double": _native.PREC_FLOAT_FLOAT, "float-float": _native.PREC_FLOAT_FLOAT,
                 "fp64": _native.PREC_FP64, "single": _native.PREC_FP32, "fp32": _native.PREC_FP32}
        if precision not in names:
            raise ValueError("precision must be 'double' / 'float-float' (FP64-class pairs, the default), "
                             "'fp64' (FP64 precision: exact fixed-point sums, block-floating products on "
                             "the integer pipes, FP64 sums) or 'single' / 'fp32'")
        self._precision = names[precision]
        self._u_dev = None

    @property
    def name(self) -> str:
        return "CliffordClifford2017"

    def set_circuit(self, circuit):
        super().set_circuit(circuit)
        self._u_dev = None

    def _unitary_device(self) -> torch.Tensor:
        if self._u_dev is None:
            _native.load()
            self._u_dev = torch.from_numpy(self._umat).to("cuda")
        return self._u_dev

    def samples_tensor(self, count: int) -> torch.Tensor:
        """``count`` samples as an int32 CUDA tensor of shape (count, m)."""
        assert self._input_state is not None, "Input state must be set before sampling"
        seed, first = _random.take_samples(count)
        return _native.cc2017_sample(self._unitary_device(), list(self._input_state), count, seed, first,
                                     self._precision)

    def samples(self, count: int) -> BSSamples:
        """Request ``count`` samples; one GPU launch draws them all."""
        arr = self.samples_tensor(count).cpu().numpy()
        return BSSamples(FockState(row) for row in arr)

    def sample(self) -> FockState:
        return self.samples(1)[0]

    def samples_many(self, input_states, counts) -> list[BSSamples]:
        """``counts[b]`` samples of each input state ``input_states[b]`` through the current
        circuit: the per-input loop of SamplesProvider (noisy_sampling_simulator.py:68-69,
        120-121) as one wavefront per photon count.  The stream advances as for one
        ``samples(sum(counts))`` call."""
        states = [FockState(s) for s in input_states]
        counts = [int(c) for c in counts]
        assert len(states) == len(counts), "one count per input state"
        m = self._umat.shape[0]
        for st in states:
            assert st.m == m, "Input state size mismatch"
        seed, first = _random.take_samples(sum(counts))
        res: list = [None] * len(states)
        groups: dict[int, list[int]] = {}
        for i, st in enumerate(states):
            groups.setdefault(st.n, []).append(i)
        offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        U = self._unitary_device()
        for n, idx in sorted(groups.items()):
            # every state keeps the counters it holds in the whole request (offset offs[i])
            arr = np.array([list(states[i]) for i in idx], dtype=np.int32)
            grp_counts = [counts[i] for i in idx]
            if idx == list(range(idx[0], idx[0] + len(idx))):
                out = _native.cc2017_sample_multi(U, arr, grp_counts, seed, first + int(offs[idx[0]]),
                                                  self._precision).cpu().numpy()
                o = 0
                for i, c in zip(idx, grp_counts):
                    res[i] = BSSamples(FockState(row) for row in out[o:o + c])
                    o += c
            else:  # states of this count are not contiguous in the request: one call per state
                for i in idx:
                    out = _native.cc2017_sample(U, list(states[i]), counts[i], seed, first + int(offs[i]),
                                                self._precision).cpu().numpy()
                    res[i] = BSSamples(FockState(row) for row in out)
        return res
