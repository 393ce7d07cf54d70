"""Differentiable unitary of a rectangular mesh of ``mzi phase last`` cells (torch).

The mesh is the one ``GenericInterferometer(m, catalog['mzi phase last'].generate)``
builds (perceval/components/generic_interferometer.py:150-165,
perceval/components/core_catalog/mzi.py:97-100): column i holds cells on mode pairs
(j, j+1), j = i % 2, i % 2 + 2, ..., numbered in placement order; cell idx has the
phases (phi_a{idx}, phi_b{idx}) and the 2x2 matrix

    M = diag(1, e^{i phi_b}) . B . diag(1, e^{i phi_a}) . B,  B = [[1, i], [i, 1]] / sqrt(2).

``phases`` has shape (batch, 2 * n_cells) laid out as
[phi_a0, phi_b0, phi_a1, phi_b1, ...].  The result is complex128 (batch, m, m) and
carries torch autograd, so a gradient dL/dU (torch convention: dL/dRe + i dL/dIm)
chains to dL/dphases by ``U.backward(G)``.
"""
from __future__ import annotations

import math

import torch


def mesh_cells(m: int) -> list[tuple[int, int]]:
    """(cell index, top mode j) in placement order for the m-mode rectangle."""
    cells = []
    for i in range(m):
        for j in range(i % 2, m - 1, 2):
            cells.append(j)
    return list(enumerate(cells))


def clements_mesh_phase_count(m: int) -> int:
    return 2 * len(mesh_cells(m))


def clements_mesh_unitary(phases: torch.Tensor, m: int) -> torch.Tensor:
    """Batched mesh unitary, differentiable w.r.t. ``phases`` (float64)."""
    if phases.dim() == 1:
        return clements_mesh_unitary(phases[None], m)[0]
    bsz = phases.shape[0]
    cells = mesh_cells(m)
    assert phases.shape[1] == 2 * len(cells), "phases must hold 2 values per MZI cell"
    dev = phases.device
    r = 1.0 / math.sqrt(2.0)
    B = torch.tensor([[r, 1j * r], [1j * r, r]], dtype=torch.complex128, device=dev)
    rows = [torch.zeros(bsz, m, dtype=torch.complex128, device=dev) for _ in range(m)]
    for i in range(m):
        rows[i] = rows[i].clone()
        rows[i][:, i] = 1.0
    for idx, j in cells:
        ea = torch.exp(1j * phases[:, 2 * idx].to(torch.complex128))
        eb = torch.exp(1j * phases[:, 2 * idx + 1].to(torch.complex128))
        x0, x1 = rows[j], rows[j + 1]
        # B, then diag(1, ea), then B, then diag(1, eb)
        y0 = B[0, 0] * x0 + B[0, 1] * x1
        y1 = B[1, 0] * x0 + B[1, 1] * x1
        y1 = ea[:, None] * y1
        z0 = B[0, 0] * y0 + B[0, 1] * y1
        z1 = B[1, 0] * y0 + B[1, 1] * y1
        z1 = eb[:, None] * z1
        rows[j], rows[j + 1] = z0, z1
    return torch.stack(rows, dim=1)
