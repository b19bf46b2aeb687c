"""Seeded real spherical-harmonic test fields.

``f(p) = offset + sum_{l<=L} sum_{m=-l..l} a_lm Y_lm(p)`` with
``a_lm ~ N(0,1) / (1+l)^2`` drawn from ``numpy.random.default_rng(seed)`` in
(l, m) order, m from -l to l. ``Y_lm`` are orthonormal real harmonics
without the Condon-Shortley phase, evaluated with the standard stable
three-term recurrence of the fully normalised associated Legendre functions.
Evaluation runs in float64 on whatever device the points tensor lives on
(the GPU for the large bench grids, the CPU in tests).
"""

from __future__ import annotations

import math

import numpy as np
import torch


def sh_coefficients(lmax: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((lmax + 1) ** 2)
    l_of = np.concatenate([np.full(2 * l + 1, l) for l in range(lmax + 1)])
    return a / (1.0 + l_of) ** 2


def sh_field(xyz, lmax: int, seed: int, offset: float = 0.0, device=None, chunk: int = 1 << 20) -> torch.Tensor:
    """Evaluate the seeded field at unit vectors ``xyz`` ([n,3]); returns a
    float64 tensor on ``device`` (default: the device of ``xyz`` if it is a
    tensor, else CPU)."""
    return sh_fields(xyz, lmax, [seed], offset, device, chunk)[0]


def sh_fields(xyz, lmax: int, seeds, offset: float = 0.0, device=None, chunk: int = 1 << 19) -> torch.Tensor:
    """Several seeded fields at once: returns float64 [len(seeds), n]."""
    if not isinstance(xyz, torch.Tensor):
        xyz = torch.as_tensor(np.ascontiguousarray(xyz), dtype=torch.float64)
    if device is not None:
        xyz = xyz.to(device)
    xyz = xyz.to(torch.float64)
    coef = torch.as_tensor(np.stack([sh_coefficients(lmax, s) for s in seeds]), dtype=torch.float64,
                           device=xyz.device)
    out = torch.empty((len(seeds), xyz.shape[0]), dtype=torch.float64, device=xyz.device)
    for s in range(0, xyz.shape[0], chunk):
        out[:, s:s + chunk] = _eval_chunk(xyz[s:s + chunk], lmax, coef) + offset
    return out


def _eval_chunk(p: torch.Tensor, lmax: int, coef: torch.Tensor) -> torch.Tensor:
    """coef: [F, (lmax+1)^2] -> [F, n]."""
    z = p[:, 2].clamp(-1.0, 1.0)
    sint = torch.sqrt(torch.clamp(1.0 - z * z, min=0.0))
    phi = torch.atan2(p[:, 1], p[:, 0])
    res = torch.zeros((coef.shape[0], z.shape[0]), dtype=z.dtype, device=z.device)

    def cidx(l, m):  # index of a_lm in the flat coefficient vector
        return l * l + (m + l)

    pmm = torch.full_like(z, 1.0 / math.sqrt(4.0 * math.pi))
    for m in range(0, lmax + 1):
        if m > 0:
            pmm = pmm * (math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * sint)
        # Legendre column P_l^m, l = m..lmax, as rows of a matrix
        cols = [pmm]
        if m + 1 <= lmax:
            p_lm1 = pmm
            p_l = math.sqrt(2.0 * m + 3.0) * z * pmm
            cols.append(p_l)
            for l in range(m + 2, lmax + 1):
                a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
                b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
                p_new = a * (z * p_l - b * p_lm1)
                p_lm1, p_l = p_l, p_new
                cols.append(p_l)
        P = torch.stack(cols)  # [lmax-m+1, n]
        ipos = [cidx(l, m) for l in range(m, lmax + 1)]
        cpos = coef[:, ipos] @ P
        if m == 0:
            res = res + cpos
        else:
            ineg = [cidx(l, -m) for l in range(m, lmax + 1)]
            cneg = coef[:, ineg] @ P
            res = res + math.sqrt(2.0) * (cpos * torch.cos(m * phi) + cneg * torch.sin(m * phi))
    return res
