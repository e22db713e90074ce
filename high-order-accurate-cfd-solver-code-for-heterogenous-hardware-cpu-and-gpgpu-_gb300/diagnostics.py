"""Integral diagnostics of a lattice solution (host, numpy): volume-weighted
kinetic energy and enstrophy, the quantities the Taylor-Green configuration
reports.  Velocity gradients use the same fourth-order central
differences in index space and node metrics as the viscous terms
(Viscous.cl:285-453), so d u_a / d x_b = sum_d (d u_a / d zeta_d) zeta_d,b."""
from __future__ import annotations

import numpy as np

from . import layout as L


def _central4(f, axis):
    r = lambda o: np.roll(f, -o, axis=axis)
    return (1.0 / 12.0) * (8.0 * (r(1) - r(-1)) - (r(2) - r(-2)))


def kinetic_energy_enstrophy(flow: np.ndarray, metric: np.ndarray, det: np.ndarray, shape) -> tuple:
    """(KE, enstrophy) = volume averages of rho |u|^2 / 2 and |curl u|^2 / 2
    over rows 1..N of a periodic lattice of `shape` (ni, nj, nk)."""
    ni, nj, nk = shape
    f = flow[1:].reshape(nk, nj, ni, L.NFLOW)
    m = metric[1:, :9].reshape(nk, nj, ni, 3, 3)        # m[..., d, b] = d zeta_d / d x_b
    vol = det[1:].reshape(nk, nj, ni)
    rho = f[..., L.FLOW["rho"]]
    u = np.stack([f[..., L.FLOW["u"]], f[..., L.FLOW["v"]], f[..., L.FLOW["w"]]], axis=-1)
    ke = 0.5 * rho * np.sum(u * u, axis=-1)
    axes = (2, 1, 0)                                     # zeta ~ i, eta ~ j, xi ~ k
    grad = np.zeros(u.shape + (3,))                      # grad[..., a, b] = d u_a / d x_b
    for d in range(3):
        du = _central4(u, axes[d])
        grad += du[..., :, None] * m[..., d, None, :]
    w = np.stack([grad[..., 2, 1] - grad[..., 1, 2], grad[..., 0, 2] - grad[..., 2, 0],
                  grad[..., 1, 0] - grad[..., 0, 1]], axis=-1)
    ens = 0.5 * np.sum(w * w, axis=-1)
    V = vol.sum()
    return float((ke * vol).sum() / V), float((ens * vol).sum() / V)
