"""Reference data layout (the drop-in ABI) as numpy dtypes and array shapes.

The reference passes packed array-of-structs buffers to its three OpenCL
kernels (functions.h:49-113; the same structs head U_Q.cl, Viscous.cl and
Weno.cl).  This module names those layouts once so that the host mirror, the
case generators and the tests agree with the C header include/cfd_rhs.h:

==============  =======  ===================================================
struct          bytes    numpy form used here
==============  =======  ===================================================
GRID            56       structured dtype GRID_DTYPE (x,y,z, N0..N5, ID, loc)
FLOW_VARIABLES  72       float64 (n, 9): u, v, w, p, t, rho, mu, a, e
Solver_Column   40       float64 (n, 5): N0..N4 = rho, rho u, rho v, rho w, E
TRANSFORMED     504      float64 (n, 63): blocks node, ip, im, jp, jm, kp, km;
                         each block zeta_{x,y,z}, eta_{x,y,z}, xi_{x,y,z}
DETERM          48       float64 (n, 6): ip, im, jp, jm, kp, km
ROE_AVERAGING   288      float64 (n, 36): blocks ip, jp, kp, im, jm, km of
                         (u, v, w, p, h, rho)
det             8        float64 (n,)
==============  =======  ===================================================

Index 0 of every array is the reference's dummy row; owned nodes are
1..sd_node and ghost nodes sd_node+1..g_node.  Neighbour codes: N0 = +j,
N1 = +i, N2 = -j, N3 = -i, N4 = +k, N5 = -k (U_Q.cl:51-56).  ``loc`` is 0 for
interior nodes, 1..56 for boundary nodes and 100 for ghost nodes.
"""
from __future__ import annotations

import numpy as np

GRID_DTYPE = np.dtype(
    [("x", "<f8"), ("y", "<f8"), ("z", "<f8"),
     ("N0", "<i4"), ("N1", "<i4"), ("N2", "<i4"), ("N3", "<i4"), ("N4", "<i4"), ("N5", "<i4"),
     ("ID", "<i4"), ("loc", "<i4")])
assert GRID_DTYPE.itemsize == 56

FLOW_FIELDS = ("u", "v", "w", "p", "t", "rho", "mu", "a", "e")
FLOW = {name: k for k, name in enumerate(FLOW_FIELDS)}
NFLOW = 9
NCOL = 5
NMETRIC = 63
NDETERM = 6
NROE = 36

# TRANSFORMED block index of the half-point metric of each face
METRIC_BLOCK = {"node": 0, "ip": 1, "im": 2, "jp": 3, "jm": 4, "kp": 5, "km": 6}
# ROE_AVERAGING block order (note: differs from DETERM's order)
ROE_BLOCK = {"ip": 0, "jp": 1, "kp": 2, "im": 3, "jm": 4, "km": 5}
ROE_FIELD = {"u": 0, "v": 1, "w": 2, "p": 3, "h": 4, "rho": 5}
DETERM_INDEX = {"ip": 0, "im": 1, "jp": 2, "jm": 3, "kp": 4, "km": 5}

# neighbour field for (+/-) along i, j, k
PLUS = ("N1", "N0", "N4")
MINUS = ("N3", "N2", "N5")

BYTES_PER_NODE_REFERENCE = 56 + 72 + 288 + 4 * 40 + 6 * 40 + 504 + 8 + 48  # 1,376


def empty_arrays(n_rows: int) -> dict:
    """Zeroed arrays of every reference buffer for ``n_rows`` rows."""
    return {
        "grid": np.zeros(n_rows, GRID_DTYPE),
        "det": np.zeros(n_rows),
        "deter": np.zeros((n_rows, NDETERM)),
        "metric": np.zeros((n_rows, NMETRIC)),
        "flow": np.zeros((n_rows, NFLOW)),
        "U0": np.zeros((n_rows, NCOL)),
        "U1": np.zeros((n_rows, NCOL)),
        "U2": np.zeros((n_rows, NCOL)),
        "Q": np.zeros((n_rows, NCOL)),
        "F": np.zeros((n_rows, NCOL)),
        "E": np.zeros((n_rows, NCOL)),
        "G": np.zeros((n_rows, NCOL)),
        "Fv": np.zeros((n_rows, NCOL)),
        "Ev": np.zeros((n_rows, NCOL)),
        "Gv": np.zeros((n_rows, NCOL)),
        "roe": np.zeros((n_rows, NROE)),
    }
