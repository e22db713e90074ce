"""The geometry producer (cfd_compact_metrics, cfd_half_point_metrics) on a
curvilinear box mesh in the reference's global form, on the CPU:

* the oracle's restatement against the reference's own metric_term()
  (Grid_Transformation.cpp) and half-point block (Main.cpp:2369-2440),
  compiled from their sources (oracle/build_ref.sh): bit for bit;
* the library's producer against the oracle: bit for bit;
* the compact scheme's node metrics against the analytic ones (a sanity
  check of the scheme itself, not of parity);
* the half-point rule of the case generators against the reference's block."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2


def _lib_metrics(grid, del_zeta=1.0):
    from cfd_gb300 import abi
    lib = abi.load()
    n = grid.shape[0]
    det = np.zeros(n)
    metric = np.zeros((n, 63))
    st = lib.cfd_compact_metrics(grid.ctypes.data, n, float(del_zeta), det.ctypes.data, metric.ctypes.data)
    return st, det, metric


@pytest.fixture(scope="module")
def box(pkg):
    from cfd_gb300 import cases
    return cases.box_mesh(shape=(14, 11, 9))


def test_oracle_compact_metrics_match_reference(oracle_mod, box):
    if not oracle_mod.ref_geom_available():
        pytest.skip("reference checkout not present")
    g, _, _ = box
    n = g.shape[0]
    det_o, met_o = np.zeros(n), np.zeros((n, 63))
    det_r, met_r = np.zeros(n), np.zeros((n, 63))
    oracle_mod.compact_metrics(g, det_o, met_o)
    oracle_mod.ref_compact_metrics(g, det_r, met_r)
    assert np.array_equal(det_o[1:], det_r[1:])
    assert np.array_equal(met_o[1:, :9], met_r[1:, :9])


def test_library_compact_metrics_match_oracle(oracle_mod, box):
    from cfd_gb300 import abi
    g, _, _ = box
    n = g.shape[0]
    st, det_l, met_l = _lib_metrics(g)
    assert st == abi.OK
    det_o, met_o = np.zeros(n), np.zeros((n, 63))
    oracle_mod.compact_metrics(g, det_o, met_o)
    assert np.array_equal(det_l[1:], det_o[1:])
    assert np.array_equal(met_l[1:, :9], met_o[1:, :9])


def test_compact_metrics_close_to_analytic(box):
    g, m9, det = box
    st, det_l, met_l = _lib_metrics(g)
    # sixth order inside, lower-order closures at the ends: a loose bound
    assert rel_l2(det_l[1:], det) < 1e-3
    assert rel_l2(met_l[1:, :9], m9) < 1e-3


def test_half_points_match_reference_and_oracle(oracle_mod, box):
    from cfd_gb300 import abi, cases
    g, _, _ = box
    n = g.shape[0]
    st, det, met = _lib_metrics(g)
    # owned rows whose three-deep stencils stay in the box (the reference
    # reads ghost rows at the box edge; the node table here has none)
    owned = n - 1
    lib_met, lib_det = met.copy(), np.zeros((n, 6))
    lib = abi.load()
    assert lib.cfd_half_point_metrics(g.ctypes.data, n, owned, det.ctypes.data, lib_met.ctypes.data,
                                      lib_det.ctypes.data) == abi.OK
    or_met, or_det = met.copy(), np.zeros((n, 6))
    oracle_mod.half_point_metrics(g, owned, det, or_met, or_det)
    assert np.array_equal(lib_met[1:], or_met[1:]) and np.array_equal(lib_det[1:], or_det[1:])
    a = {"grid": g, "metric": met.copy(), "det": det.copy(), "deter": np.zeros((n, 6))}
    cases.half_point_metrics(a, owned)
    assert np.array_equal(a["metric"][1:], or_met[1:]) and np.array_equal(a["deter"][1:], or_det[1:])
    if oracle_mod.ref_geom_available():
        ref_met, ref_det = met.copy(), np.zeros((n, 6))
        oracle_mod.ref_half_point_metrics(g, owned, det, ref_met, ref_det)
        assert np.array_equal(ref_met[1:], or_met[1:]) and np.array_equal(ref_det[1:], or_det[1:])


def test_wake_cut_rows_unsupported_and_short_lines_refused(box):
    from cfd_gb300 import abi, cases
    g, _, _ = box
    g2 = g.copy()
    g2["ID"][5] = 10
    assert _lib_metrics(g2)[0] == abi.EUNSUPPORTED
    gs, _, _ = cases.box_mesh(shape=(2, 6, 6))
    assert _lib_metrics(gs)[0] == abi.EINVAL
