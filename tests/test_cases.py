"""Case generators and the oracle's known-answer properties (CPU)."""
from __future__ import annotations

import numpy as np

from helpers import copy_arrays, rel_l2


def test_vortex_neighbour_table_is_periodic_lattice(pkg):
    from cfd_gb300 import cases
    c = cases.isentropic_vortex(n=6, shape=(6, 5, 4))
    g = c.arrays["grid"]
    ni, nj, nk = c.shape
    for r in (1, 7, ni * nj * nk):
        n = r - 1
        i, j, k = n % ni, (n // ni) % nj, n // (ni * nj)
        row = lambda a, b, d: 1 + (a % ni) + ni * ((b % nj) + nj * (d % nk))
        assert g["N1"][r] == row(i + 1, j, k) and g["N3"][r] == row(i - 1, j, k)
        assert g["N0"][r] == row(i, j + 1, k) and g["N2"][r] == row(i, j - 1, k)
        assert g["N4"][r] == row(i, j, k + 1) and g["N5"][r] == row(i, j, k - 1)


def test_tgv_metrics_invert_jacobian(pkg):
    from cfd_gb300 import cases
    c = cases.taylor_green(n=8)
    m = c.arrays["metric"][1:, :9].reshape(-1, 3, 3)
    det = c.arrays["det"][1:]
    assert np.all(det > 0)
    # face metrics interpolate node metrics: close to them for a smooth map
    assert rel_l2(c.arrays["metric"][1:, 9:18], c.arrays["metric"][1:, :9]) < 0.05
    assert np.isfinite(m).all()


def test_free_stream_gives_zero_rhs(oracle_mod):
    """Uniform flow on a Cartesian periodic grid: every flux difference
    vanishes, so L == 0 and the RK step is the identity."""
    from cfd_gb300 import cases
    c = cases.isentropic_vortex(n=8)
    f = c.arrays["flow"]
    f[1:, 0], f[1:, 1], f[1:, 2], f[1:, 3], f[1:, 5] = 0.5, 0.1, -0.2, 1.0, 1.0
    a = copy_arrays(c.arrays)
    L = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, 0, c.dt, want_L=True)
    assert np.abs(L[1:]).max() < 1e-13


def test_axis_permutation_symmetry(oracle_mod):
    """A vortex in the x-y plane and the same vortex rotated into the y-z
    plane give permuted right-hand sides."""
    from cfd_gb300 import cases
    n = 10
    c = cases.isentropic_vortex(n=n)
    a = copy_arrays(c.arrays)
    L1 = oracle_mod.stage(a, c.g_node, c.sd_node, c.params, 0, c.dt, want_L=True)[1:]
    # rotate: (x,y,z) -> (z,x,y): node (i,j,k) of case 2 holds node (j,k,i) of case 1
    c2 = cases.isentropic_vortex(n=n)
    f1 = c.arrays["flow"][1:].reshape(n, n, n, 9)      # [k][j][i]
    f2 = np.transpose(f1, (1, 0, 2, 3))                  # [k2][j2][i2] = f1[j2 idx...]
    # build by explicit index mapping for clarity
    f2 = np.empty_like(f1)
    for k in range(n):
        for j in range(n):
            for i in range(n):
                # case-2 node (i,j,k) <- case-1 node (j,k,i); velocities (u,v,w) -> (w,u,v)
                src = f1[i, k, j]
                dst = src.copy()
                dst[0], dst[1], dst[2] = src[2], src[0], src[1]
                f2[k, j, i] = dst
    c2.arrays["flow"][1:] = f2.reshape(-1, 9)
    a2 = copy_arrays(c2.arrays)
    L2 = oracle_mod.stage(a2, c2.g_node, c2.sd_node, c2.params, 0, c2.dt, want_L=True)[1:]
    L1g = L1.reshape(n, n, n, 5)
    L2g = L2.reshape(n, n, n, 5)
    exp = np.empty_like(L2g)
    for k in range(n):
        for j in range(n):
            for i in range(n):
                s = L1g[i, k, j]
                exp[k, j, i] = [s[0], s[3], s[1], s[2], s[4]]
    assert rel_l2(L2g, exp) < 1e-12


def test_request_stream_is_seeded(pkg):
    """The serving workload generator is deterministic and follows the
    configured distributions (Poisson mean 50/s, n in [32, 160], steps in
    [50, 400])."""
    from cfd_gb300 import serving
    a = serving.poisson_requests(40)
    b = serving.poisson_requests(40)
    assert [(r.arrival, r.n, r.steps, r.kind) for r in a] == [(r.arrival, r.n, r.steps, r.kind) for r in b]
    assert all(32 <= r.n <= 160 and 50 <= r.steps <= 400 for r in a)
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert 0.005 < gaps.mean() < 0.06
    assert {r.kind for r in a} == {"vortex", "tgv"}


def test_tgv_initial_kinetic_energy(pkg):
    """At t = 0 the TGV kinetic energy is 1/8 of rho V0^2 (volume average of
    (sin x cos y cos z)^2 + (cos x sin y cos z)^2 over the box, times 1/2)."""
    from cfd_gb300 import cases, diagnostics
    c = cases.taylor_green(n=32, amp=0.0)
    ke, ens = diagnostics.kinetic_energy_enstrophy(c.arrays["flow"], c.arrays["metric"], c.arrays["det"], c.shape)
    assert abs(ke - 0.125) < 1e-12
    assert abs(ens - 0.375) < 2e-3            # 3/8 for the analytic field, 4th-order differences


def test_naca0012_ogrid_geometry_and_lists(pkg):
    """The O-grid: right-handed and unfolded, owned rows first, wall rows on
    the section (loc 3), far-field rows (loc 1) split upstream/downstream,
    three ghost layers (loc 100) on each side of the wall-normal direction."""
    import numpy as np
    from cfd_gb300 import cases
    c = cases.naca0012(ni=48, nj=16, nk=4)
    g = c.arrays["grid"]
    assert c.shape == (48, 16, 4) and c.sd_node == 48 * 16 * 4 and c.g_node == 48 * 22 * 4
    assert np.all(c.arrays["det"][1:] > 0)
    loc = g["loc"]
    assert np.all(loc[1:c.sd_node + 1] != 100) and np.all(loc[c.sd_node + 1:] == 100)
    assert set(loc[c.bc.wall].tolist()) == {3} and len(c.bc.wall) == 48 * 4
    far = np.concatenate([c.bc.inlet, c.bc.outlet])
    assert set(loc[far].tolist()) == {1} and len(far) == 48 * 4
    assert len(c.bc.inlet) == len(c.bc.outlet)               # upstream half / downstream half
    a = np.radians(1.25)

    def unrotated(rows):   # undo the angle-of-attack rotation about the quarter chord
        x, y = g["x"][rows] - 0.25, g["y"][rows]
        return 0.25 + x * np.cos(a) - y * np.sin(a), x * np.sin(a) + y * np.cos(a)
    assert np.all(unrotated(c.bc.inlet)[0] < 0.5) and np.all(unrotated(c.bc.outlet)[0] >= 0.5)
    x, y = unrotated(c.bc.wall)                               # wall rows lie on the section
    assert np.allclose(np.abs(y), cases.naca0012_thickness(np.clip(x, 0, 1)), atol=1e-12)
