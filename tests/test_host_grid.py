"""Host-side product code against the oracle, on CPU: the grid mirror
(grid2d/init.m:1-38, grid3d/init.m:1-47: linspace axes, spacing, FFT-ordered
wave numbers, kk, weight, MATLAB memory order), the descriptor it passes to
gpe_create (dx, span), and the vortex imprint of example1_vortex.m:26-30."""
import numpy as np
import pytest

from oracle import gpe_oracle as O


@pytest.mark.parametrize("axes", [(17.0, 64, 12.0, 48), (12.0, 32, 10.0, 24, 8.0, 16)], ids=["2d", "3d"])
def test_grid_mirror_matches_the_oracle_grid(axes):
    import gpe_gb300 as gpe

    g = gpe.grid2d(*axes) if len(axes) == 4 else gpe.grid3d(*axes)
    o = O.Grid(*axes)
    assert g.shape == o.shape and g.weight == o.weight
    for k in ("x", "y"):
        np.testing.assert_array_equal(g.mesh[k], o.mesh[k])
    np.testing.assert_array_equal(g.kx, o.kx1)
    np.testing.assert_array_equal(g.ky, o.ky1)
    np.testing.assert_allclose(g.kk, o.kk, rtol=0, atol=0)
    d = g.desc()
    axes_arr = [g.x, g.y] + ([g.z] if g.ndims == 3 else [])
    for i, a in enumerate(axes_arr):
        assert d.n[i] == a.size and d.dx[i] == a[1] - a[0] and d.span[i] == a[-1] - a[0]
        # init.m:27-28: k = [0:n/2, -(n/2-1):-1] * 2 pi / (span + dx)
        n = a.size
        idx = np.r_[0:n // 2 + 1, -(n // 2 - 1):0]
        np.testing.assert_allclose(g.kx if i == 0 else (g.ky if i == 1 else g.kz),
                                   idx * 2 * np.pi / (d.span[i] + d.dx[i]), rtol=1e-15, atol=0)


def test_vortex_imprint_matches_the_oracle():
    import gpe_gb300 as gpe

    g = gpe.grid2d(17.0, 64, 17.0, 64)
    o = O.Grid(17.0, 64, 17.0, 64)
    X, Y = o.mesh["x"], o.mesh["y"]
    phi = (30 * np.exp(-(X ** 2 + Y ** 2) / 32)).astype(complex)
    a = gpe.imprint_vortex(g, phi, 0.06, 5.0)
    b = O.imprint_vortex(o, phi, 0.06, 5.0)
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)


def test_vortex_ring_imprint_winds_once_around_its_core():
    """imprint_vortex_ring (the 512^3 workload's defect): the phase winds
    once around the ring core in the (x, z) half plane y = 0, x > 0, the amplitude
    vanishes on the core circle and is untouched far from it."""
    import gpe_gb300 as gpe

    g = gpe.grid3d(8.0, 32, 8.0, 32, 8.0, 32)
    phi = np.ones(g.shape, complex)
    R, xi = 4.0, 0.5
    out = gpe.imprint_vortex_ring(g, phi, 1.0, R, xi=xi)
    # the plaquette phase winding of the imprinted state in the y = 0 plane
    # (x > 0 half) is +1 at the core and 0 elsewhere
    iy0 = np.argmin(np.abs(g.y))
    sl = out[:, :, iy0]  # (z, x)
    a, b, c, e = sl[:-1, :-1], sl[:-1, 1:], sl[1:, 1:], sl[1:, :-1]
    w = np.angle(b / a) + np.angle(c / b) + np.angle(e / c) + np.angle(a / e)
    charges = np.rint(w / (2 * np.pi)).astype(int)
    xs = g.x[:-1]
    assert np.sum(np.abs(charges[:, xs > 0])) == 1
    X, Y, Z = g.mesh["x"], g.mesh["y"], g.mesh["z"]
    d = np.sqrt((np.sqrt(X ** 2 + Y ** 2) - R) ** 2 + Z ** 2)
    assert np.all(np.abs(out[d < 0.05 * xi]) < 0.06)
    far = d > 8 * xi
    np.testing.assert_allclose(np.abs(out[far]), 1.0, atol=1e-6)
    # the imprinted phase is atan2(Z, rho - R) (mod 2 pi) wherever the amplitude is not zero
    ph = np.angle(out[far])
    ref = np.arctan2(Z[far], np.sqrt(X[far] ** 2 + Y[far] ** 2) - R)
    np.testing.assert_allclose(np.angle(np.exp(1j * (ph - ref))), 0.0, atol=1e-12)
