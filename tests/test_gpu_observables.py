"""On-device observables against the oracle restatements:

* vortex-core detection (lib/util/detect_core.m) on the device state: the
  same cores in the same (MATLAB find()) order as oracle.detect_core on the
  same values (FP32 states: the oracle sees the FP32 values), positions to
  1e-12 (cell positions) or 1e-9 (refine_core, closed-form 2x2 generalized
  eigenproblem against LAPACK's), 2D, a 3D slice, a spinor component, caps,
  no cores;
* the Thomas-Fermi guess (lib/@GPEtask/groundstate_tf.m): mu and the state.
"""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu

CORES = [(-2.03, 1.51, 1), (1.27, -0.88, -1), (2.55, 2.14, 1), (-0.61, -2.37, -1), (0.35, 0.42, 1)]


def vortex_field(X, Y, cores, width=2.5):
    phi = np.exp(-(X ** 2 + Y ** 2) / (2 * width ** 2)).astype(complex)
    for xk, yk, sk in cores:
        z = (X - xk) + 1j * sk * (Y - yk)
        phi = phi * z / np.sqrt(1.0 + np.abs(z) ** 2)
    return phi


def as_seen(phi, precision):
    return phi.astype(np.complex64).astype(np.complex128) if precision == "single" else phi


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("refine", [0, 1])
def test_detect_core_2d_matches_oracle(gpe, precision, refine):
    grid = gpe.grid2d(8.0, 64, 7.0, 48, precision=precision)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    og = O.Grid(8.0, 64, 7.0, 48)
    phi = vortex_field(og.mesh["x"], og.mesh["y"], CORES)
    task.init_state = phi
    resp, resm = gpe.detect_core(task, refine=refine)
    op, om = O.detect_core(as_seen(phi, precision), og.mesh["x"], og.mesh["y"], refine=refine)
    assert resp.shape == op.shape == (3, 2) and resm.shape == om.shape == (2, 2)
    tol = 1e-9 if refine else 1e-12
    np.testing.assert_allclose(resp, op, rtol=0, atol=tol)
    np.testing.assert_allclose(resm, om, rtol=0, atol=tol)


def test_detect_core_3d_slice_spinor_component_caps_and_empty(gpe):
    axes = (6.0, 48, 6.0, 32, 3.0, 16)
    grid = gpe.grid3d(*axes, precision="double")
    og = O.Grid(*axes)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    phi = vortex_field(X, Y, CORES[:3]) * np.exp(-Z ** 2)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    task.init_state = phi
    k = 9
    resp, resm = gpe.detect_core(task, z_index=k)
    op, om = O.detect_core(phi[k], X[k], Y[k])
    np.testing.assert_allclose(resp, op, rtol=0, atol=1e-12)
    np.testing.assert_allclose(resm, om, rtol=0, atol=1e-12)
    # caps: the counts come back, the first `cap` entries are written
    import ctypes as C

    from gpe_gb300 import _lib as L

    pos = np.zeros((1, 2))
    neg = np.zeros((1, 2))
    npos, nneg = C.c_int(), C.c_int()
    L.check(task._ctx, L.lib.gpe_detect_core(task._ctx, 0, k, 0, L.dptr(pos), 1, C.byref(npos), L.dptr(neg), 1,
                                             C.byref(nneg)))
    assert (npos.value, nneg.value) == (len(op), len(om))
    np.testing.assert_allclose(pos[0], op[0], atol=1e-12)
    with pytest.raises(gpe.GPEError):
        gpe.detect_core(task, z_index=16)
    # no cores
    task.init_state = np.exp(-(X ** 2 + Y ** 2 + Z ** 2)).astype(complex)
    e1, e2 = gpe.detect_core(task, z_index=k)
    assert e1.shape == (0, 2) and e2.shape == (0, 2)
    # second component of a spinor
    g2 = gpe.grid2d(8.0, 64, 7.0, 48, precision="single")
    sp = gpe.GPEtaskSpinor(g2, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X])
    o2 = O.Grid(8.0, 64, 7.0, 48)
    p2 = vortex_field(o2.mesh["x"], o2.mesh["y"], CORES[1:])
    sp.init_state = [np.exp(-(o2.mesh["x"] ** 2 + o2.mesh["y"] ** 2)).astype(complex), p2]
    rp, rm = gpe.detect_core(sp, component=1)
    op, om = O.detect_core(as_seen(p2, "single"), o2.mesh["x"], o2.mesh["y"])
    np.testing.assert_allclose(rp, op, atol=1e-12)
    np.testing.assert_allclose(rm, om, atol=1e-12)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_groundstate_tf_matches_oracle(gpe, precision):
    axes = (10.0, 64, 9.0, 48)
    grid = gpe.grid2d(*axes, precision=precision)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.4 * Y ** 2)
    task = gpe.GPEtask(grid, V)
    og = O.Grid(*axes)
    ot = O.GPEtask(og, V)
    for t in (task, ot):
        t.Ntotal, t.g = 1e3, 0.3
    phi, mu = task.groundstate_tf(1e-12)
    ophi, omu = ot.groundstate_tf(1e-12)
    assert mu == pytest.approx(omu, rel=1e-12)
    tol = 1e-12 if precision == "double" else 1e-6
    np.testing.assert_allclose(phi, ophi, rtol=0, atol=tol * np.max(ophi))
    # explicit bounds and a particle number (groundstate_tf(eps, N, V, mul, mur))
    phi2, mu2 = task.groundstate_tf(1e-10, 2e3, None, 0.0, 200.0)
    ophi2, omu2 = ot.groundstate_tf(1e-10, 2e3, None, 0.0, 200.0)
    assert mu2 == pytest.approx(omu2, rel=1e-10)
    np.testing.assert_allclose(phi2, ophi2, rtol=0, atol=tol * np.max(ophi2))
    # 'tf' initial state of groundstate_itp (GPEtask.m:147-149) starts from it
    task.g = 0.0
    with pytest.raises(gpe.GPEError):
        task.groundstate_tf(1e-10)
