"""Host logic of the Python mirror (gpe_gb300.task) without a GPU: the calls it
makes into the C ABI are recorded by a fake of the library, so these tests
check what the mirror packs and in which order (parameters, the two
components stacked component after component, the time-dependent potential it
writes into the library's buffer, the omega array, the SGPE parameters, the
vortex-core capacity retry), not any numerics."""
import ctypes as C

import numpy as np
import pytest


class FakeLib:
    """Records every call; answers the few the mirror reads back."""

    def __init__(self, L):
        self.L = L
        self.calls = []
        self.core_counts = (0, 0)

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            if name == "gpe_solve_split" or name == "gpe_solve_sgpe":
                prm = args[1]._obj
                if prm.vtd:
                    n = self.npoints_fill
                    buf = (C.c_double * n)()
                    assert prm.vtd(None, 0.25, buf) == 0
                    self.vtd_values = np.ctypeslib.as_array(buf).copy()
                if prm.on_step:
                    self.step_rc = prm.on_step(None, 1, 0.5, 1.5, 2.5)
            if name in ("gpe_get_history", "gpe_get_history_energy"):
                args[-1]._obj.value = 0
            if name == "gpe_detect_core":
                npos, nneg = self.core_counts
                args[6]._obj.value, args[9]._obj.value = npos, nneg
            return 0
        return call

    def gpe_last_error(self, ctx):
        return b""

    def names(self):
        return [c[0] for c in self.calls]

    def last(self, name):
        return [c for c in self.calls if c[0] == name][-1][1]


@pytest.fixture
def fake(monkeypatch):
    from gpe_gb300 import _lib as L
    from gpe_gb300 import task as T

    f = FakeLib(L)
    monkeypatch.setattr(L, "lib", f)
    monkeypatch.setattr(T.L, "lib", f)
    return f


def test_spinor_states_and_potentials_are_stacked_component_after_component(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8, precision="double")
    t = gpe.GPEtaskSpinor(grid, [lambda X, Y, Z: 0 * X + 1.0, lambda X, Y, Z: 0 * X + 2.0])
    t.g = np.array([[1.0, 0.5], [0.25, 2.0]])
    t.coupling = 0.3 - 0.2j
    t.nlincpl = 0.1
    a = np.full(grid.shape, 1 + 0j)
    b = np.full(grid.shape, 2 + 0j)
    t.init_state = [a, b]
    fake.npoints_fill = 2 * grid.npoints
    t.Vtd = lambda task, time: 10.0 * time + 0 * grid.mesh["x"]
    seen = []
    t.user_callback = lambda task: seen.append(task.current_iter)
    t.solve_split(0.01, 10, 1)
    # the state upload: component 1 then component 2
    st = np.ctypeslib.as_array(C.cast(fake.last("gpe_set_state")[1], C.POINTER(C.c_double)),
                               shape=(4 * grid.npoints,))
    assert np.all(st[: 2 * grid.npoints: 2] == 1.0) and np.all(st[2 * grid.npoints:: 2] == 2.0)
    # Vtd: V1 + vtd then V2 + vtd at time 0.25
    v = fake.vtd_values
    assert np.allclose(v[: grid.npoints], 1.0 + 2.5) and np.allclose(v[grid.npoints:], 2.0 + 2.5)
    # the spinor parameters: g row-major, complex coupling split, nlincpl
    sp = fake.last("gpe_set_spinor_params")[1]._obj
    assert list(sp.g) == [1.0, 0.5, 0.25, 2.0]
    assert (sp.coupling_re, sp.coupling_im, sp.nlincpl) == (0.3, -0.2, 0.1)
    # the scalar g of the one-component parameters is not used by a spinor context
    assert fake.last("gpe_set_params")[1]._obj.g == 0.0
    assert seen == [1]


def test_omega_array_goes_through_set_omega_field(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    t.omega = 0.2 + 0.01 * grid.mesh["x"]
    t.n_crank = 5
    t._push_params()
    args = fake.last("gpe_set_omega_field")
    om = np.ctypeslib.as_array(C.cast(args[1], C.POINTER(C.c_double)), shape=(grid.npoints,))
    assert np.allclose(om, np.ravel(0.2 + 0.01 * grid.mesh["x"])) and args[2] == 5
    assert fake.last("gpe_set_params")[1]._obj.omega == 0.0
    t.omega = 0.35
    t._push_params()
    assert fake.last("gpe_set_omega_field")[1] is None
    assert fake.last("gpe_set_params")[1]._obj.omega == 0.35


def test_sgpe_parameters_and_seed(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.SGPEtask(grid, lambda X, Y, Z: 0 * X)
    t.T, t.ecut, t.seed = 0.7, 12.5, -1  # a negative seed is taken modulo 2^64
    t.init_state = np.ones(grid.shape, complex)
    t.solve_split(0.01, 10, 1)
    sg = fake.last("gpe_solve_sgpe")[2]._obj
    assert (sg.T, sg.ecut, sg.seed) == (0.7, 12.5, 2 ** 64 - 1)


def test_detect_core_grows_its_buffers_to_the_reported_counts(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    t.init_state = np.ones(grid.shape, complex)
    fake.core_counts = (7, 3)
    rp, rm = gpe.detect_core(t, refine=1, z_index=0, cap=4)
    caps = [c[1][5] for c in fake.calls if c[0] == "gpe_detect_core"]
    assert caps == [4, 7] and rp.shape == (7, 2) and rm.shape == (3, 2)
    assert fake.last("gpe_detect_core")[3] == 1  # refine


def test_energy_history_and_itp_outputs_are_sliced_to_the_reported_lengths(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtaskSpinor(grid, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X])
    t.Ntotal = 1.0
    phi, MU, MU2, EE = t.groundstate_itp(0.01, 1e-6, [np.ones(grid.shape, complex)] * 2, nargout=4)
    prm = fake.last("gpe_groundstate_itp")[1]._obj
    assert (prm.want_mu2, prm.want_energy) == (1, 1)
    assert len(MU) == len(MU2) == len(EE) == 0  # the fake reports zero iterations
    assert isinstance(phi, list) and len(phi) == 2


def test_two_component_itp_passes_particle_numbers_and_masses(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtask2comp(grid, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X + 1.0])
    t.g = np.array([[1.0, 0.5], [0.5, 2.0]])
    t.N1, t.N2, t.M1, t.M2, t.Ntotal = 2.0, 3.0, 1.0, 4.0, 5.0
    phi, MU1 = t.groundstate_itp(0.01, 1e-6, [np.ones(grid.shape, complex)] * 2, nargout=2)
    args = fake.last("gpe_groundstate_itp_2comp")
    assert args[2:6] == (2.0, 3.0, 1.0, 4.0)
    assert args[1]._obj.want_energy == 0  # EE is MU2 unless nargout >= 4
    assert "gpe_groundstate_itp" not in fake.names()
    # the coupling of the spinor parameters stays zero
    sp = fake.last("gpe_set_spinor_params")[1]._obj
    assert (sp.coupling_re, sp.coupling_im, sp.nlincpl) == (0.0, 0.0, 0.0)
    t.groundstate_itp(0.01, 1e-6, [np.ones(grid.shape, complex)] * 2, nargout=4)
    assert fake.last("gpe_groundstate_itp_2comp")[1]._obj.want_energy == 1
    t.coupling = 0.1
    with pytest.raises(ValueError):
        t.groundstate_itp(0.01, 1e-6, [np.ones(grid.shape, complex)] * 2)


def test_two_component_observables_and_split_refuse_a_rotating_frame(fake):
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtask2comp(grid, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X])
    t.omega = 0.2
    with pytest.raises(NotImplementedError):
        t.observables([np.ones(grid.shape, complex)] * 2)
    with pytest.raises(NotImplementedError):
        t.solve_split(0.01, 10, 1)
    assert "gpe_observables" not in fake.names() and "gpe_solve_split" not in fake.names()


@pytest.mark.parametrize("cls,stops", [("SGPEtask", 1), ("GPEtask", 0)])
def test_term_from_the_user_callback_stops_only_the_sgpe(fake, cls, stops):
    """SGPEtask.solve_split ends the run when ext_callback returns 'TERM'
    (@SGPEtask/solve_split.m:77-80, SGPEtask.m:33-43); GPEtask ignores the
    callback's result (@GPEtask/solve_split.m:80)."""
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = getattr(gpe, cls)(grid, lambda X, Y, Z: 0 * X)
    t.init_state = np.ones(grid.shape, complex)
    t.user_callback = lambda task: "TERM"
    t.solve_split(0.01, 10, 3)
    assert fake.step_rc == stops


def test_two_component_itp_pushes_a_scalar_omega(fake):
    """The rotating branch of GPEtask2comp.groundstate_itp takes the scalar
    omega through gpe_set_params (no omega array on a two-component context)."""
    import gpe_gb300 as gpe

    grid = gpe.grid2d(4.0, 16, 3.0, 8)
    t = gpe.GPEtask2comp(grid, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X])
    t.N1, t.N2, t.omega = 1.0, 1.0, 0.3
    t.groundstate_itp(0.01, 1e-6, [np.ones(grid.shape, complex)] * 2)
    assert fake.last("gpe_set_params")[1]._obj.omega == 0.3
    assert fake.last("gpe_set_omega_field")[1] is None
    assert fake.names().index("gpe_set_params") < fake.names().index("gpe_groundstate_itp_2comp")
