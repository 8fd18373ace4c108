"""GPEtask: the reference's solver class API over libgpe.

Mirrors the public surface of lib/@GPEtask/GPEtask.m (constructor, properties,
getVtotal, groundstate_itp, solve_split, get_energy, the ext_callback
bookkeeping) so scripts written against GPE-MATLAB port line by line.  The
loops themselves (groundstate_itp.m, solve_split.m) run inside libgpe on the
GPU; this class only packs properties, uploads arrays, evaluates host-side
callbacks (time-dependent potential, user callback) and exposes the results.

Differences from the reference, all deliberate:
* ``omega``: a scalar rotating frame (set_kinop.m:5-7, ssft_kin_step.m:12-15)
  and an omega array (the Lz Crank-Nicolson branch, ssft_kin_step.m:3-11)
  both run on the GPU.
* ``'rand'`` initial states use a seeded numpy generator (the reference calls
  an unseeded ``rand``, GPEtask.m:49-52).
* ``show_image`` and the console status line are not implemented (UI).
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np

from . import _lib as L
from .grid import _GridBase


class GPEtask:
    """GPEtask(grid, V) (GPEtask.m:41-60); V is an array or V(X, Y, Z)."""

    def __init__(self, grid: _GridBase, trappot, device: int = 0):
        self.grid = grid
        self._ctx = C.c_void_p()
        L.check(None, L.lib.gpe_create(C.byref(grid.desc(device)), C.byref(self._ctx)))
        # public properties with the reference defaults (GPEtask.m:4-34)
        self.g = 0.0
        self.omega = 0.0
        self.n_crank = 3
        self.n_recalc = 10
        self.gamma = 0.0
        self.decay_rate = 0.0
        self.Ntotal = 0.0
        self.mu_init = 0.0
        self.Vtd = None
        self.V0 = 0
        self.user_callback = None
        self.itp_max_iter = 5000
        self.itp_min_iter = 50
        self.itp_adjust_stepsize = False
        self.fp64_polish = True      # FP32 grids: finish ITP in FP64 once FP32 stalls
        self.history = {"mu": np.zeros(0), "n": np.zeros(0)}
        self.current_time = 0.0
        self.current_iter = 0
        self.current_mu = 0.0
        self.current_n = 0.0
        self.init_state = np.zeros(grid.shape, dtype=np.complex128)
        self._current_state = None
        self._state_on_device = None     # 'current' when the device holds current_state
        self._V_key = None
        if callable(trappot):
            V = trappot(grid.mesh["x"], grid.mesh["y"], grid.mesh["z"])
        else:
            V = trappot
        self.Vtrap = np.broadcast_to(np.asarray(V, dtype=np.float64), grid.shape).copy()
        self.last_itp = None

    # ---- lifetime ----------------------------------------------------------
    def close(self):
        if self._ctx:
            L.lib.gpe_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- properties ---------------------------------------------------------
    @property
    def Vtrap(self):
        return self._Vtrap

    @Vtrap.setter
    def Vtrap(self, v):
        self._Vtrap = np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), self.grid.shape))
        self._V_key = None

    @property
    def current_state(self):
        if self._state_on_device == "current" and self._current_state is None:
            self._current_state = self._download()
        return self._current_state

    @current_state.setter
    def current_state(self, v):
        self._current_state = None if v is None else np.asarray(v, dtype=np.complex128)
        self._state_on_device = None

    def _push_params(self):
        p = L.gpe_params()
        if np.size(self.omega) != 1:
            # array omega: the Lz Crank-Nicolson branch (ssft_kin_step.m:3-11)
            om = np.ascontiguousarray(np.broadcast_to(np.asarray(self.omega, dtype=np.float64), self.grid.shape))
            L.check(self._ctx, L.lib.gpe_set_omega_field(self._ctx, L.dptr(om), int(self.n_crank)))
            p.omega = 0.0
        else:
            L.check(self._ctx, L.lib.gpe_set_omega_field(self._ctx, None, int(self.n_crank)))
            p.omega = float(np.asarray(self.omega).ravel()[0])
        p.g = self._g_scalar()
        p.gamma = float(self.gamma)
        p.decay_rate = float(self.decay_rate)
        p.Ntotal = float(self.Ntotal)
        p.mu_init = float(self.mu_init)
        p.n_recalc = int(self.n_recalc)
        p.itp_max_iter = int(self.itp_max_iter)
        p.itp_min_iter = int(self.itp_min_iter)
        p.itp_adjust_stepsize = int(bool(self.itp_adjust_stepsize))
        L.check(self._ctx, L.lib.gpe_set_params(self._ctx, C.byref(p)))
        cur = L.gpe_current()
        cur.current_iter = int(self.current_iter)
        cur.current_time = float(self.current_time)
        cur.current_mu = float(self.current_mu)
        cur.current_n = float(self.current_n)
        L.check(self._ctx, L.lib.gpe_set_current(self._ctx, C.byref(cur)))

    def _g_scalar(self):
        return float(self.g)

    def _upload_V(self, V):
        key = (id(V), V.ctypes.data)
        if key == self._V_key:
            return
        V = np.ascontiguousarray(V, dtype=np.float64)
        L.check(self._ctx, L.lib.gpe_set_potential(self._ctx, L.dptr(V)))
        self._V_key = (id(V), V.ctypes.data)
        self._V_keep = V

    def _upload_state(self, phi):
        phi = np.broadcast_to(phi, self.grid.shape)
        if phi.dtype == np.complex64:  # single-precision host arrays go as they are
            phi = np.ascontiguousarray(phi)
            L.check(self._ctx, L.lib.gpe_set_state_f32(self._ctx, L.fptr(phi.view(np.float32))))
            return
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        L.check(self._ctx, L.lib.gpe_set_state(self._ctx, L.dptr(phi.view(np.float64))))

    def _download(self, out=None):
        """The device state as a host array: complex64 on single-precision
        grids, complex128 otherwise (or into `out`, e.g. a pinned buffer)."""
        if out is None:
            dt = np.complex64 if self.grid.precision == "single" else np.complex128
            out = np.empty(self.grid.shape, dtype=dt)
        if out.dtype == np.complex64:
            L.check(self._ctx, L.lib.gpe_get_state_f32(self._ctx, L.fptr(out.view(np.float32))))
        else:
            L.check(self._ctx, L.lib.gpe_get_state(self._ctx, L.dptr(out.view(np.float64))))
        return out

    # ---- GPEtask.m methods ---------------------------------------------------
    def getVtotal(self, time):
        """GPEtask.m:62-71."""
        if time == 0 and np.size(self.V0) > 1:
            return np.broadcast_to(np.asarray(self.V0, dtype=np.float64), self.grid.shape)
        if callable(self.Vtd):
            return self.Vtrap + self.Vtd(self, time)
        return self.Vtrap

    def _time_dependent(self):
        return callable(self.Vtd) or np.size(self.V0) > 1

    def process_init_state(self, phi0, rng=None):
        """GPEtask.m:144-164 for string arguments; arrays are normalised on the
        device by groundstate_itp."""
        if isinstance(phi0, str):
            if self.Ntotal > 0:
                if phi0 == "tf":
                    return self.groundstate_tf(np.finfo(float).eps)[0].astype(np.complex128)
                rng = rng or np.random.default_rng()
                r = rng.random(self.grid.shape) + 1j * rng.random(self.grid.shape)
                return math.sqrt(self.Ntotal) * self.grid.normalize(r)
            V = self.getVtotal(0)
            return np.real(np.sqrt((self.mu_init - V).astype(np.complex128) / self.g)).astype(np.complex128)
        return np.asarray(phi0, dtype=np.complex128)

    def groundstate_tf(self, eps, N=None, V=None, mul=None, mur=None):
        """Thomas-Fermi state and mu, lib/@GPEtask/groundstate_tf.m:1-37, on the
        device (gpe_groundstate_tf): bisection against getVtotal(0) (or V),
        phi = sqrt(vvv/g).  Returns (phi, mu); the device state holds phi."""
        N = self.Ntotal if N is None else N
        self._push_params()
        self._upload_V(np.ascontiguousarray(self.getVtotal(0) if V is None else
                                            np.broadcast_to(np.asarray(V, dtype=np.float64), self.grid.shape)))
        bounds = None
        if mul is not None:
            bounds = np.array([float(mul), float(mur)])
        mu = C.c_double()
        L.check(self._ctx, L.lib.gpe_groundstate_tf(self._ctx, float(eps), float(N),
                                                    None if bounds is None else L.dptr(bounds), C.byref(mu)))
        if V is not None:
            self._V_key = None  # the next call uploads its own potential again
        phi = np.real(self._download())
        self._state_on_device = None
        return phi, mu.value

    def detect_core(self, refine=0, z_index=0, component=0, cap=4096):
        """lib/util/detect_core.m on the current device state (slice z_index of
        a 3D grid): (resp, resm), k x 2 arrays of [x, y]."""
        return detect_core(self, refine=refine, z_index=z_index, component=component, cap=cap)

    def groundstate_itp(self, dt, eps, phi0="rand", nargout=1, rng=None):
        """groundstate_itp.m:1-112.  Returns phi, or (phi, MU, MU2, EE)[:nargout].
        ``last_itp`` then holds the run's gpe_itp_result: iterations, the FP32
        iterations before an FP64 polish, and the device time of each phase
        (ms_main, ms_fp64)."""
        self._push_params()
        self._upload_V(np.ascontiguousarray(self.getVtotal(0)))
        phi = self.process_init_state(phi0, rng=rng)
        self._upload_state(phi)
        prm = L.gpe_itp_params()
        prm.dt = float(dt)
        prm.eps = float(eps)
        prm.want_mu2 = int(nargout >= 3)
        prm.want_energy = int(nargout >= 4)
        prm.fp64_polish = int(bool(self.fp64_polish))
        prm.switch_delta = 0.0
        cap = int(self.itp_max_iter)
        MU = np.zeros(cap)
        MU2 = np.zeros(cap)
        EE = np.zeros(cap)
        res = L.gpe_itp_result()
        L.check(self._ctx, L.lib.gpe_groundstate_itp(self._ctx, C.byref(prm), L.dptr(MU), L.dptr(MU2),
                                                     L.dptr(EE), cap, C.byref(res)))
        n = res.iters
        self.last_itp = res
        if not res.converged:
            warnings.warn("Convergence not reached")  # groundstate_itp.m:79
        cur = L.gpe_current()
        L.check(self._ctx, L.lib.gpe_get_current(self._ctx, C.byref(cur)))
        if nargout >= 2 or self.Ntotal <= 0:
            self.current_mu, self.current_n = cur.current_mu, cur.current_n
        phi = self._download()
        self.init_state = phi                      # groundstate_itp.m:111
        self._current_state = phi
        self._state_on_device = "current"
        outs = (phi, MU[:n].copy(), MU2[:n].copy(), EE[:n].copy())
        return phi if nargout <= 1 else outs[:nargout]

    def _prepare_split(self):
        """Parameters and the start state on the device (solve_split.m:29,34-38)."""
        self._push_params()
        start = int(self.current_iter)
        if start > 0:
            if self._state_on_device != "current":
                if self._current_state is None:
                    raise RuntimeError("current_iter > 0 but no current_state")
                self._upload_state(self._current_state)
        else:
            self._upload_state(self.init_state)

    def _after_split(self):
        cur = L.gpe_current()
        L.check(self._ctx, L.lib.gpe_get_current(self._ctx, C.byref(cur)))
        self.current_iter, self.current_time = cur.current_iter, cur.current_time
        self.current_mu, self.current_n = cur.current_mu, cur.current_n
        self._sync_history()
        self._current_state = None
        self._state_on_device = "current"

    def solve_split(self, ddt, niter_inner, niter_outer):
        """solve_split.m:1-84: run outer steps current_iter+1 .. niter_outer."""
        return self._run_split(ddt, niter_inner, niter_outer, None)

    def _run_split(self, ddt, niter_inner, niter_outer, sgpe):
        """The shared driver of solve_split and SGPEtask.solve_split (sgpe:
        a gpe_sgpe_params, or None)."""
        self._prepare_split()
        errors = []
        vtd_cb = L.VTD_FN()
        if self._time_dependent():

            def _vtd(user, time, out):
                try:
                    self._vtd_fill(time, out)
                    return 0
                except BaseException as e:  # surfaced after the call returns
                    errors.append(e)
                    return 1

            vtd_cb = L.VTD_FN(_vtd)
            self._V_key = None
        else:
            self._upload_V(self.Vtrap)

        def _step(user, step, time, mu, n):
            try:
                return 1 if self._ext_callback(step, time, mu, n) else 0  # nonzero: end the run here
            except BaseException as e:
                errors.append(e)
                return 1

        step_cb = L.STEP_FN(_step) if self.user_callback is not None else L.STEP_FN()
        prm = L.gpe_split_params()
        prm.ddt = float(ddt)
        prm.niter_inner = int(niter_inner)
        prm.niter_outer = int(niter_outer)
        prm.vtd = vtd_cb
        prm.on_step = step_cb
        if sgpe is None:
            st = L.lib.gpe_solve_split(self._ctx, C.byref(prm))
        else:
            st = L.lib.gpe_solve_sgpe(self._ctx, C.byref(prm), C.byref(sgpe))
        if errors:
            raise errors[0]
        L.check(self._ctx, st)
        self._after_split()
        return self.current_state

    def _vtd_fill(self, time, out):
        """getVtotal(time) into the library's buffer (P doubles)."""
        v = np.asarray(self.getVtotal(time), dtype=np.float64)
        np.ctypeslib.as_array(out, shape=(self.grid.npoints,))[:] = np.broadcast_to(v, self.grid.shape).ravel()

    def _sync_history(self):
        n = C.c_int()
        L.check(self._ctx, L.lib.gpe_get_history(self._ctx, None, None, 0, C.byref(n)))
        mu = np.zeros(n.value)
        nn = np.zeros(n.value)
        ee = np.zeros(n.value)
        L.check(self._ctx, L.lib.gpe_get_history(self._ctx, L.dptr(mu), L.dptr(nn), n.value, C.byref(n)))
        L.check(self._ctx, L.lib.gpe_get_history_energy(self._ctx, L.dptr(ee), n.value, C.byref(n)))
        # "energy" is an addition (get_energy at every outer step, on the device)
        self.history["mu"], self.history["n"], self.history["energy"] = mu, nn, ee

    def _ext_callback(self, step, time, mu, n):
        """GPEtask.m:115-142 (plot and console line omitted).  Returns True to
        end the run after this outer step; GPEtask.solve_split ignores the
        callback's result (solve_split.m:80)."""
        self.current_time = time
        self.current_iter = step
        self.current_mu = mu
        self.current_n = n
        self._current_state = None
        self._state_on_device = "current"
        self._sync_history()
        if callable(self.user_callback):
            self.user_callback(self)
        return False

    def observables(self, phi=None):
        """<psi|H psi> pieces of psi (default: the current device state)."""
        self._push_params()
        self._upload_V(np.ascontiguousarray(self.getVtotal(self.current_time)))
        if phi is not None:
            self._upload_state(phi)
            self._state_on_device = None
        o = L.gpe_obs()
        L.check(self._ctx, L.lib.gpe_observables(self._ctx, C.byref(o)))
        return {k: getattr(o, k) for k, _ in L.gpe_obs._fields_}

    def get_energy(self, phi=None):
        """GPEtask.m:97-107."""
        return self.observables(phi if phi is not None else self.current_state)["energy"]

    def chemical_potential_integral(self, phi=None):
        """real(inner(phi, applyham(phi))) (GPEtask.m:73-78 with grid.inner)."""
        return self.observables(phi if phi is not None else self.current_state)["mu_integral"]

    # ---- gradient ------------------------------------------------------------
    def adjoint_grad(self, psi_target, ddt, nsteps, phi0=None, V=None, checkpoint_every=0, mem_budget=0.0,
                     precision=None):
        """dloss/dV through `nsteps` gamma = 0 split steps of ddt from phi0
        (default init_state) in the static potential V (default Vtrap), with
        loss = 1 - |<target|psi(T)>|^2 / (<target|target> <phi0|phi0>).

        Returns (loss, dLdV): dLdV[i] is the derivative with respect to the
        potential's value at grid point i (same shape as the grid).  The
        derivative with respect to a parameter a of V(x; a) is
        sum(dLdV * dV/da), see ``project_gradient``.  precision "double" on a
        single-precision grid runs the sweep in FP64 from the FP32 state."""
        self._push_params()
        V = self.Vtrap if V is None else V
        self._upload_V(np.ascontiguousarray(np.broadcast_to(np.asarray(V, dtype=np.float64), self.grid.shape)))
        self._upload_state(self.init_state if phi0 is None else phi0)
        self._state_on_device = None
        tgt = np.ascontiguousarray(np.broadcast_to(psi_target, self.grid.shape), dtype=np.complex128)
        prm = L.gpe_adjoint_params()
        prm.ddt = float(ddt)
        prm.nsteps = int(nsteps)
        prm.checkpoint_every = int(checkpoint_every)
        prm.mem_budget = float(mem_budget)
        prm.precision = {None: 0, "single": L.GPE_FP32, "double": L.GPE_FP64}[precision]
        dLdV = np.zeros(self.grid.shape)
        loss = C.c_double()
        L.check(self._ctx, L.lib.gpe_adjoint_grad(self._ctx, C.byref(prm), L.dptr(tgt.view(np.float64)),
                                                  L.dptr(dLdV), C.byref(loss)))
        return loss.value, dLdV

    @staticmethod
    def project_gradient(dLdV, basis):
        """dloss/da_j = sum_i dLdV[i] * basis[j][i] for V = V_0 + sum_j a_j basis[j]."""
        return np.array([float(np.sum(dLdV * b)) for b in basis])

    # ---- profiling -----------------------------------------------------------
    def profile(self, on: bool = True):
        L.check(self._ctx, L.lib.gpe_profile_enable(self._ctx, int(on)))

    def profile_read(self):
        cap = 32
        arr = (L.gpe_kernel_stat * cap)()
        n = C.c_int()
        L.check(self._ctx, L.lib.gpe_profile_read(self._ctx, arr, cap, C.byref(n)))
        return [{"name": arr[i].name.decode(), "launches": arr[i].launches, "total_ms": arr[i].total_ms,
                 "bytes_per_launch": arr[i].bytes_per_launch} for i in range(n.value)]

    def kernel_launches(self) -> int:
        return int(L.lib.gpe_kernel_launches(self._ctx))

    def autotune(self, mode: int = 1):
        """FFT plan autotuner (gpe_autotune): 0 default plans, 1 tune now,
        2 automatic (default), 3 alternative plans, 4 / 5 paired passes on
        the alternative / default plans, 16 + m, 32 + m, 48 + m the same on
        the axes of bit mask m.  Returns the plan variant per axis (x, y, z:
        0 default, 1 alternative, 2 paired alternative, 3 paired default);
        -1 where an axis has a single plan."""
        ch = (C.c_int * 3)()
        L.check(self._ctx, L.lib.gpe_autotune(self._ctx, int(mode), ch))
        return tuple(ch)

    def set_pass_variant(self, variant: int):
        """0: direct passes with L2 prefetch (default), 1: TMA-staged passes where
        they apply, 2: direct passes without prefetch."""
        L.check(self._ctx, L.lib.gpe_set_pass_variant(self._ctx, int(variant)))


class SGPEtask(GPEtask):
    """SGPEtask (lib/@SGPEtask/SGPEtask.m:1-48): GPEtask with temperature T,
    noise cut-off ecut and (an addition) the noise seed.  solve_split runs
    SGPEtask.solve_split on the GPU: mu = mu_init, no renormalisation, noise
    sqrt(T*gamma*ddt/weight)*(n1 + 1i*n2) before every kinetic step."""

    def __init__(self, grid: _GridBase, trappot, device: int = 0):
        super().__init__(grid, trappot, device=device)
        self.T = 0.0
        self.ecut = 0.0
        self.seed = 0

    def _ext_callback(self, step, time, mu, n):
        """SGPEtask.m:20-44: as GPEtask's, and a user_callback that returns
        'TERM' ends the run after this outer step (solve_split.m:77-80)."""
        self.current_time = time
        self.current_iter = step
        self.current_mu = mu
        self.current_n = n
        self._current_state = None
        self._state_on_device = "current"
        self._sync_history()
        res = self.user_callback(self) if callable(self.user_callback) else None
        return isinstance(res, str) and res == "TERM"

    def solve_split(self, ddt, niter_inner, niter_outer):
        """lib/@SGPEtask/solve_split.m:1-81."""
        sg = L.gpe_sgpe_params()
        sg.T = float(self.T)
        sg.ecut = float(self.ecut)
        sg.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return self._run_split(ddt, niter_inner, niter_outer, sg)


class GPEtaskSpinor(GPEtask):
    """GPEtaskSpinor(grid, {V1, V2}) (lib/@GPEtaskSpinor/GPEtaskSpinor.m:1-147):
    two coherently coupled components.  ``trappot`` is a pair of arrays or
    V(X, Y, Z) callables; ``g`` a 2x2 matrix; ``coupling`` the (complex) Rabi
    coupling, ``nlincpl`` its density-dependent part.  States are pairs
    [phi1, phi2].  solve_split runs GPEtaskSpinor.solve_split on the GPU
    (one context holding both components); ``Vtd`` is a callable added to
    both potentials or a pair of callables (GPEtaskSpinor.m:23-42).
    groundstate_itp is the spinor's own (groundstate_itp.m, with its rotating
    branch for a scalar omega on 2D grids); solve_split and the observables
    take a scalar omega as GPEtaskSpinor does (plain kinetic step, -omega lz
    in mu and the energies)."""

    def __init__(self, grid: _GridBase, trappot, device: int = 0):
        self.grid = grid
        self._ctx = C.c_void_p()
        L.check(None, L.lib.gpe_create_spinor(C.byref(grid.desc(device)), C.byref(self._ctx)))
        self.g = np.zeros((2, 2))
        self.coupling = 0.0
        self.nlincpl = 0.0
        self.ncomp = 2
        self.omega = 0.0
        self.n_crank = 3
        self.n_recalc = 10
        self.gamma = 0.0
        self.decay_rate = 0.0
        self.Ntotal = 0.0
        self.mu_init = 0.0
        self.Vtd = None
        self.V0 = 0
        self.user_callback = None
        self.itp_max_iter = 500000  # the spinor ITP's own cap (groundstate_itp.m:123)
        self.itp_min_iter = 50
        self.itp_adjust_stepsize = False
        self.last_itp = None
        self.history = {"mu": np.zeros(0), "n": np.zeros(0)}
        self.current_time = 0.0
        self.current_iter = 0
        self.current_mu = 0.0
        self.current_n = 0.0
        self.init_state = [np.zeros(grid.shape, np.complex128), np.zeros(grid.shape, np.complex128)]
        self._current_state = None
        self._state_on_device = None
        self._V_key = None
        if len(trappot) != 2:
            raise ValueError("GPEtaskSpinor: two trap potentials (one per component)")
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        self.Vtrap = [f(X, Y, Z) if callable(f) else f for f in trappot]

    @property
    def Vtrap(self):
        return self._Vtrap

    @Vtrap.setter
    def Vtrap(self, v):
        self._Vtrap = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), self.grid.shape))
                       for x in v]
        self._V_key = None

    @property
    def current_state(self):
        if self._state_on_device == "current" and self._current_state is None:
            self._current_state = self._download()
        return self._current_state

    @current_state.setter
    def current_state(self, v):
        self._current_state = None if v is None else [np.asarray(x, dtype=np.complex128) for x in v]
        self._state_on_device = None

    def _g_scalar(self):
        return 0.0  # the matrix goes through gpe_set_spinor_params

    def _push_params(self):
        super()._push_params()
        p = L.gpe_spinor_params()
        g = np.broadcast_to(np.asarray(self.g, dtype=np.float64), (2, 2))
        for k in range(4):
            p.g[k] = float(g[k // 2, k % 2])
        cpl = complex(self.coupling)
        p.coupling_re, p.coupling_im = cpl.real, cpl.imag
        p.nlincpl = float(self.nlincpl)
        L.check(self._ctx, L.lib.gpe_set_spinor_params(self._ctx, C.byref(p)))

    def _pair(self, v, dtype):
        return np.ascontiguousarray(np.concatenate([np.broadcast_to(np.asarray(x), self.grid.shape).ravel()
                                                    for x in v]), dtype=dtype)

    def _upload_V(self, V):
        key = tuple((id(x), x.ctypes.data) for x in V)
        if key == self._V_key:
            return
        flat = self._pair(V, np.float64)
        L.check(self._ctx, L.lib.gpe_set_potential(self._ctx, L.dptr(flat)))
        self._V_key = key
        self._V_keep = V

    def _upload_state(self, phi):
        """A pair [phi1, phi2], or one contiguous array of both components
        (2*npoints values, e.g. a pinned host buffer), uploaded as it is."""
        n = self.grid.npoints
        if isinstance(phi, np.ndarray) and phi.size == 2 * n and phi.flags.c_contiguous and \
                phi.dtype in (np.complex64, np.complex128):
            flat = phi
        else:
            flat = self._pair(phi, np.complex128)
        if flat.dtype == np.complex64:
            L.check(self._ctx, L.lib.gpe_set_state_f32(self._ctx, L.fptr(flat.view(np.float32))))
        else:
            L.check(self._ctx, L.lib.gpe_set_state(self._ctx, L.dptr(flat.view(np.float64))))

    def _download(self, out=None):
        """[phi1, phi2], or both components into `out` (2*npoints values)."""
        n = self.grid.npoints
        if out is None:
            dt = np.complex64 if self.grid.precision == "single" else np.complex128
            flat = np.empty(2 * n, dtype=dt)
        else:
            flat = out
        if flat.dtype == np.complex64:
            L.check(self._ctx, L.lib.gpe_get_state_f32(self._ctx, L.fptr(flat.view(np.float32))))
        else:
            L.check(self._ctx, L.lib.gpe_get_state(self._ctx, L.dptr(flat.view(np.float64))))
        if out is not None:
            return out
        return [flat[:n].reshape(self.grid.shape), flat[n:].reshape(self.grid.shape)]

    def getVtotal(self, time):
        """GPEtaskSpinor.m:23-42 (the internal V0 branch is not mirrored)."""
        if callable(self.Vtd):
            return [V + self.Vtd(self, time) for V in self.Vtrap]
        if isinstance(self.Vtd, (list, tuple)):
            return [V + f(self, time) for V, f in zip(self.Vtrap, self.Vtd)]
        return self.Vtrap

    def _time_dependent(self):
        return self.Vtd is not None

    def _vtd_fill(self, time, out):
        P = self.grid.npoints
        V = self.getVtotal(time)
        arr = np.ctypeslib.as_array(out, shape=(2 * P,))
        for k in range(2):
            arr[k * P:(k + 1) * P] = np.broadcast_to(np.asarray(V[k], dtype=np.float64), self.grid.shape).ravel()

    def groundstate_itp(self, dt, eps, phi0=None, nargout=1, rng=None):
        """lib/@GPEtaskSpinor/groundstate_itp.m:1-145 on the GPU.  phi0: a pair, or
        None for the reference's random start (normalised uniform complex noise
        per component / sqrt(2), seeded here).  Returns phi, or (phi, MU, MU2,
        EE)[:nargout]; MU2/EE are evaluated when nargout asks for them (the
        convergence test then uses them, as in the reference)."""
        self._push_params()
        self._upload_V(self.getVtotal(0))
        if phi0 is None:
            rng = rng or np.random.default_rng()
            phi0 = [self.grid.normalize(rng.random(self.grid.shape) + 1j * rng.random(self.grid.shape)) / math.sqrt(2)
                    for _ in range(2)]
        self._upload_state(phi0)
        prm = L.gpe_itp_params()
        prm.dt = float(dt)
        prm.eps = float(eps)
        prm.want_mu2 = int(nargout >= 3)
        prm.want_energy = int(nargout >= 4)
        cap = int(self.itp_max_iter)
        MU, MU2, EE = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        res = L.gpe_itp_result()
        L.check(self._ctx, L.lib.gpe_groundstate_itp(self._ctx, C.byref(prm), L.dptr(MU), L.dptr(MU2),
                                                     L.dptr(EE), cap, C.byref(res)))
        if not res.converged:
            warnings.warn("Convergence not reached")
        self.last_itp = res
        n = res.iters
        phi = self._download()
        self.init_state = phi
        self._current_state = phi
        self._state_on_device = "current"
        outs = (phi, MU[:n].copy(), MU2[:n].copy(), EE[:n].copy())
        return phi if nargout <= 1 else outs[:nargout]

    def observables(self, phi=None):
        """<psi|H psi> pieces of the pair (default: the current device state),
        V at current_time (GPEtaskSpinor.applyham)."""
        self._push_params()
        self._upload_V(self.getVtotal(self.current_time))
        if phi is not None:
            self._upload_state(phi)
            self._state_on_device = None
        o = L.gpe_obs()
        L.check(self._ctx, L.lib.gpe_observables(self._ctx, C.byref(o)))
        return {k: getattr(o, k) for k, _ in L.gpe_obs._fields_}

    def get_energy(self, phi=None):
        """GPEtaskSpinor.m:98-110."""
        return self.observables(phi if phi is not None else self.current_state)["energy"]


class GPEtask2comp(GPEtaskSpinor):
    """GPEtask2comp(grid, {V1, V2}) (lib/@GPEtask2comp/GPEtask2comp.m:1-150): an
    incoherent two-component mixture.  ``g`` is a 2x2 matrix, ``N1``/``N2`` the
    particle numbers and ``M1``/``M2`` the masses of the components.
    groundstate_itp is the class's own (groundstate_itp.m: each component with
    its own kinetic factor exp(-kk dt/2/M_j) and its own normalisation N_j);
    solve_split, get_energy and observables are GPEtaskSpinor's with coupling =
    nlincpl = 0, which is what @GPEtask2comp/solve_split.m and
    GPEtask2comp.m:41-118 compute (that class declares no coupling)."""

    def __init__(self, grid: _GridBase, trappot, device: int = 0):
        super().__init__(grid, trappot, device)
        self.N1 = 0.0
        self.N2 = 0.0
        self.M1 = 1.0
        self.M2 = 1.0

    def _plain_frame_only(self, what):
        if np.size(self.omega) != 1 or float(np.asarray(self.omega).ravel()[0]) != 0.0:
            raise NotImplementedError(
                f"GPEtask2comp.{what} with omega != 0: its applyham takes lap(phi, omega) (GPEtask2comp.m:60), "
                "which the library evaluates only inside groundstate_itp")

    def solve_split(self, ddt, niter_inner, niter_outer):
        self._plain_frame_only("solve_split")
        return super().solve_split(ddt, niter_inner, niter_outer)

    def observables(self, phi=None):
        self._plain_frame_only("observables")
        return super().observables(phi)

    def groundstate_itp(self, dt, eps, phi0=None, nargout=1, rng=None):
        """lib/@GPEtask2comp/groundstate_itp.m:1-157 on the GPU (a scalar
        omega on 2D grids takes the reference's rotating branch).
        phi0: a pair, or None for the reference's random start.  Returns phi,
        or (phi, MU1, MU2, EE)[:nargout]: MU_j(i) = log(sqrt(N_j/n_j))/dt of
        each component; EE = get_energy/Ntotal when nargout >= 4 (else MU2,
        which the convergence test then uses, :98-102)."""
        if self.coupling != 0 or self.nlincpl != 0:
            raise ValueError("GPEtask2comp: an incoherent mixture has coupling = nlincpl = 0")
        self._push_params()
        self._upload_V(self.getVtotal(0))
        if phi0 is None:
            rng = rng or np.random.default_rng()
            phi0 = [self.grid.normalize(rng.random(self.grid.shape) + 1j * rng.random(self.grid.shape)) / math.sqrt(2)
                    for _ in range(2)]
        self._upload_state(phi0)
        prm = L.gpe_itp_params()
        prm.dt = float(dt)
        prm.eps = float(eps)
        prm.want_energy = int(nargout >= 4)
        cap = int(self.itp_max_iter)
        MU1, MU2, EE = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        res = L.gpe_itp_result()
        L.check(self._ctx, L.lib.gpe_groundstate_itp_2comp(
            self._ctx, C.byref(prm), float(self.N1), float(self.N2), float(self.M1), float(self.M2),
            L.dptr(MU1), L.dptr(MU2), L.dptr(EE), cap, C.byref(res)))
        if not res.converged:
            warnings.warn("Convergence not reached")
        self.last_itp = res
        n = res.iters
        phi = self._download()
        self.init_state = phi
        self._current_state = phi
        self._state_on_device = "current"
        outs = (phi, MU1[:n].copy(), MU2[:n].copy(), EE[:n].copy())
        return phi if nargout <= 1 else outs[:nargout]


def detect_core(task, refine=0, z_index=0, component=0, cap=4096):
    """detect_core(phi, rx, ry, refine) (lib/util/detect_core.m:1-67) of the
    task's current device state, on the device (gpe_detect_core): (resp,
    resm), k x 2 arrays of the positive and negative cores' [x, y] in MATLAB's
    find() order.  3D grids: the slice z_index; spinor tasks: `component`."""
    if task._state_on_device != "current":
        st = task._current_state if task._current_state is not None else task.init_state
        task._upload_state(st)
    while True:
        pos = np.zeros((cap, 2))
        neg = np.zeros((cap, 2))
        npos, nneg = C.c_int(), C.c_int()
        L.check(task._ctx, L.lib.gpe_detect_core(task._ctx, int(component), int(z_index), int(refine),
                                                 L.dptr(pos), cap, C.byref(npos), L.dptr(neg), cap,
                                                 C.byref(nneg)))
        if npos.value <= cap and nneg.value <= cap:
            return pos[:npos.value].copy(), neg[:nneg.value].copy()
        cap = max(npos.value, nneg.value)


def noise_variates(seed, step, n):
    """The stochastic GPE's noise for points 0..n-1 of `step` (device FP32):
    an (n, 2) array of standard normal pairs (gpe_selftest_noise)."""
    out = np.empty(2 * int(n), dtype=np.float32)
    L.check(None, L.lib.gpe_selftest_noise(int(seed), int(step), int(n), L.fptr(out)))
    return out.reshape(-1, 2)


def solve_split_batch(tasks, ddt, niter_inner, niter_outer):
    """solve_split(ddt, niter_inner, niter_outer) of many independent GPEtask
    objects at once, through gpe_solve_split_batch: grids of any sizes, one
    CUDA graph per block of n_recalc steps with the tasks' chains running
    concurrently.  Each task keeps its own properties, state, history and
    current_*.  Tasks need static potentials (no Vtd / V0), no user_callback,
    no decay, the same n_recalc and the same current_iter."""
    tasks = list(tasks)
    if not tasks:
        return
    for t in tasks:
        if t._time_dependent() or t.user_callback is not None:
            raise ValueError("solve_split_batch: tasks need a static potential and no user_callback")
        t._prepare_split()
        t._upload_V(t.Vtrap)
    arr = (C.c_void_p * len(tasks))(*[t._ctx.value for t in tasks])
    prm = L.gpe_split_params()
    prm.ddt = float(ddt)
    prm.niter_inner = int(niter_inner)
    prm.niter_outer = int(niter_outer)
    L.check(tasks[0]._ctx, L.lib.gpe_solve_split_batch(arr, len(tasks), C.byref(prm)))
    for t in tasks:
        t._after_split()
