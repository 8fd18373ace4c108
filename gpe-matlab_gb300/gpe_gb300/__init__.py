"""gpe_gb300: GPE-MATLAB's split-step hot path on GB300 (sm_103a).

Host mirror of the reference's MATLAB class API over libgpe.so:

    from gpe_gb300 import grid2d, GPEtask
    grid = grid2d(17, 256, 17, 256, precision='single')
    task = GPEtask(grid, lambda X, Y, Z: 0.5 * (X**2 + Y**2))
    task.Ntotal = 1e5; task.g = 0.06
    phi = task.groundstate_itp(0.02, 1e-6, phi0)
    task.init_state = imprint_vortex(grid, phi, task.g, 5.0)
    task.solve_split(0.004, 50, 20)
"""
from ._lib import GPEError, lib  # noqa: F401  (loads libgpe.so or raises)
from .grid import grid2d, grid3d  # noqa: F401
from .imprint import imprint_vortex, imprint_vortex_ring  # noqa: F401
from .task import GPEtask, GPEtask2comp, GPEtaskSpinor, SGPEtask, detect_core, noise_variates, solve_split_batch  # noqa: F401


def device_available() -> bool:
    return bool(lib.gpe_device_available())


class pinned:
    """Page-lock a numpy array for the duration of a with-block."""

    def __init__(self, arr):
        self.arr = arr

    def __enter__(self):
        from . import _lib as L

        L.check(None, lib.gpe_host_register(self.arr.ctypes.data, self.arr.nbytes))
        return self.arr

    def __exit__(self, *exc):
        lib.gpe_host_unregister(self.arr.ctypes.data)
        return False
