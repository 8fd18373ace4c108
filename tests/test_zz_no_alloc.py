"""gpe_norm_noalloc: the norm of a caller's device array without any device
allocation by the library (for callers such as MEX code on MATLAB-owned
gpuArray memory, or code inside a solve_split callback, that cannot allocate
at that point).  Checked through the C ABI against the context-based
entry point (gpe_set_state_device + gpe_observables) on two calls in a row,
so the second call also shows that the shared fixed scratch array carries no
state over from the first; a further call leaves the device's free memory and
torch's allocated bytes unchanged (the property the entry point exists for);
host memory and misaligned pointers are refused before they reach a kernel."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_copy(torch, arr):
    """A device buffer holding arr's interleaved complex values (test-owned)."""
    real = np.ascontiguousarray(arr).view(np.float32 if arr.dtype == np.complex64 else np.float64)
    return torch.from_numpy(real.ravel().copy()).to("cuda")


def _context_norm(gpe, grid, dev_buf, precision):
    from gpe_gb300 import _lib as L

    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
    task._push_params()
    task._upload_V(np.ascontiguousarray(task.Vtrap))
    L.check(task._ctx, L.lib.gpe_set_state_device(task._ctx, C.c_void_p(dev_buf.data_ptr()), precision))
    o = L.gpe_obs()
    L.check(task._ctx, L.lib.gpe_observables(task._ctx, C.byref(o)))
    task.close()
    return o.norm


def _noalloc_norm(dev_buf, npoints, precision, weight):
    from gpe_gb300 import _lib as L

    out = C.c_double(-1.0)
    st = L.lib.gpe_norm_noalloc(C.c_void_p(dev_buf.data_ptr()), npoints, precision, weight, None, C.byref(out))
    L.check(None, st)
    return out.value


def test_norm_noalloc_matches_context_entry_point_twice(gpe):
    torch = pytest.importorskip("torch")
    from gpe_gb300 import _lib as L

    rng = np.random.default_rng(11)
    # call 1: 3D complex FP32 state
    g3 = gpe.grid3d(5, 64, 5, 48, 4, 32, precision="single")
    psi3 = (rng.standard_normal(g3.shape) + 1j * rng.standard_normal(g3.shape)).astype(np.complex64)
    d3 = _device_copy(torch, psi3)
    ref3 = _context_norm(gpe, g3, d3, L.GPE_FP32)
    got3 = _noalloc_norm(d3, psi3.size, L.GPE_FP32, g3.weight)
    assert got3 == pytest.approx(ref3, rel=1e-6)
    # call 2: a smaller 2D complex FP64 state right after (the shared scratch
    # still holds call 1's partials)
    g2 = gpe.grid2d(6, 96, 4, 128, precision="double")
    psi2 = np.exp(-(g2.mesh["x"] ** 2 + g2.mesh["y"] ** 2) / 4) * np.exp(0.7j * g2.mesh["x"])
    d2 = _device_copy(torch, psi2)
    ref2 = _context_norm(gpe, g2, d2, L.GPE_FP64)
    got2 = _noalloc_norm(d2, psi2.size, L.GPE_FP64, g2.weight)
    assert got2 == pytest.approx(ref2, rel=1e-12)
    assert got2 == pytest.approx(g2.integrate(np.abs(psi2) ** 2), rel=1e-12)


def test_norm_noalloc_rejects_inputs_beyond_its_scratch(gpe):
    torch = pytest.importorskip("torch")
    from gpe_gb300 import _lib as L

    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = C.c_double()
    st = L.lib.gpe_norm_noalloc(C.c_void_p(buf.data_ptr()), 512 ** 3 + 1, L.GPE_FP32, 1.0, None, C.byref(out))
    assert st == L.GPE_ERR_INVALID
    assert b"exceed" in L.lib.gpe_last_error(None)


def test_norm_noalloc_allocates_no_device_memory(gpe):
    torch = pytest.importorskip("torch")
    from gpe_gb300 import _lib as L

    rng = np.random.default_rng(5)
    psi = (rng.standard_normal(64 * 64 * 32) + 1j * rng.standard_normal(64 * 64 * 32))
    bufs = {L.GPE_FP32: _device_copy(torch, psi.astype(np.complex64)),
            L.GPE_FP64: _device_copy(torch, psi.astype(np.complex128))}
    # warm-up calls: the per-device scratch lookup and the lazy loading of
    # both kernels' code happen here, once per process
    for prec, buf in bufs.items():
        _noalloc_norm(buf, psi.size, prec, 0.5)
    torch.cuda.synchronize()
    for prec, buf in bufs.items():
        free0, _ = torch.cuda.mem_get_info()
        alloc0 = torch.cuda.memory_allocated()
        got = _noalloc_norm(buf, psi.size, prec, 0.5)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, f"device free bytes changed by {free0 - free1}"
        assert torch.cuda.memory_allocated() == alloc0
        tol = 1e-6 if prec == L.GPE_FP32 else 1e-12
        assert got == pytest.approx(0.5 * float(np.sum(np.abs(psi) ** 2)), rel=tol)


def test_norm_noalloc_refuses_host_and_misaligned_pointers(gpe):
    torch = pytest.importorskip("torch")
    from gpe_gb300 import _lib as L

    out = C.c_double(-1.0)
    host = np.zeros(2 * 4096, dtype=np.float64)
    st = L.lib.gpe_norm_noalloc(C.c_void_p(host.ctypes.data), 4096, L.GPE_FP64, 1.0, None, C.byref(out))
    assert st == L.GPE_ERR_INVALID and b"host memory" in L.lib.gpe_last_error(None)
    pinned = torch.zeros(2 * 4096, dtype=torch.float64).pin_memory()
    st = L.lib.gpe_norm_noalloc(C.c_void_p(pinned.data_ptr()), 4096, L.GPE_FP64, 1.0, None, C.byref(out))
    assert st == L.GPE_ERR_INVALID and b"host memory" in L.lib.gpe_last_error(None)
    dev = torch.zeros(2 * 4096 + 2, dtype=torch.float64, device="cuda")
    st = L.lib.gpe_norm_noalloc(C.c_void_p(dev.data_ptr() + 8), 4096, L.GPE_FP64, 1.0, None, C.byref(out))
    assert st == L.GPE_ERR_INVALID and b"aligned" in L.lib.gpe_last_error(None)
    assert out.value == -1.0
    # the library is still usable afterwards
    assert _noalloc_norm(dev, 4096, L.GPE_FP64, 1.0) == 0.0


def test_norm_noalloc_refuses_a_capturing_stream(gpe):
    """The call waits on the host for its result, which a stream under
    capture cannot do: it is refused before the stream is touched, and the
    caller's capture goes on."""
    torch = pytest.importorskip("torch")
    from gpe_gb300 import _lib as L

    buf = torch.ones(64, dtype=torch.float32, device="cuda")
    _noalloc_norm(buf, 32, L.GPE_FP32, 1.0)  # first call on the device: the scratch lookup
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    out = C.c_double(-1.0)
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            y = buf * 2.0
            st = L.lib.gpe_norm_noalloc(C.c_void_p(buf.data_ptr()), 32, L.GPE_FP32, 1.0,
                                        C.c_void_p(s.cuda_stream), C.byref(out))
    assert st == L.GPE_ERR_INVALID
    assert b"capturing" in L.lib.gpe_last_error(None)
    g.replay()
    torch.cuda.synchronize()
    assert float(y.sum()) == pytest.approx(128.0)
    assert _noalloc_norm(buf, 32, L.GPE_FP32, 1.0) == pytest.approx(64.0)  # 32 points of 1 + 1i
