"""The allocation-free kinetic-energy entry point, through the C ABI, on the GPU.

souffle_gpu_kinetic_energy_noalloc serves callers that must not allocate device memory once they
are running (all GPU memory reserved up front, or a framework that owns the device heap): it reads
their device arrays and keeps its scratch in a fixed array inside the library.  Here its result
must match the handle-based souffle_gpu_kinetic_energy on the same state, on two calls in a row,
and it must refuse inputs larger than its fixed scratch.  This file sorts last so a run that stops
at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_workload, load_golden

pytestmark = pytest.mark.gpu


def _state_on_gpu():
    from souffle_gb300 import gpu
    g = load_golden("bilayer_dense")
    t, opt, d = golden_workload(g)
    s = gpu.GpuSystem(t, [gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))])
    s.set_state(g["pos"], g["vel"])
    s.md_begin()
    s.md_steps(0, 7)
    return s, t


def test_noalloc_kinetic_energy_matches_handle_entry_point():
    import torch
    from souffle_gb300 import gpu
    lib = gpu.load()
    s, t = _state_on_gpu()
    ke_ref = C.c_double()
    gpu._check(lib.souffle_gpu_kinetic_energy(s.h, 0, C.byref(ke_ref)))
    _, vel = s.get_state()
    mass = np.tile(t.mass, vel.shape[0] // t.n_beads)
    # the caller owns (and here allocates, outside the entry point) every device buffer
    d_vel = torch.tensor(vel.reshape(-1), dtype=torch.float64, device="cuda")
    d_mass = torch.tensor(mass, dtype=torch.float64, device="cuda")
    d_out = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    dp = C.POINTER(C.c_double)
    results = []
    for _ in range(2):
        rc = lib.souffle_gpu_kinetic_energy_noalloc(C.cast(d_vel.data_ptr(), dp), C.cast(d_mass.data_ptr(), dp),
                                                    vel.shape[0], C.cast(d_out.data_ptr(), dp),
                                                    C.c_void_p(stream))
        assert rc == 0, lib.souffle_gpu_last_error()
        torch.cuda.synchronize()
        results.append(d_out.cpu().numpy().copy())
    for out in results:
        assert out[0] == pytest.approx(ke_ref.value, rel=1e-12)
        np.testing.assert_allclose(out[1:], vel.sum(axis=0), rtol=0, atol=1e-9)
    assert np.array_equal(results[0], results[1])   # same bits on repeated calls
    # unit masses when no mass array is given
    rc = lib.souffle_gpu_kinetic_energy_noalloc(C.cast(d_vel.data_ptr(), dp), None, vel.shape[0],
                                                C.cast(d_out.data_ptr(), dp), C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert d_out[0].item() == pytest.approx(0.5 * (vel ** 2).sum(), rel=1e-12)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    from souffle_gb300 import gpu
    lib = gpu.load()
    dp = C.POINTER(C.c_double)
    buf = torch.zeros(12, dtype=torch.float64, device="cuda")
    p = C.cast(buf.data_ptr(), dp)
    # the size check runs on the host before anything is launched
    rc = lib.souffle_gpu_kinetic_energy_noalloc(p, None, 4194305, p, None)
    assert rc == 1
    assert b"scratch limit" in lib.souffle_gpu_last_error()
    assert torch.count_nonzero(buf).item() == 0


@pytest.mark.parametrize("n", [600_001, 4_194_304])
def test_noalloc_large_inputs_against_float64_sums(n):
    """Sizes where the 2048-block grid takes several beads per thread, up to the limit itself."""
    import torch
    from souffle_gb300 import gpu
    lib = gpu.load()
    rng = np.random.default_rng(n)
    vel = rng.normal(size=(n, 3))
    mass = rng.uniform(0.5, 2.0, size=n)
    d_vel = torch.tensor(vel.reshape(-1), dtype=torch.float64, device="cuda")
    d_mass = torch.tensor(mass, dtype=torch.float64, device="cuda")
    d_out = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    dp = C.POINTER(C.c_double)
    results = []
    for _ in range(2):
        rc = lib.souffle_gpu_kinetic_energy_noalloc(C.cast(d_vel.data_ptr(), dp), C.cast(d_mass.data_ptr(), dp), n,
                                                    C.cast(d_out.data_ptr(), dp), C.c_void_p(stream))
        assert rc == 0, lib.souffle_gpu_last_error()
        torch.cuda.synchronize()
        results.append(d_out.cpu().numpy().copy())
    ke = 0.5 * (mass * (vel ** 2).sum(axis=1)).sum()
    for out in results:
        assert out[0] == pytest.approx(ke, rel=1e-12)
        # velocity sums cancel: compare against the scale of the summed magnitudes
        np.testing.assert_allclose(out[1:], vel.sum(axis=0), rtol=0, atol=1e-12 * np.abs(vel).sum(axis=0).max())
    assert np.array_equal(results[0], results[1])
