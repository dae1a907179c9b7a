"""zgpu_solve_static, the solve entry point that allocates nothing.

It serves callers that must not allocate device memory (a plug-in whose host application
owns the GPU memory budget, a real-time loop that forbids cudaMalloc after start-up): its
scratch is a fixed array inside the library.  Here it is called through the C ABI on device
arrays and must give the same statistics as zgpu_solve on the same inputs, on two calls in
a row (the second call accumulates onto the first, so leftovers of the shared scratch from
the previous call would show up).  This file is collected last so a failure here leaves
every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _device_arrays(gp):
    return gp.device_arrays()


def _solve_static(gp, arrays, stream_ptr):
    from zombie_gb300 import _lib
    q = gp.queries.to_c()
    pde = gp.pde.to_c()
    ws = gp.problem.settings
    sp, st = arrays.to_c()
    rep = A.SolveReport()
    status = _lib.lib().zgpu_solve_static(stream_ptr, gp.problem.solver, C.byref(q), C.byref(pde), C.byref(ws),
                                          C.byref(sp), C.byref(st), C.byref(rep))
    return status, rep


def _host(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("make", [lambda: P.laplace_wos_2d(n_segments=512, grid=32, spp=64),
                                  lambda: P.mixed_wost_2d(n_segments=1024, grid=24, spp=64),
                                  lambda: P.screened_wos_3d(level=3, n_points=600, spp=32, sigma=4.0)])
def test_static_entry_matches_solve_on_two_calls(zgpu, make):
    import torch
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(make())
    assert gp.points.shape[0] <= A.ZGPU_STATIC_MAX_POINTS
    ref = _device_arrays(gp)
    new = _device_arrays(gp)
    stream = torch.cuda.current_stream()
    for call in range(2):
        gp.solve(ref)                      # the existing entry point (context stream)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        status, rep = _solve_static(gp, new, stream.cuda_stream)
        assert status == A.ZGPU_OK, call
        assert rep.error_word == 0 and rep.total_steps > 0
        torch.cuda.synchronize()
        # nothing was allocated on the device by the call (the first call of the process may
        # load the module that holds the fixed array, before this loop's first static call)
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        assert np.array_equal(_host(ref["n_solution_estimates"]), _host(new["n_solution_estimates"]))
        assert np.array_equal(_host(ref["total_walk_length"]), _host(new["total_walk_length"]))
        assert np.allclose(_host(ref["solution_mean"]), _host(new["solution_mean"]), rtol=0, atol=1e-9)
        assert np.allclose(_host(ref["solution_m2"]), _host(new["solution_m2"]), rtol=1e-9, atol=1e-9)
        assert np.array_equal(_host(ref["first_sphere_radius"]), _host(new["first_sphere_radius"]))


def test_static_entry_rejects_what_it_cannot_hold(zgpu):
    import torch
    from zombie_gb300 import _lib
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.laplace_wos_2d(n_segments=256, grid=16, spp=8))
    arrays = _device_arrays(gp)
    stream = torch.cuda.current_stream().cuda_stream
    q, pde = gp.queries.to_c(), gp.pde.to_c()
    sp, st = arrays.to_c()
    # more points than the fixed scratch holds
    sp.n = 65536 + 1
    assert _lib.lib().zgpu_solve_static(stream, gp.problem.solver, C.byref(q), C.byref(pde),
                                        C.byref(gp.problem.settings), C.byref(sp), C.byref(st), None) == A.ZGPU_ERR_INVALID_ARG
    assert b"at most 65536 points" in _lib.lib().zgpu_last_error()
    # walk splitting needs per-walk scratch the fixed array does not have
    sp.n = arrays.n
    ws = P.default_walk_settings(splitting=1.5)
    assert _lib.lib().zgpu_solve_static(stream, gp.problem.solver, C.byref(q), C.byref(pde), C.byref(ws),
                                        C.byref(sp), C.byref(st), None) == A.ZGPU_ERR_INVALID_ARG
    # host arrays are refused (the caller passes device memory)
    h = gp.host_arrays()
    hsp, hst = h.to_c()
    assert _lib.lib().zgpu_solve_static(stream, gp.problem.solver, C.byref(q), C.byref(pde),
                                        C.byref(gp.problem.settings), C.byref(hsp), C.byref(hst), None) == A.ZGPU_ERR_INVALID_ARG


def test_static_entry_with_no_points(zgpu):
    import torch
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.screened_wos_3d(level=2, n_points=64, spp=8, sigma=4.0))
    arrays = _device_arrays(gp)
    stream = torch.cuda.current_stream().cuda_stream
    q, pde = gp.queries.to_c(), gp.pde.to_c()
    sp, st = arrays.to_c()
    sp.n = 0
    rep = A.SolveReport()
    status = _lib_call(stream, gp, q, pde, gp.problem.settings, sp, st, rep)
    assert status == A.ZGPU_OK
    assert rep.total_walks == 0 and rep.total_steps == 0 and rep.error_word == 0
    torch.cuda.synchronize()
    assert int(arrays["n_solution_estimates"].sum().item()) == 0


def test_static_entry_rejects_gradients_and_scene_ids(zgpu):
    import torch
    from zombie_gb300 import _lib
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.laplace_wos_2d(n_segments=256, grid=16, spp=8))
    stream = torch.cuda.current_stream().cuda_stream
    q, pde = gp.queries.to_c(), gp.pde.to_c()
    # gradient statistics: the fixed scratch holds no gradient moments
    g = gp.device_arrays(gradients=True)
    sp, st = g.to_c()
    assert _lib_call(stream, gp, q, pde, gp.problem.settings, sp, st, None) == A.ZGPU_ERR_UNSUPPORTED
    assert b"solutions only" in _lib.lib().zgpu_last_error()
    # a scene table index per point: one scene only
    arrays = _device_arrays(gp)
    sid = torch.zeros(arrays.n, dtype=torch.int32, device=arrays["pt"].device)
    sp, st = arrays.to_c()
    sp.scene_id = sid.data_ptr()
    assert _lib_call(stream, gp, q, pde, gp.problem.settings, sp, st, None) == A.ZGPU_ERR_UNSUPPORTED
    assert b"one scene" in _lib.lib().zgpu_last_error()


def _lib_call(stream, gp, q, pde, ws, sp, st, rep):
    from zombie_gb300 import _lib
    return _lib.lib().zgpu_solve_static(stream, gp.problem.solver, C.byref(q), C.byref(pde), C.byref(ws),
                                        C.byref(sp), C.byref(st), C.byref(rep) if rep is not None else None)
