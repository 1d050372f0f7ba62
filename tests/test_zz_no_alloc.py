"""nn_pcg_solve_noalloc: the Jacobi-PCG solve for callers that may not allocate
device memory (a host framework owning the GPU memory budget, or a real-time
loop that cannot take cudaMalloc's device-wide synchronisation).

Called through the C ABI; each result is compared with the allocating entry
point (nn_pcg_create + nn_pcg_solve) on the same inputs, within the PCG tests'
tolerance, on two calls in a row with different right-hand sides (the shared
fixed scratch keeps the previous call's contents).  The device's free memory
(cuMemGetInfo), taken after a warm-up call, is the same after those calls,
which a single cudaMalloc would change.  This file is collected last so that
a run stopping at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

import neuronephys_clean_gb300 as nn

pytestmark = pytest.mark.gpu


def _free_device_bytes() -> int:
    """Free memory of the current device (driver API, current context)."""
    cuda = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert cuda.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return free.value


def _solve_noalloc(ctx, shape, alpha, beta, D, b, x):
    lib = nn.lib()
    nz, ny, nx = shape
    it, rel = C.c_int(0), C.c_double(0.0)
    st = lib.nn_pcg_solve_noalloc(C.c_void_p(lib.nn_ctx_stream(ctx.handle)), nx, ny, nz, alpha, beta,
                                  None if D is None else D.ptr, b.ptr, x.ptr, 1e-6, 5000, C.byref(it), C.byref(rel))
    return st, it.value, rel.value


@pytest.mark.parametrize("hetero", [True, False])
def test_noalloc_matches_allocating_solver(ctx, hetero):
    shape = (40, 48, 64)  # 122,880 cells, below the 64^3 limit
    G = int(np.prod(shape))
    rng = np.random.default_rng(11)
    D = ctx.to_device(np.exp(rng.normal(0.0, 0.5, G)).astype(np.float32)) if hetero else None
    alpha, beta = 6.0, 0.1
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, D)
    cases = []
    for call in range(2):
        b_h = rng.random(G).astype(np.float32)
        b_h[rng.integers(0, G, 50)] += 5.0
        b = ctx.to_device(b_h)
        x_ref = ctx.to_device(np.zeros(G, np.float32))
        it_ref, rel_ref = pc.solve(b, x_ref, rtol=1e-6, max_iter=5000)
        cases.append((b, x_ref, it_ref, ctx.to_device(np.zeros(G, np.float32))))
    # a warm-up call does the per-device set-up (and loads the kernels it
    # launches); the compared calls then must leave the free memory unchanged
    warm = ctx.to_device(np.zeros(G, np.float32))
    assert _solve_noalloc(ctx, shape, alpha, beta, D, cases[0][0], warm)[0] == 0
    ctx.synchronize()
    free0 = _free_device_bytes()
    results = [_solve_noalloc(ctx, shape, alpha, beta, D, b, x) for (b, _, _, x) in cases]
    ctx.synchronize()
    assert _free_device_bytes() == free0
    for call, ((st, it, rel), (_, x_ref, it_ref, x)) in enumerate(zip(results, cases)):
        assert st == 0, nn.lib().nn_status_string(st)
        assert rel <= 1e-6 and abs(it - it_ref) <= 1
        ref = x_ref.numpy().astype(np.float64)
        got = x.numpy().astype(np.float64)
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref), call


def test_noalloc_rejects_grids_beyond_its_scratch(ctx):
    lib = nn.lib()
    b = ctx.to_device(np.zeros(8, np.float32))
    x = ctx.to_device(np.zeros(8, np.float32))
    it, rel = C.c_int(0), C.c_double(0.0)
    st = lib.nn_pcg_solve_noalloc(None, 65, 64, 64, 1.0, 0.0, None, b.ptr, x.ptr, 1e-6, 10, C.byref(it),
                                  C.byref(rel))
    assert st == 7  # NN_ERR_UNSUPPORTED: larger than NN_PCG_NOALLOC_MAX_CELLS, nothing launched
