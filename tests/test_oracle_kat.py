"""Known-answer and property checks of the oracle itself (CPU)."""
import numpy as np
import pytest

STENCIL = np.array([1, 3, 1, 3, 14, 3, 1, 3, 1, 3, 14, 3, 14, -128, 14, 3, 14, 3,
                    1, 3, 1, 3, 14, 3, 1, 3, 1], np.float64)


def test_philox_known_answers(orc):
    # Random123 known-answer vectors for Philox4x32-10
    assert list(orc.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_philox2x32_known_answers(orc):
    # Random123 known-answer vectors for Philox2x32-10 (the noise stream)
    assert list(orc.philox2([0, 0], 0)) == [0xFF1DAE59, 0x6CD10DF2]
    assert list(orc.philox2([0xFFFFFFFF, 0xFFFFFFFF], 0xFFFFFFFF)) == [0x2C3F628B, 0xAB4FD7AD]
    assert list(orc.philox2([0x243F6A88, 0x85A308D3], 0x13198A2E)) == [0xDD7CE038, 0xF62A4C12]


def test_stencil_sum_identity(orc):
    """The reference's sanity check (src/paracrine.cu:82-103): a delta on a 7^3
    grid convolved with A sums to sum(delta) * sum(A)."""
    h, D, dt, k = 0.7, 2e-5, 40.0, 3e-4
    L = STENCIL / (30.0 * h * h)
    A = -0.5 * D * dt * L
    A[13] += 1 + 0.5 * dt * k
    u = np.zeros(7 ** 3)
    u[7 * 7 * 4 + 7 * 5 + 5] = 1.0
    out = orc.conv27(u, (7, 7, 7), A)
    assert out.sum() == pytest.approx(u.sum() * A.sum(), rel=1e-12)
    assert abs(STENCIL.sum()) == 0.0


def test_cn_solver_solves_its_system(orc):
    rng = np.random.default_rng(0)
    shape = (9, 8, 10)
    u0 = rng.random(int(np.prod(shape)))
    h, D, k, dt = 1.0, 0.05, 0.01, 1.0
    u, it, rr = orc.paracrine_cn_solve(u0, shape, h, D, k, dt, abs_tol=1e-20, max_iter=200, quirk_b=0)
    L = STENCIL / (30.0 * h * h)
    A = -0.5 * D * dt * L
    A[13] += 1 + 0.5 * dt * k
    lap = orc.conv27(u0, shape, L)
    b = (1 - dt * k / 2) * u0 + dt * D / 2 * lap
    assert np.allclose(orc.conv27(u, shape, A), b, atol=1e-9)
    assert 0 < it <= 200


def test_pcg7_against_scipy(orc):
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    nz, ny, nx = 6, 7, 8
    G = nx * ny * nz
    rng = np.random.default_rng(1)
    D = np.exp(rng.standard_normal(G)).astype(np.float32)
    alpha, beta = 3.0, 0.1
    # assemble A column by column from the oracle's apply
    A = np.stack([orc.apply7(np.eye(G)[j], (nz, ny, nx), alpha, beta, D) for j in range(G)], axis=1)
    assert np.allclose(A, A.T, atol=1e-12)
    b = rng.random(G)
    x, it, rel = orc.pcg7(b, np.zeros(G), (nz, ny, nx), alpha, beta, D, rtol=1e-10)
    xs = spl.spsolve(sp.csr_matrix(A), b)
    assert it > 0 and rel <= 1e-10
    assert np.allclose(x, xs, rtol=1e-8, atol=1e-12)


def test_hh_rest_and_rk4_order(orc):
    p = orc.hh_params()
    m, h, n = orc.steady_state(-65.0)
    assert 0.05 < m < 0.06 and 0.59 < h < 0.6 and 0.31 < n < 0.32
    # fourth order: halving dt cuts the error ~16x on a smooth stretch
    import ctypes as C

    def run(dt, T=2.0):
        p.dt = dt
        y = np.array([-65.0, m, h, n, 0.3, 0.1])
        for _ in range(int(round(T / dt))):
            orc.lib().orc_hh_rk4(C.byref(p), 1.0, 3.0, 0.0, orc.ptr(y))
        return y
    ref = run(0.0025)
    e1 = np.abs(run(0.02) - ref).max()
    e2 = np.abs(run(0.01) - ref).max()
    assert 10 < e1 / e2 < 22
