"""Poisson solves (config: mixed-precision iterative refinement).

The solver is project-defined (the reference has no red-black SOR): its
oracle is the CPU restatement of the red-black SOR sweep in oracle/ plus the
residual itself, computed on the CPU in FP64 from the returned solution.
"""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def poisson_rhs(shape, seed=7):
    """f uniform [-1,1) on the interior with its mean removed, 0 on the outer planes."""
    nx, ny, ns = shape
    rng = np.random.default_rng(seed)
    f = np.zeros((ns, ny, nx))
    inner = rng.uniform(-1, 1, (ns - 2, ny - 2, nx - 2))
    f[1:-1, 1:-1, 1:-1] = inner - inner.mean()
    return f.reshape(-1)


def test_sor_sweeps_match_oracle():
    shape = (21, 18, 16)
    f = poisson_rhs(shape)
    u_cpu = np.zeros_like(f)
    ol.rbsor_sweeps(u_cpu, f, shape, 1.8, 30)
    fd = torch.from_numpy(f).cuda()
    ud = torch.zeros_like(fd)
    st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kgb200.KG_SOLVE_SOR_F64,
                                   rtol=1e-30, sweeps_per_check=30, max_sweeps=30, raise_on_timeout=False)
    assert st == 4 and rep.sweeps == 30          # capped: KG_ETIMEOUT, no hang
    u = ud.cpu().numpy()
    assert np.max(np.abs(u - u_cpu)) <= 1e-13 * np.max(np.abs(u_cpu))


@pytest.mark.parametrize("kind", [kgb200.KG_SOLVE_SOR_F64, kgb200.KG_SOLVE_IR_SOR_F32])
def test_solve_to_tolerance(kind):
    shape = (40, 36, 30)
    f = poisson_rhs(shape)
    fd = torch.from_numpy(f).cuda()
    ud = torch.zeros_like(fd)
    st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kind, omega=1.8, rtol=1e-10,
                                   sweeps_per_check=25)
    assert st == 0 and rep.rel_residual <= 1e-10
    u = ud.cpu().numpy()
    rel = ol.residual_norm(u, f, shape) / np.linalg.norm(f)
    assert rel <= 1.05e-10, rel
    # the boundary stays zero
    g = u.reshape(shape[2], shape[1], shape[0])
    assert not g[0].any() and not g[-1].any() and not g[:, 0].any() and not g[:, :, -1].any()


def fp32_rbsor(e, r, shape, omega, sweeps):
    """FP32 red-black SOR on A e = r in place (numpy float32, one rounding per
    operation, the GPU sweep's operand order): colour 0 then colour 1, each
    colour's points read only the other colour."""
    nx, ny, ns = shape
    g = e.reshape(ns, ny, nx)
    rr = r.reshape(ns, ny, nx)
    k, j, i = np.meshgrid(np.arange(ns), np.arange(ny), np.arange(nx), indexing="ij")
    inner = (i > 0) & (i < nx - 1) & (j > 0) & (j < ny - 1) & (k > 0) & (k < ns - 1)
    w, sixth = np.float32(omega), np.float32(1.0 / 6.0)
    for _ in range(sweeps):
        for color in (0, 1):
            mask = inner & (((i + j + k) & 1) == color)
            s = np.zeros_like(g)
            s[1:-1, 1:-1, 1:-1] = (((((g[1:-1, 1:-1, :-2] + g[1:-1, 1:-1, 2:]) + g[1:-1, :-2, 1:-1]) +
                                     g[1:-1, 2:, 1:-1]) + g[:-2, 1:-1, 1:-1]) + g[2:, 1:-1, 1:-1])
            new = g + w * ((s + rr) * sixth - g)
            g[mask] = new[mask]


@pytest.mark.parametrize("shape", [(21, 18, 16), (20, 17, 15), (5, 4, 3)])
def test_refinement_sweeps_match_fp32_restatement(shape):
    """One outer step of refinement from u = 0: e relaxed by FP32 red-black SOR
    on the colour-split layout, then u = e.  Equal to the FP32 restatement up
    to FMA contraction (a wrong neighbour or colour would be O(1) off); odd and
    even nx (the split rows' padding)."""
    m = 6
    f = poisson_rhs(shape)
    fd = torch.from_numpy(f).cuda()
    ud = torch.zeros_like(fd)
    st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kgb200.KG_SOLVE_IR_SOR_F32, omega=1.8,
                                   rtol=1e-30, sweeps_per_check=m, max_sweeps=m, raise_on_timeout=False)
    assert st == 4 and rep.sweeps == m and rep.outer == 1
    e = np.zeros(f.size, np.float32)
    fp32_rbsor(e, f.astype(np.float32), shape, 1.8, m)
    u = ud.cpu().numpy()
    assert np.max(np.abs(u - e.astype(np.float64))) <= 1e-5 * max(np.max(np.abs(e)), 1e-30)


def fp32_jacobi(r, shape, sweeps):
    """FP32 Jacobi sweeps on A e = r from e = 0 (numpy float32, the GPU
    sweep's operand order); returns e."""
    nx, ny, ns = shape
    rr = r.reshape(ns, ny, nx)
    e = np.zeros((ns, ny, nx), np.float32)
    sixth = np.float32(1.0 / 6.0)
    for _ in range(sweeps):
        n = np.zeros_like(e)
        s = (((((e[1:-1, 1:-1, :-2] + e[1:-1, 1:-1, 2:]) + e[1:-1, :-2, 1:-1]) + e[1:-1, 2:, 1:-1]) +
              e[:-2, 1:-1, 1:-1]) + e[2:, 1:-1, 1:-1])
        n[1:-1, 1:-1, 1:-1] = (s + rr[1:-1, 1:-1, 1:-1]) * sixth
        e = n
    return e.reshape(-1)


@pytest.mark.parametrize("shape", [(20, 17, 15), (21, 18, 16), (136, 9, 7)])
def test_jacobi_refinement_sweeps_match_fp32_restatement(shape):
    """One outer step of refinement around FP32 Jacobi sweeps from u = 0
    (16-byte vectors with shuffled x neighbours where nx is a multiple of 4):
    bit for bit the FP32 restatement (no product to contract)."""
    m = 5
    f = poisson_rhs(shape)
    fd = torch.from_numpy(f).cuda()
    ud = torch.zeros_like(fd)
    st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kgb200.KG_SOLVE_IR_JACOBI_F32,
                                   rtol=1e-30, sweeps_per_check=m, max_sweeps=m, raise_on_timeout=False)
    assert st == 4 and rep.sweeps == m and rep.outer == 1
    e = fp32_jacobi(f.astype(np.float32), shape, m)
    assert np.array_equal(ud.cpu().numpy(), e.astype(np.float64))


def test_refinement_keeps_the_sor_rate():
    """Refinement with FP32 inner SOR needs about as many sweeps as FP64 SOR."""
    shape = (48, 40, 32)
    f = poisson_rhs(shape)
    fd = torch.from_numpy(f).cuda()
    res = {}
    for kind in (kgb200.KG_SOLVE_SOR_F64, kgb200.KG_SOLVE_IR_SOR_F32):
        ud = torch.zeros_like(fd)
        st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kind, rtol=1e-10, sweeps_per_check=20)
        assert st == 0
        res[kind] = rep.sweeps
    assert res[kgb200.KG_SOLVE_IR_SOR_F32] <= 1.15 * res[kgb200.KG_SOLVE_SOR_F64] + 20


def test_jacobi_refinement_converges():
    shape = (14, 12, 10)
    f = poisson_rhs(shape)
    fd = torch.from_numpy(f).cuda()
    ud = torch.zeros_like(fd)
    st, rep = kgb200.poisson_solve(shape, fd.data_ptr(), ud.data_ptr(), kgb200.KG_SOLVE_IR_JACOBI_F32,
                                   rtol=1e-10, sweeps_per_check=200, max_sweeps=200000)
    assert st == 0
    rel = ol.residual_norm(ud.cpu().numpy(), f, shape) / np.linalg.norm(f)
    assert rel <= 1.05e-10


def test_solve_rejects_bad_options():
    fd = torch.zeros(27, dtype=torch.float64, device="cuda")
    with pytest.raises(kgb200.KgError):
        kgb200.poisson_solve((3, 3, 3), fd.data_ptr(), fd.data_ptr(), 7)
    with pytest.raises(kgb200.KgError):
        kgb200.poisson_solve((3, 3, 3), fd.data_ptr(), fd.data_ptr(), 0, omega=2.5)
