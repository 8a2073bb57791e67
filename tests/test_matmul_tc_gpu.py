"""The tensor-core form of matmul (kg_matmul_tc: tcgen05 kind::tf32, three
TF32 products per product) against the FP64 product of the same FP32 inputs.

Reference loop: matmul/matmul.F90:56-68, C(i,j) += A(i,k) B(k,j), column-major.
The oracle here is numpy's FP64 product (the k order does not matter at FP64
against an FP32 result).  The bound is relative to sum_k |A(i,k)| |B(k,j)|:
3xTF32 keeps about 2^-21 of each product and the FP32 accumulation adds up
to about 3K 2^-24 of the magnitude; a wrong descriptor, swizzle or tile index
is off by the size of the values themselves.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def run(nx, ny, ns, seed, c0=True):
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1, 1, nx * ny).astype(np.float32)
    B = rng.uniform(-1, 1, ny * ns).astype(np.float32)
    C = rng.uniform(-1, 1, nx * ns).astype(np.float32) if c0 else np.zeros(nx * ns, np.float32)
    a, b, c = (torch.from_numpy(x).cuda() for x in (A, B, C))
    lib = kgb200.load()
    kgb200.check(lib.kg_matmul_tc(nx, ny, ns, a.data_ptr(), b.data_ptr(), c.data_ptr(), None))
    kgb200.engine_status()
    got = c.cpu().numpy().astype(np.float64).reshape(ns, nx)          # [j][i]
    A64 = A.astype(np.float64).reshape(ny, nx)                        # [k][i]
    B64 = B.astype(np.float64).reshape(ns, ny)                        # [j][k]
    ref = C.astype(np.float64).reshape(ns, nx) + B64 @ A64            # [j][i] = sum_k B[j][k] A[k][i]
    mag = np.abs(C.astype(np.float64)).reshape(ns, nx) + np.abs(B64) @ np.abs(A64)
    return got, ref, mag


# (2000, 100, 2600): more than a wave of 128 x 128 tiles, ragged in both
# directions; (2000, 70, 2000): 128 x 256 tiles (one wave of them against two
# of 128 x 128), ragged in M, N and K
@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 5, 3), (33, 17, 40), (128, 32, 128), (130, 70, 129),
                                   (256, 96, 384), (512, 256, 256), (2000, 100, 2600), (2000, 70, 2000)])
def test_matmul_tc_matches_fp64(shape):
    got, ref, mag = run(*shape, seed=sum(shape))
    err = np.abs(got - ref)
    # elementwise: every term's rounding at its worst; normwise: typical
    assert np.all(err <= 3e-5 * mag + 1e-30), (shape, float(np.max(err / mag)))
    assert np.linalg.norm(err) <= 3e-6 * np.linalg.norm(mag), (shape, float(np.linalg.norm(err) / np.linalg.norm(mag)))


def test_matmul_tc_accumulates_into_c_and_keeps_the_rest():
    """C starts at its own values (the Fortran kernel accumulates into C);
    the tail tile's rows and columns past nx, ns are never written."""
    nx, ny, ns = 70, 40, 50
    rng = np.random.default_rng(3)
    A = torch.from_numpy(rng.uniform(-1, 1, nx * ny).astype(np.float32)).cuda()
    B = torch.from_numpy(rng.uniform(-1, 1, ny * ns).astype(np.float32)).cuda()
    big = torch.full((nx * ns + 4096,), 7.0, dtype=torch.float32, device="cuda")
    big[:nx * ns] = 0
    kgb200.check(kgb200.load().kg_matmul_tc(nx, ny, ns, A.data_ptr(), B.data_ptr(), big.data_ptr(), None))
    kgb200.engine_status()
    tail = big[nx * ns:].cpu().numpy()
    assert np.all(tail == 7.0)
    ref = (B.double().cpu().numpy().reshape(ns, ny) @ A.double().cpu().numpy().reshape(ny, nx)).reshape(-1)
    assert np.max(np.abs(big[:nx * ns].double().cpu().numpy() - ref)) <= 1e-5 * np.max(np.abs(ref))


def test_matmul_tc_rejects_bad_arguments():
    lib = kgb200.load()
    x = torch.zeros(64, dtype=torch.float32, device="cuda")
    p = x.data_ptr()
    assert lib.kg_matmul_tc(-1, 2, 2, p, p, p, None) == 1   # KG_EINVAL
    assert lib.kg_matmul_tc(2, 2, 2, p, p + 64, p + 8, None) == 1   # C overlaps A
    assert lib.kg_matmul_tc(2, 2, 2, None, p, p + 128, None) == 1
    assert lib.kg_matmul_tc(0, 2, 2, p, p, p, None) == 0              # KG_OK: nothing to do
