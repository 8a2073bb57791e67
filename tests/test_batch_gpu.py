"""Batches: many uneven problems, one persistent launch per step.

Every problem of a batch must end bit-for-bit equal to the same number of
kg_sweep calls on that problem alone (same tile body, same arithmetic), in
plain steps, through a replayed CUDA graph, and after tuning.
"""
import os

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import kgb200  # noqa: E402

KINDS = ["laplacian", "divergence", "wave13pt", "gaussblur"]


@pytest.fixture(scope="module", autouse=True)
def _device():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def make_batch(n, dtype, seed=3, lo=6, hi=48):
    rng = np.random.default_rng(seed)
    tdt = torch.float32 if dtype == kgb200.KG_F32 else torch.float64
    probs, bufs, meta = [], [], []
    for q in range(n):
        name = KINDS[rng.integers(0, 4)]
        nx, ny, ns = (int(np.exp(rng.uniform(np.log(lo), np.log(hi)))) for _ in range(3))
        shape = (nx, ny * ns) if name == "gaussblur" else (nx, ny, ns)
        narr = ol.NARR[ol.TEST_ID[name]]
        npts = nx * ny * ns
        arrs = [torch.from_numpy(rng.uniform(-1, 1, npts)).to(tdt).cuda() for _ in range(narr)]
        if name == "laplacian":
            coef = [rng.uniform(-1, 1), rng.uniform(-1, 1) / 6]
        elif name == "divergence":
            coef = list(rng.uniform(-1, 1, 3))
        elif name == "wave13pt":
            coef = [rng.uniform(-1, 1), rng.uniform(-1, 1) / 6, rng.uniform(-1, 1) / 6]
        else:
            coef = list(rng.uniform(0, 1, 6))
        probs.append(kgb200.problem(name, dtype, shape, coef, [a.data_ptr() for a in arrs]))
        bufs.append(arrs)
        meta.append((name, shape, coef))
    return probs, bufs, meta


def reference_run(meta, bufs, dtype, nsteps):
    """Each problem alone through kg_sweep; returns arrays in final roles."""
    out = []
    for (name, shape, coef), arrs in zip(meta, bufs):
        own = [a.clone() for a in arrs]
        by = {a.data_ptr(): a for a in own}
        ptrs = [a.data_ptr() for a in own]
        for _ in range(nsteps):
            kgb200.sweep(kgb200.problem(name, dtype, shape, coef, ptrs))
            ptrs = kgb200.rotate(name, ptrs)
        out.append([by[p] for p in ptrs])
    torch.cuda.synchronize()
    return out


def batch_final(batch, bufs, n):
    res = []
    for q in range(n):
        p = batch.final_roles(q)
        by = {a.data_ptr(): a for a in bufs[q]}
        res.append([by[p.arr[k]] for k in range(len(bufs[q]))])
    return res


@pytest.mark.parametrize("dtype", [kgb200.KG_F32, kgb200.KG_F64])
def test_batch_equals_individual_sweeps(dtype):
    n = 48
    probs, bufs, meta = make_batch(n, dtype)
    ref = reference_run(meta, bufs, dtype, 11)
    b = kgb200.Batch(probs)
    b.step(5)
    b.capture(3)
    b.launch()
    b.launch()
    torch.cuda.synchronize()
    assert b.config().steps_done == 11
    got = batch_final(b, bufs, n)
    for q in range(n):
        for k, (g, w) in enumerate(zip(got[q], ref[q])):
            assert torch.equal(g, w), "problem %d (%s) array %d differs" % (q, meta[q][0], k)
    b.close()


def test_batch_every_tile_shape_and_tuning(tmp_path):
    n = 24
    probs, bufs, meta = make_batch(n, kgb200.KG_F32, seed=9)
    ref = reference_run(meta, bufs, kgb200.KG_F32, 4)
    saved = [[a.clone() for a in arrs] for arrs in bufs]
    b = kgb200.Batch(probs)
    for shape in range(b.config().nshapes):
        for q in range(n):
            for a, s in zip(bufs[q], saved[q]):
                a.copy_(s)
        try:
            b.set_config(shape, 2 + shape % 3)
        except kgb200.KgError as e:
            # a temporal block too large for the shared memory of an SM
            assert "shared memory" in str(e)
            continue
        b.set_step(0)
        b.step(4)
        torch.cuda.synchronize()
        got = batch_final(b, bufs, n)
        for q in range(n):
            for g, w in zip(got[q], ref[q]):
                assert torch.equal(g, w), "shape %d problem %d" % (shape, q)
    cache = str(tmp_path / "tune.txt")
    b.tune(cache)
    c1 = b.config()
    assert os.path.exists(cache) and open(cache).read().count("\n") == 1
    b.set_config(0, 8)
    b.tune(cache)          # answered from the cache file
    c2 = b.config()
    assert (c1.shape, c1.ctas_per_sm) == (c2.shape, c2.ctas_per_sm)
    assert open(cache).read().count("\n") == 1
    b.close()


def temporal_configs(b):
    """Configuration indices of the temporal blocks (steps per launch > 1)."""
    out = []
    for shape in range(b.config().nshapes):
        try:
            b.set_config(shape, 2)
        except kgb200.KgError:
            continue            # its blocks need more shared memory than an SM has
        if b.config().temporal > 1:
            out.append((shape, b.config().temporal))
    return out


@pytest.mark.parametrize("dtype", [kgb200.KG_F32, kgb200.KG_F64])
def test_batch_temporal_blocks_equal_individual_sweeps(dtype):
    """Every temporal configuration, with step counts that leave a shorter
    last launch and an odd or even number of launches, plain and replayed
    from a graph: every array of every problem equals the problem's own
    kg_sweep calls bit for bit."""
    n = 40
    probs, bufs, meta = make_batch(n, dtype, seed=17)
    saved = [[a.clone() for a in arrs] for arrs in bufs]
    ref = reference_run(meta, bufs, dtype, 11)
    b = kgb200.Batch(probs)
    configs = temporal_configs(b)
    assert configs, "no temporal configuration fits"
    for shape, t in configs:
        for q in range(n):
            for a, s in zip(bufs[q], saved[q]):
                a.copy_(s)
        b.set_config(shape, 1 + shape % 3)
        b.set_step(0)
        b.step(5)
        b.capture(3)
        b.launch()
        b.launch()
        torch.cuda.synchronize()
        assert b.config().steps_done == 11
        got = batch_final(b, bufs, n)
        for q in range(n):
            for k, (g, w) in enumerate(zip(got[q], ref[q])):
                assert torch.equal(g, w), "config %d (T=%d) problem %d (%s) array %d differs" % (
                    shape, t, q, meta[q][0], k)
    b.close()


def bulk_configs(b):
    """Configuration indices of the bulk-staged tiles (and why others were
    refused)."""
    out, why = [], []
    for shape in range(b.config().nshapes):
        try:
            b.set_config(shape, 2)
        except kgb200.KgError as e:
            why.append(str(e))
            continue
        if b.config().staged:
            out.append(shape)
    return out, why


@pytest.mark.parametrize("dtype", [kgb200.KG_F32, kgb200.KG_F64])
def test_batch_bulk_tiles_equal_individual_sweeps(dtype):
    """The tiles whose inputs are staged in shared memory by bulk copies, in
    every shape, on problems whose sizes leave arrays that end off a 16-byte
    boundary (their last range is read from global memory), plain steps and
    graph replays: every array equals the problem's own kg_sweep calls."""
    n = 40
    probs, bufs, meta = make_batch(n, dtype, seed=23, lo=12, hi=70)
    saved = [[a.clone() for a in arrs] for arrs in bufs]
    ref = reference_run(meta, bufs, dtype, 7)
    b = kgb200.Batch(probs)
    configs, why = bulk_configs(b)
    assert configs, "no bulk configuration is available: %s" % why
    for shape in configs:
        for q in range(n):
            for a, s in zip(bufs[q], saved[q]):
                a.copy_(s)
        b.set_config(shape, 1 + shape % 4)
        b.set_step(0)
        b.step(3)
        b.capture(2)
        b.launch()
        b.launch()
        torch.cuda.synchronize()
        kgb200.engine_status()
        assert b.config().steps_done == 7
        got = batch_final(b, bufs, n)
        for q in range(n):
            for k, (g, w) in enumerate(zip(got[q], ref[q])):
                assert torch.equal(g, w), "config %d problem %d (%s %s) array %d differs" % (
                    shape, q, meta[q][0], meta[q][1], k)
    b.close()


def test_batch_f64_matches_oracle():
    probs, bufs, meta = make_batch(6, kgb200.KG_F64, seed=21)
    host = [[a.cpu().numpy().copy() for a in arrs] for arrs in bufs]
    b = kgb200.Batch(probs)
    b.step(3)
    torch.cuda.synchronize()
    got = batch_final(b, bufs, 6)
    for q, (name, shape, coef) in enumerate(meta):
        case = ol.Case.from_arrays(name, shape, coef, host[q])
        case.run(3)
        for g, w in zip(got[q], case.arrays()):
            assert np.array_equal(g.cpu().numpy().view(np.uint64), w.view(np.uint64))
    b.close()


def test_batch_rejects():
    x = torch.zeros(1000, device="cuda")
    y = torch.zeros(1000, device="cuda")
    lib = kgb200.load()
    import ctypes
    h = ctypes.c_void_p()
    bad = (kgb200.KgProblem * 1)(kgb200.problem("tricubic", kgb200.KG_F32, (10, 10, 10), [],
                                                [x.data_ptr(), y.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr()]))
    assert lib.kg_batch_create(ctypes.byref(h), bad, 1) == 5
    mixed = (kgb200.KgProblem * 2)(kgb200.problem("laplacian", kgb200.KG_F32, (10, 10, 10), [1, 1], [x.data_ptr(), y.data_ptr()]),
                                   kgb200.problem("laplacian", kgb200.KG_F64, (10, 10, 5), [1, 1], [x.data_ptr(), y.data_ptr()]))
    assert lib.kg_batch_create(ctypes.byref(h), mixed, 2) == 1
