#!/usr/bin/env python3
"""Benchmark of the suite's stencil sweeps on GB300.

Default workload (the suite in plain FP64, `benchmark 512 256 256 10`): one
step runs all eleven stencils (laplacian, divergence, gradient, uxx1,
wave13pt, tricubic, tricubic2, jacobi, lapgsrb, gaussblur, gameoflife), ten
sweeps each with the reference's pointer rotation, 3D tests on 512x256x256
and 2D tests on 512x65536, inputs drawn as the reference main() draws them
(glibc rand(), default seed).  Metric: grid-point updates per second
(Gpts/s, N = nx*ny*ns points per sweep, the reference's t_krn convention).

  value   device-resident: arrays already in HBM, each program's ten sweeps
          as one CUDA graph (kg_plan; tricubic and tricubic2 evaluate their
          loop-invariant weights once per program).  The same step with every
          sweep a kg_sweep call (weights evaluated in every sweep, as the
          reference does) is reported beside it (weights_per_sweep).
  e2e     the same steps through kg_program_run with pinned HOST arrays:
          allocate, copy in, ten sweeps, copy the checksum arrays out, free.
  --impl reference
          the reference's CPU implementation of the sweeps: the oracle's C
          restatement of the reference kernels built with the suite's -O3
          -ffast-math flags and OpenMP over all host cores (the reference tree
          is not on the GPU host), on the same steps: ten sweeps of each
          program from its initial inputs, drawn by the oracle itself.

Multi-GPU: the sweeps do not exchange data between problems; each rank runs
an independent replica of the workload ("replicas only", weak scaling).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "kernelgen-perf-tests_gb300")
sys.path.insert(0, PKG)

import kgb200  # noqa: E402

SUITE = kgb200.STENCILS
SHAPE3 = (512, 256, 256)
SHAPE2 = (512, 256 * 256)
NT = 10
NPTS = 512 * 256 * 256

# Compulsory HBM bytes per point per sweep in FP64 (every input array read
# once, every output array written once).
BYTES_PER_PT = {"laplacian": 16, "divergence": 32, "gradient": 32, "uxx1": 48, "wave13pt": 24,
                "tricubic": 40, "tricubic2": 40, "jacobi": 16, "lapgsrb": 16, "gaussblur": 16,
                "gameoflife": 16}
# FP64 operations per point in the reference expressions, counted after
# common-subexpression elimination (tricubic: 12 weight products + 3 adds per
# axis, 16 wa*wb, 64 *wc, 64 *u0, 63 adds); a division counts as one.
FP64_OPS_PER_PT = {"laplacian": 8, "divergence": 8, "gradient": 6, "uxx1": 25, "wave13pt": 16,
                   "tricubic": 252, "tricubic2": 253, "jacobi": 11, "lapgsrb": 28, "gaussblur": 31,
                   "gameoflife": 14}
# Arrays whose contents are the reference's checksum ("final mean") input.
def result_mask(name):
    return {"divergence": 0x1, "gradient": 0xE}.get(name, 0x2)


PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
# DRAM bytes (read + write) per full-size launch from one ncu capture of a
# smaller case (256x256x128, and 256^3 for laplacian) scaled by the points
# processed: the sweep of a tricubic program reads its 64 precomputed weight
# planes, 512 B per point; tricubic reads and writes the same arrays over a
# domain one plane larger per axis, so it takes tricubic2's.
NCU_TRAFFIC = {"tricubic": 4 * 4.194e9, "tricubic2": 4 * 4.194e9, "laplacian": 2 * 227.5e6}


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def replica_max(x, world, device="cuda"):
    """Max over the ranks of a local time (every rank gets it): the replicas
    are timed as one job, ending when the slowest ends."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, points_per_step, steps, seconds):
    """Whole-job rate of N replicas (weak scaling): all ranks' points over the
    slowest rank's time, in Gpts/s."""
    return world * points_per_step * steps / seconds / 1e9


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---- inputs (the product's host code: the reference main()'s draws) -------

_host = None


def host_lib():
    global _host
    if _host is None:
        _host = ctypes.CDLL(os.path.join(PKG, "build", "libkg_host.so"))
        _host.kgh_init.argtypes = [ctypes.c_int] * 5 + [ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p]
        _host.kgh_init.restype = None
    return _host


def shape_of(name):
    return SHAPE2 if name in kgb200.IS2D else SHAPE3


def make_inputs(names, variant=0, pinned=False, shape=None):
    """{name: (coef[6], [numpy float64 arrays])}, filled in parallel threads."""
    import numpy as np
    import torch
    from concurrent.futures import ThreadPoolExecutor

    out = {}

    def one(name):
        sh = shape or shape_of(name)
        nx, ny, ns = (sh[0], sh[1], 1) if len(sh) == 2 else sh
        n = nx * ny * ns
        narr = kgb200.load().kg_stencil_narrays(kgb200.STENCIL_ID[name])
        if pinned:
            ts = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(narr)]
            arrs = [t.numpy() for t in ts]
        else:
            ts = None
            arrs = [np.empty(n, dtype=np.float64) for _ in range(narr)]
        coef = (ctypes.c_double * 6)()
        ptrs = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in arrs])
        host_lib().kgh_init(kgb200.STENCIL_ID[name], nx, ny, ns, variant, 1, coef, ptrs)
        return name, (list(coef), arrs, ts)

    with ThreadPoolExecutor(max_workers=min(len(names), os.cpu_count() or 4)) as ex:
        for name, v in ex.map(one, names):
            out[name] = v
    return out


# ---- clocks -----------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- device-resident steps ------------------------------------------------

def run_device(args, inputs, dtype_of, want_state=False):
    """K steps (after W warm-up steps) of the suite on resident arrays.  Each
    step is the ten-sweep compute phase of every program from its initial
    inputs: the working arrays are first restored from device copies of the
    inputs, then swept with the reference's pointer rotation.  Returns the
    step time, per-stencil mean sweep time, clocks, kernel launches, whether
    every value stayed finite, the final means, and (optionally) the final
    arrays in their roles."""
    import torch

    stream = torch.cuda.current_stream()
    work, pristine, plans = {}, {}, {}
    for name in SUITE:
        coef, arrs, _ = inputs[name]
        pristine[name] = [torch.from_numpy(a).to("cuda") for a in arrs]
        work[name] = [t.clone() for t in pristine[name]]
        ptrs = [b.data_ptr() for b in work[name]]
        # each program's ten-sweep loop as one CUDA graph (tricubic: with its
        # loop-invariant weights evaluated once per replay)
        plans[name] = kgb200.Plan(kgb200.problem(name, dtype_of[name], shape_of(name), coef[:6], ptrs), NT)
    torch.cuda.synchronize()
    launches = {"n": 0}

    def one_step(events=None):
        for name in SUITE:
            for w, p0 in zip(work[name], pristine[name]):
                w.copy_(p0, non_blocking=True)
            if events is not None:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            plans[name].launch(stream)
            if events is not None:
                e1.record(stream)
                events[name].append((e0, e1))
            launches["n"] += plans[name].kernels()

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    events = {n: [] for n in SUITE}
    if args.world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    launches["n"] = 0
    t_start = torch.cuda.Event(enable_timing=True)
    t_stop = torch.cuda.Event(enable_timing=True)
    with ClockSampler(args.local_rank) as clk:
        t_start.record(stream)
        for _ in range(args.steps):
            one_step(events)
        t_stop.record(stream)
        torch.cuda.synchronize()
    if args.world > 1:
        dist.barrier()
    total_ms = t_start.elapsed_time(t_stop)
    # a TMA-engine sweep whose bounded wait gave up would have left its output
    # incomplete: fail loudly rather than report its time
    kgb200.engine_status(stream)
    # For comparison: the same step with every sweep a kg_sweep call, so the
    # tricubic sweeps evaluate their weights inline (one warm-up step, one timed).
    seqs = {}
    for name in SUITE:
        coef = inputs[name][0]
        ptrs = [b.data_ptr() for b in work[name]]
        seqs[name] = []
        for _ in range(NT):
            seqs[name].append(kgb200.problem(name, dtype_of[name], shape_of(name), coef[:6], ptrs))
            ptrs = kgb200.rotate(name, ptrs)
    lib = kgb200.load()
    sp = kgb200.stream_ptr(stream)

    def inline_step():
        for name in SUITE:
            for w, p0 in zip(work[name], pristine[name]):
                w.copy_(p0, non_blocking=True)
            for pr in seqs[name]:
                kgb200.check(lib.kg_sweep(ctypes.byref(pr), sp))

    inline_step()
    torch.cuda.synchronize()
    i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    i0.record(stream)
    inline_step()
    i1.record(stream)
    torch.cuda.synchronize()
    inline_ms = i0.elapsed_time(i1)
    # the arrays again as the timed steps leave them
    for name in SUITE:
        for w, p0 in zip(work[name], pristine[name]):
            w.copy_(p0, non_blocking=True)
        plans[name].launch(stream)
    torch.cuda.synchronize()
    per = {}
    for name in SUITE:
        # mean sweep time: the program's replay (ten sweeps; tricubic also
        # its weight pass) divided by the ten sweeps
        ds = [a.elapsed_time(b) for a, b in events[name]]
        per[name] = sum(ds) / len(ds) / NT
    finite = all(bool(torch.isfinite(b).all()) for name in SUITE for b in work[name])
    # final roles after NT sweeps and the reference's final means
    state, means = {}, {}
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for name in SUITE:
        ptrs = [b.data_ptr() for b in work[name]]
        for _ in range(NT):
            ptrs = kgb200.rotate(name, ptrs)
        by = {b.data_ptr(): b for b in work[name]}
        roles = [by[q] for q in ptrs]
        state[name] = roles
        n = roles[0].numel()
        if name == "gradient":
            fin = [roles[1], roles[2], roles[3]]
        elif name == "divergence":
            fin = [roles[0]]
        else:
            fin = [roles[1]]
        kgb200.checksum(kgb200.KG_F64, n, [t.data_ptr() for t in fin], out.data_ptr(), stream)
        means[name] = "final mean = %f" % (float(out.item()) / n / len(fin))
    del pristine
    if not want_state:
        state = None
    return total_ms, per, clk.summary(), launches["n"], finite, means, state, inline_ms


def reference_final_means():
    """The final-mean lines the reference's gcc binary printed for
    `benchmark 512 256 256 10` (tests/golden/reference_checksums.json)."""
    path = os.path.join(ROOT, "tests", "golden", "reference_checksums.json")
    try:
        runs = json.load(open(path))["runs"]
    except Exception:
        return {}
    out = {}
    for name, rs in runs.items():
        for r in rs:
            if r.get("readme_config"):
                out[name] = [ln for ln in r["lines"] if ln.startswith("final mean")][0].rstrip()
    return out


# ---- bandwidth forms: FP32 and BF16 storage, one sweep ------------------------

# Arrays read or written per sweep (the compulsory bytes are these times the
# element size).
ARRAYS_PER_PT = {"laplacian": 2, "divergence": 4, "gradient": 4, "uxx1": 6, "wave13pt": 3, "tricubic": 5,
                 "tricubic2": 5, "jacobi": 2, "lapgsrb": 2, "gaussblur": 2, "gameoflife": 2}


def run_bandwidth_forms(shape3=SHAPE3, reps=20):
    """One sweep of every stencil in FP32 and in BF16 storage (FP32
    arithmetic), engine chosen by the library, inputs uniform [-1,1) (uxx1's
    density in [1,2)), timed with CUDA events over `reps` sweeps after three
    warm-up sweeps; Gpts/s and the compulsory bytes per second against the
    measured HBM peak.  Every array is larger than L2 at this size except the
    2D tests' at 512x65536 FP32 (134 MB) and BF16 (67 MB)."""
    import torch

    hbm, kind = peaks()
    lib = kgb200.load()
    stream = torch.cuda.current_stream()
    out = {"shape_3d": list(shape3), "shape_2d": list(SHAPE2), "peak_gbs": hbm, "peak_kind": kind}
    for dname, dt, tdt, es in (("f32", kgb200.KG_F32, torch.float32, 4), ("bf16", kgb200.KG_BF16, torch.bfloat16, 2)):
        row = {}
        for name in SUITE:
            if name == "gameoflife" and dt == kgb200.KG_BF16:
                continue
            sh = SHAPE2 if name in kgb200.IS2D else shape3
            n = int(np_prod(sh))
            narr = lib.kg_stencil_narrays(kgb200.STENCIL_ID[name])
            gen = torch.Generator(device="cuda")
            gen.manual_seed(7)
            bufs = [(torch.rand(n, generator=gen, device="cuda") * 2 - 1).to(tdt) for _ in range(narr)]
            if name == "uxx1":
                bufs[2] = (1.5 + 0.5 * bufs[2].float()).to(tdt)
            coef = [0.5, 0.1, 0.05, 0.02, 0.01, 0.3][:lib.kg_stencil_ncoefs(kgb200.STENCIL_ID[name])]
            ptrs = [b.data_ptr() for b in bufs]
            seq = []
            for _ in range(6):
                seq.append(kgb200.problem(name, dt, sh, coef, ptrs))
                ptrs = kgb200.rotate(name, ptrs)
            sp = kgb200.stream_ptr(stream)
            for r in range(3):
                kgb200.check(lib.kg_sweep(ctypes.byref(seq[r % 6]), sp))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for r in range(reps):
                kgb200.check(lib.kg_sweep(ctypes.byref(seq[r % 6]), sp))
            e1.record(stream)
            torch.cuda.synchronize()
            kgb200.engine_status(stream)
            ms = e0.elapsed_time(e1) / reps
            gbs = ARRAYS_PER_PT[name] * es * n / (ms * 1e-3) / 1e9
            row[name] = {"ms_per_sweep": round(ms, 4), "gpts": round(n / (ms * 1e-3) / 1e9, 1),
                         "hbm_gbs": round(gbs, 1), "hbm_frac_of_measured": round(gbs / hbm, 3)}
            del bufs
        out[dname] = row
        torch.cuda.empty_cache()
    out["bf16_over_f32_gpts"] = {n: round(out["bf16"][n]["gpts"] / out["f32"][n]["gpts"], 2)
                                 for n in out["bf16"] if n in out["f32"]}
    return out


# ---- the full-suite workload's project-defined inputs ----------------------

def run_project_inits(reps=5):
    """gameoflife on Bernoulli(0.3) 0/1 byte cells (KG_U8, B3/S23, 512x65536)
    and tricubic/tricubic2 with offsets uniform in [0,1) (KG_F64, 512x256x256),
    each as its ten-sweep program (plan), restarted from its inputs every
    repetition.  Their bit-for-bit parity with the oracle at this size is a
    GPU test; here their time."""
    import torch

    stream = torch.cuda.current_stream()
    hbm, _ = peaks()
    out = {}
    for key, name, variant, dtype, tdt, bpp in (
            ("gameoflife_u8_bernoulli", "gameoflife", 1, kgb200.KG_U8, torch.uint8, 2),
            ("tricubic_unit_offsets", "tricubic", 2, kgb200.KG_F64, torch.float64, 40),
            ("tricubic2_unit_offsets", "tricubic2", 2, kgb200.KG_F64, torch.float64, 40)):
        coef, arrs, _ = make_inputs([name], variant=variant)[name]
        pristine = [torch.from_numpy(a).to("cuda").to(tdt) for a in arrs]
        work = [t.clone() for t in pristine]
        plan = kgb200.Plan(kgb200.problem(name, dtype, shape_of(name), coef[:6], [w.data_ptr() for w in work]), NT)
        times = []
        for r in range(reps + 1):
            for w, p0 in zip(work, pristine):
                w.copy_(p0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.launch(stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
        kgb200.engine_status(stream)
        ms = statistics.median(times) / NT
        out[key] = {"stencil": name, "dtype": "u8" if dtype == kgb200.KG_U8 else "f64",
                    "shape": list(shape_of(name)), "ms_per_sweep": round(ms, 4),
                    "gpts": round(NPTS / (ms * 1e-3) / 1e9, 2),
                    "hbm_gbs": round(bpp * NPTS / (ms * 1e-3) / 1e9, 1),
                    "hbm_frac_of_measured": round(bpp * NPTS / (ms * 1e-3) / 1e9 / hbm, 4),
                    "bytes_per_point": bpp,
                    "what": "ten-sweep program (one CUDA graph), median of %d, per sweep%s" % (
                        reps, "; weight planes evaluated once per program" if dtype == kgb200.KG_F64 else "")}
        plan.close()
        del pristine, work
        torch.cuda.empty_cache()
    return out


# ---- precision sweep (wave13pt, uxx1; FP64 / float-float / mixed / FP32 / BF16)

PRECISION_SHAPE = (1024, 512, 512)


def run_precision(shape=PRECISION_SHAPE, nsteps=100, every=10, names=("wave13pt", "uxx1")):
    """The stencils advanced nsteps time steps from a Gaussian pulse (sigma 16
    cells) + 1e-3 noise with stable coefficients, in FP64 (strict), FP64 with
    float-float arithmetic, FP64 state with FP32 increments (KG_F64_MIX), and FP32
    and BF16 storage with FP32 arithmetic, side by side.  Every `every` steps the
    newest level of each narrow form is compared with FP64's (max and RMS of
    the difference relative to max and RMS of the FP64 field) and its FP64
    checksum taken.  Returns a dict per stencil."""
    import numpy as np
    import torch

    nx, ny, ns = shape
    n = nx * ny * ns
    lib = kgb200.load()
    stream = torch.cuda.current_stream()
    sp = kgb200.stream_ptr(stream)
    all_forms = [("f64", kgb200.KG_F64, torch.float64), ("f64ff", kgb200.KG_F64_FF, torch.float64),
                 ("f64mix", kgb200.KG_F64_MIX, torch.float64),
                 ("f32", kgb200.KG_F32, torch.float32), ("bf16", kgb200.KG_BF16, torch.bfloat16)]
    out = {}
    for name in names:
        forms = all_forms
        inputs = make_inputs([name], variant=3, shape=shape)
        coef, arrs, _ = inputs[name]
        f64 = [torch.from_numpy(a).to("cuda") for a in arrs]
        del inputs, arrs
        state = {}
        for key, dt, tdt in forms:
            bufs = f64 if key == "f64" else ([t.clone() for t in f64] if tdt == torch.float64 else [t.to(tdt) for t in f64])
            state[key] = {"dt": dt, "bufs": bufs, "ptrs": [b.data_ptr() for b in bufs], "ms": 0.0,
                          "newest": None}
        out_slot = 2 if name == "wave13pt" else 1
        stats = torch.zeros(4, dtype=torch.float64, device="cuda")
        sums = torch.zeros(1, dtype=torch.float64, device="cuda")
        errs = {key: [] for key, _, _ in forms if key != "f64"}
        checks = {key: [] for key, _, _ in forms}
        for block in range(nsteps // every):
            for key, dt, _ in forms:
                st = state[key]
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(every):
                    p = kgb200.problem(name, dt, shape, coef[:6], st["ptrs"])
                    kgb200.check(lib.kg_sweep(ctypes.byref(p), sp))
                    st["newest"] = st["ptrs"][out_slot]
                    st["ptrs"] = kgb200.rotate(name, st["ptrs"])
                e1.record(stream)
                torch.cuda.synchronize()
                st["ms"] += e0.elapsed_time(e1)
            step = (block + 1) * every
            ref = state["f64"]["newest"]
            for key, dt, _ in forms:
                kgb200.checksum(dt, n, [state[key]["newest"]], sums.data_ptr(), stream)
                checks[key].append(float(sums.item()) / n)
                if key == "f64":
                    continue
                kgb200.error_stats(dt, n, state[key]["newest"], ref, stats.data_ptr(), stream)
                mx, s2, mref, sref2 = stats.tolist()
                errs[key].append([step, mx / mref if mref else 0.0,
                                  (s2 / sref2) ** 0.5 if sref2 else 0.0])
        res = {}
        t64 = state["f64"]["ms"]
        for key, dt, _ in forms:
            ms = state[key]["ms"]
            r = {"gpts": round(nsteps * n / (ms * 1e-3) / 1e9, 2), "ms_per_step": round(ms / nsteps, 4),
                 "speedup_vs_f64": round(t64 / ms, 2), "mean_every_10": [float("%.9g" % c) for c in checks[key]]}
            if key != "f64":
                r["max_rel_err"] = [float("%.3g" % e[1]) for e in errs[key]]
                r["rms_rel_err"] = [float("%.3g" % e[2]) for e in errs[key]]
            res[key] = r
        out[name] = res
        del state, f64
        torch.cuda.empty_cache()
    return out


# ---- batched uneven grids ----------------------------------------------------

BATCH_KINDS = ["laplacian", "divergence", "wave13pt", "gaussblur"]


def batch_specs(nprob=256, seed=2024):
    """nx, ny, ns log-uniform in [32, 256], stencil uniform over BATCH_KINDS
    (gaussblur as 2D nx x ny*ns).  Coefficients are drawn so that 50 steps
    stay finite in FP32: laplacian beta and wave13pt m1, m2 in [-1/6, 1/6),
    gaussblur weights in [0, 1) (its normaliser makes it a convex blur)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(nprob):
        name = BATCH_KINDS[int(rng.integers(0, 4))]
        nx, ny, ns = (int(round(float(np.exp(rng.uniform(np.log(32), np.log(256)))))) for _ in range(3))
        shape = (nx, ny * ns) if name == "gaussblur" else (nx, ny, ns)
        if name == "laplacian":
            coef = [rng.uniform(-1, 1), rng.uniform(-1, 1) / 6]
        elif name == "divergence":
            coef = list(rng.uniform(-1, 1, 3))
        elif name == "wave13pt":
            coef = [rng.uniform(-1, 1), rng.uniform(-1, 1) / 6, rng.uniform(-1, 1) / 6]
        else:
            coef = list(rng.uniform(0, 1, 6))
        specs.append((name, shape, [float(c) for c in coef]))
    return specs


def run_batched(nsteps=50, reps=3, tune_cache=None, config=None):
    """256 problems, FP32 (inputs uniform [-1,1)): one persistent launch per
    step in a captured 50-step CUDA graph, tuned tile shape and CTAs/SM,
    against 256 sequential plain launches per step (host loop, and the same
    launches captured in a graph), against the FP64 batch (tuned on its own),
    and the FP32 result's error relative to FP64 after 50 steps.  config =
    (configuration, CTAs per SM) skips the tuning of the FP32 batch."""
    import torch

    specs = batch_specs()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(2024)
    lib = kgb200.load()
    stream = torch.cuda.current_stream()
    sp = kgb200.stream_ptr(stream)
    init32, bufs32, bufs64 = [], [], []
    npts = 0
    for name, shape, coef in specs:
        n = int(np_prod(shape))
        npts += n
        narr = lib.kg_stencil_narrays(kgb200.STENCIL_ID[name])
        a = [torch.rand(n, generator=gen, device="cuda", dtype=torch.float32) * 2 - 1 for _ in range(narr)]
        init32.append(a)
        bufs32.append([x.clone() for x in a])
        bufs64.append([x.double() for x in a])

    def problems(dtype, bufs):
        return [kgb200.problem(nm, dtype, sh, cf, [x.data_ptr() for x in b]) for (nm, sh, cf), b in zip(specs, bufs)]

    def restore():
        for b, a in zip(bufs32, init32):
            for x, y in zip(b, a):
                x.copy_(y)
        for b, a in zip(bufs64, init32):
            for x, y in zip(b, a):
                x.copy_(y.double())

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, n=reps):
        fn()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(n):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / n

    out = {"problems": len(specs), "points_per_step": npts, "steps": nsteps,
           "kinds": {k: sum(1 for s in specs if s[0] == k) for k in BATCH_KINDS}}
    b32 = kgb200.Batch(problems(kgb200.KG_F32, bufs32))
    t0 = time.perf_counter()
    if config:
        b32.set_config(*config)
    else:
        b32.tune(tune_cache, stream)
    out["tune_s"] = round(time.perf_counter() - t0, 3)
    cfg = b32.config()
    out["tuned"] = {"config": cfg.shape, "bx": cfg.bx, "by": cfg.by, "kc": cfg.kc, "temporal": cfg.temporal,
                    "staged": cfg.staged, "ctas_per_sm": cfg.ctas_per_sm, "tiles": cfg.tiles,
                    "configs_tried": cfg.nshapes,
                    "what": "staged == 1: tiles of bx threads x by columns each (consecutive columns), kc planes, "
                            "inputs staged in shared memory by bulk copies; temporal == 1 and staged == 0: tiles of "
                            "bx*by threads on consecutive columns, kc planes each, loads through L1; temporal T > 1: "
                            "output blocks of bx x by x kc points evaluated T steps deep in shared memory per launch"}
    restore()
    b32.set_step(0)
    b32.capture(nsteps)
    ms = timed(lambda: b32.launch(stream))
    out["fp32_batched_graph_gpts"] = round(nsteps * npts / (ms * 1e-3) / 1e9, 2)
    # compulsory FP32 bytes of one step (each problem's arrays once, per its stencil)
    bpp32 = {"laplacian": 8, "divergence": 16, "wave13pt": 12, "gaussblur": 8}
    step_bytes = sum(bpp32[nm] * int(np_prod(sh)) for nm, sh, _ in specs)
    hbm, _ = peaks()
    out["fp32_batched_graph_hbm"] = {
        "algorithmic_bytes_per_step": step_bytes,
        "gbs": round(step_bytes * nsteps / (ms * 1e-3) / 1e9, 1),
        "frac_of_measured": round(step_bytes * nsteps / (ms * 1e-3) / 1e9 / hbm, 3),
        "note": "algorithmic bytes of the steps over their time; with temporal blocking each value crosses "
                "HBM about twice per T steps, so this can exceed the DRAM throughput"}
    ms = timed(lambda: b32.step(nsteps, stream))
    out["fp32_batched_launches_gpts"] = round(nsteps * npts / (ms * 1e-3) / 1e9, 2)

    def sequential(dtype, bufs, steps):
        sp = kgb200.stream_ptr(torch.cuda.current_stream())   # the capture stream inside a graph
        ptrs = [[x.data_ptr() for x in b] for b in bufs]
        for _ in range(steps):
            for q, (nm, sh, cf) in enumerate(specs):
                p = kgb200.problem(nm, dtype, sh, cf, ptrs[q])
                rc = lib.kg_sweep(ctypes.byref(p), sp)
                if rc:
                    kgb200.check(rc)
                ptrs[q] = kgb200.rotate(nm, ptrs[q])

    ms = timed(lambda: sequential(kgb200.KG_F32, bufs32, nsteps), n=1)
    out["fp32_sequential_host_gpts"] = round(nsteps * npts / (ms * 1e-3) / 1e9, 2)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        sequential(kgb200.KG_F32, bufs32, 6)   # 6 steps: a whole number of rotations
    ms = timed(lambda: g.replay())
    out["fp32_sequential_graph_gpts"] = round(6 * npts / (ms * 1e-3) / 1e9, 2)
    del g

    # FP64 (strict) batch and sequential, then errors after nsteps from the same inputs
    b64 = kgb200.Batch(problems(kgb200.KG_F64, bufs64))
    # the FP64 batch takes the faster of the FP32 batch's configuration and
    # the one-step tiles the tuner preferred before the staged tiles existed
    # (32x16 threads x 16 planes, 3 CTAs/SM); its sums keep it bound by the
    # FP64 unit rather than by load latency
    best64 = None
    for c in ((cfg.shape, cfg.ctas_per_sm), (7, 3)):
        b64.set_config(*c)
        ms = timed(lambda: b64.step(6, stream), n=1)
        if best64 is None or ms < best64[0]:
            best64 = (ms, c)
    b64.set_config(*best64[1])
    c64 = b64.config()
    out["tuned_fp64"] = {"config": c64.shape, "bx": c64.bx, "by": c64.by, "kc": c64.kc, "temporal": c64.temporal,
                         "staged": c64.staged, "ctas_per_sm": c64.ctas_per_sm}
    ms = timed(lambda: b64.step(6, stream), n=1)
    out["fp64_batched_gpts"] = round(6 * npts / (ms * 1e-3) / 1e9, 2)
    ms = timed(lambda: sequential(kgb200.KG_F64, bufs64, 6), n=1)
    out["fp64_sequential_host_gpts"] = round(6 * npts / (ms * 1e-3) / 1e9, 2)
    restore()
    b32.set_step(0)
    b64.set_step(0)
    b32.launch(stream)
    b64.step(nsteps, stream)
    torch.cuda.synchronize()
    stats = torch.zeros(4, dtype=torch.float64, device="cuda")
    mx = s2 = mref = sref2 = 0.0
    worst = 0.0
    per_problem = []
    for q, (nm, sh, cf) in enumerate(specs):
        p32, p64 = b32.final_roles(q), b64.final_roles(q)
        slot = {"laplacian": 0, "gaussblur": 0, "wave13pt": 1, "divergence": 0}[nm]
        n = int(np_prod(sh))
        kgb200.error_stats(kgb200.KG_F32, n, p32.arr[slot], p64.arr[slot], stats.data_ptr(), stream)
        a, b_, c, d = stats.tolist()
        mx, s2, mref, sref2 = max(mx, a), s2 + b_, max(mref, c), sref2 + d
        if c > 0:
            worst = max(worst, a / c)
            per_problem.append((a / c, q, nm, list(sh)))
    over = sorted((p for p in per_problem if p[0] > 1e-6), reverse=True)
    by_kind = {}
    for e, q, nm, sh in per_problem:
        by_kind[nm] = max(by_kind.get(nm, 0.0), e)
    out["fp32_vs_fp64_after_%d_steps" % nsteps] = {
        "max_rel": float("%.3g" % (mx / mref if mref else 0.0)),
        "rms_rel": float("%.3g" % ((s2 / sref2) ** 0.5 if sref2 else 0.0)),
        "worst_problem_max_rel": float("%.3g" % worst),
        "per_kind_worst_max_rel": {k: float("%.3g" % v) for k, v in by_kind.items()},
        "problems_over_1e-6": len(over),
        "over_1e-6": [{"problem": q, "stencil": nm, "shape": sh, "max_rel": float("%.3g" % e)}
                      for e, q, nm, sh in over[:16]],
        "note": "max_rel of a problem: max |fp32 - fp64| / max |fp64| over its newest array"}
    out["speedup_batched_graph_vs_sequential_host"] = round(
        out["fp32_batched_graph_gpts"] / out["fp32_sequential_host_gpts"], 2)
    out["speedup_batched_graph_vs_sequential_graph"] = round(
        out["fp32_batched_graph_gpts"] / out["fp32_sequential_graph_gpts"], 2)
    out["speedup_fp32_batched_vs_fp64_sequential"] = round(
        out["fp32_batched_graph_gpts"] / out["fp64_sequential_host_gpts"], 2)
    b32.close()
    b64.close()
    del bufs32, bufs64, init32
    torch.cuda.empty_cache()
    return out


# ---- mixed-precision iterative refinement (Poisson) -------------------------

IR_SHAPE = (768, 768, 512)
IR_SMALL = (192, 192, 128)


def run_ir(shape=IR_SMALL, rtol=1e-10, omega=1.8, per_check=100, fp64_cap=None, kinds=None):
    """A u = f, 7-point Laplacian, u = 0 on the outer planes, f uniform
    [-1,1) on the interior with its mean removed: time to ||f - A u|| <=
    rtol ||f|| for plain FP64 red-black SOR and for FP64 refinement around
    FP32 red-black SOR (and Jacobi, where it is given the sweeps)."""
    import torch

    nx, ny, ns = shape
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    f = torch.zeros((ns, ny, nx), dtype=torch.float64, device="cuda")
    inner = torch.rand((ns - 2, ny - 2, nx - 2), generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
    f[1:-1, 1:-1, 1:-1] = inner - inner.mean()
    del inner
    f = f.reshape(-1)
    npts = nx * ny * ns
    out = {"shape": list(shape), "rtol": rtol, "omega": omega, "sweeps_per_check": per_check}
    kinds = kinds or [("fp64_sor", kgb200.KG_SOLVE_SOR_F64, fp64_cap),
                      ("ir_fp32_sor", kgb200.KG_SOLVE_IR_SOR_F32, args.ir_sor_cap or None)]
    for key, kind, cap in kinds:
        u = torch.zeros_like(f)
        torch.cuda.synchronize()
        st, rep = kgb200.poisson_solve(shape, f.data_ptr(), u.data_ptr(), kind, omega=omega, rtol=rtol,
                                       sweeps_per_check=per_check, max_sweeps=cap or 10**7,
                                       raise_on_timeout=False)
        r = {"status": kgb200.STATUS[st], "sweeps": rep.sweeps, "seconds": round(rep.seconds, 3),
             "rel_residual": float("%.3g" % rep.rel_residual), "outer": rep.outer,
             "ms_per_sweep": round(rep.seconds * 1e3 / max(rep.sweeps, 1), 4),
             "gpts": round(rep.sweeps * npts / max(rep.seconds, 1e-9) / 1e9, 2)}
        out[key] = r
        del u
    # time to tolerance against FP64 SOR run to tolerance; where the FP64 run
    # was capped, only the per-sweep ratio (refinement around FP32 SOR needs
    # the same sweeps as FP64 SOR: 63,400 both at 768x768x512)
    base = out["fp64_sor"]
    for key in list(out):
        if isinstance(out[key], dict) and key != "fp64_sor" and out[key].get("status") == "KG_OK":
            if base["status"] == "KG_OK":
                out[key]["speedup_vs_fp64_sor"] = round(base["seconds"] / out[key]["seconds"], 2)
            else:
                out[key]["per_sweep_speedup_vs_fp64_sor"] = round(base["ms_per_sweep"] / out[key]["ms_per_sweep"], 2)
    torch.cuda.empty_cache()
    return out


def np_prod(shape):
    r = 1
    for v in shape:
        r *= int(v)
    return r


# ---- end to end through the C ABI with host buffers -----------------------

E2E_LANES = (2, 2)   # host threads for compute-heavy / copy-heavy programs


def run_e2e(args, dtype, lanes=E2E_LANES):
    """The 11 programs through kg_program_run on pinned host arrays, one step =
    every program once, each from the initial inputs (restored on the host
    between steps, outside the timed steps: kg_program_run writes its results
    back into the host arrays, as the reference's programs do).

    Each program runs on a host thread with its own stream; kg_program_run
    orders every phase on its stream and waits once.  The two tricubic
    programs (252 FP64 operations per 40 bytes) go to lanes[0] threads with
    normal-priority streams, the other nine (at most 31 operations per 16
    bytes, so their copies weigh as much as their sweeps) to lanes[1] threads
    with high-priority streams: their copies run under the tricubic sweeps and
    their own sweeps are not queued behind them.  Returns the summed step
    times, the copied bytes, each step's time, whether the tricubic programs
    took their weights once, and the slowest step's per-program times (call
    wall time and the load, compute and save phases, ms)."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    inputs = make_inputs(SUITE, pinned=True)
    pristine = {name: [a.copy() for a in inputs[name][1]] for name in SUITE}
    pairs = [(w, p) for name in SUITE for w, p in zip(inputs[name][1], pristine[name])]
    n_heavy, n_light = lanes
    streams = [torch.cuda.Stream(priority=0) for _ in range(n_heavy)] + \
              [torch.cuda.Stream(priority=-1) for _ in range(n_light)]   # -1: high priority
    h2d = d2h = 0
    for name in SUITE:
        coef, arrs, _ = inputs[name]
        h2d += sum(a.nbytes for a in arrs)
        d2h += bin(result_mask(name)).count("1") * arrs[0].nbytes
    heavy = [n for n in SUITE if FP64_OPS_PER_PT[n] > 4 * BYTES_PER_PT[n]]
    # largest first within each class, so the lanes finish together
    light = sorted((n for n in SUITE if n not in heavy), key=lambda nm: -(FP64_OPS_PER_PT[nm] + 2 * BYTES_PER_PT[nm]))
    if n_light == 0:
        heavy, light = heavy + light, []
    errors, once, phases = [], [], {}

    def lane(k, todo, lock):
        try:
            while True:
                with lock:
                    if not todo:
                        return
                    name = todo.pop(0)
                coef, arrs, _ = inputs[name]
                p = kgb200.problem(name, dtype, shape_of(name), coef[:6], [a.ctypes.data for a in arrs])
                w0 = time.perf_counter()
                t = kgb200.program_run(p, NT, result_mask(name), streams[k])
                phases[name] = [round((time.perf_counter() - w0) * 1e3, 1), round(t.load * 1e3, 1),
                                round(t.compute * 1e3, 1), round(t.save * 1e3, 1)]
                if name in heavy:
                    once.append(t.weights_once)
        except Exception as e:  # surfaced after the join
            errors.append(e)

    def step():
        hq, lq, hl, ll = list(heavy), list(light), threading.Lock(), threading.Lock()
        ts = [threading.Thread(target=lane, args=(k, hq, hl)) for k in range(n_heavy)] + \
             [threading.Thread(target=lane, args=(n_heavy + k, lq, ll)) for k in range(n_light)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        if errors:
            raise errors[0]

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        def restore():
            list(ex.map(lambda wp: np.copyto(wp[0], wp[1]), pairs))

        for _ in range(max(1, min(args.warmup, 2))):
            restore()
            step()
        dt, each, slowest = 0.0, [], None
        for _ in range(args.steps):
            restore()
            phases.clear()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step()
            torch.cuda.synchronize()
            each.append(time.perf_counter() - t0)
            dt += each[-1]
            if each[-1] >= max(each):
                slowest = dict(phases)
    del inputs, pristine, pairs
    return dt, h2d, d2h, each, all(once), slowest


# ---- the suite's other tests (vecadd, matvec, matmul, sincos, whispering) ----

OTHER = {   # command line of the suite's own size; compulsory bytes and FP64 operations per step
    "vecadd": ((512, 256, 256), lambda a: 24 * a[0] * a[1] * a[2], lambda a: a[0] * a[1] * a[2]),
    "matvec": ((512, 65536), lambda a: 8 * (a[0] * a[1] + a[0] + a[1]), lambda a: 2 * a[0] * a[1]),
    "matmul": ((512, 256, 256), lambda a: 8 * (a[0] * a[1] + a[1] * a[2] + 2 * a[0] * a[2]),
               lambda a: 2 * a[0] * a[1] * a[2]),
    "sincos": ((512, 256, 256), lambda a: 24 * a[0] * a[1] * a[2], lambda a: 0),
    "whispering": ((512, 65536), lambda a: 96 * a[0] * a[1], lambda a: 33 * a[0] * a[1]),
}


def run_other(reps=10):
    """Device time of one step of each test at the suite's size (strict FP64 and
    FP32), with the roofline of its bound, and the oracle's fast-math build on
    the host cores for a CPU reference point."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol

    hbm_peak, _ = peaks()
    out = {}
    for name, (args, nbytes, nops) in OTHER.items():
        init, coef, _, _ = ol.extra_program(name, tuple(args) + (0,), flavour="fast")
        row = {"args": list(args)}
        for dname, dt, tdt in (("f64", kgb200.KG_F64, torch.float64), ("f32", kgb200.KG_F32, torch.float32)):
            bufs = [torch.from_numpy(a).cuda().to(tdt) for a in init]
            ptrs = [b.data_ptr() for b in bufs]
            for _ in range(2):
                kgb200.extra_step(name, dt, args, ptrs, coef)
            torch.cuda.synchronize()
            best = 1e30
            for _ in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    kgb200.extra_step(name, dt, args, ptrs, coef)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1) / reps * 1e-3)
            b = nbytes(args) * (4 if dt == kgb200.KG_F32 else 8) / 8
            r = {"ms_per_step": round(best * 1e3, 4), "hbm_gbs": round(b / best / 1e9, 1),
                 "hbm_frac_of_measured": round(b / best / 1e9 / hbm_peak, 3)}
            if dt == kgb200.KG_F64 and nops(args):
                r["fp64_tops"] = round(nops(args) / best / 1e12, 3)
            row[dname] = r
            del bufs
        t0 = time.perf_counter()
        ol.extra_program(name, tuple(args) + (1,), flavour="fast")
        t1 = time.perf_counter()
        ol.extra_program(name, tuple(args) + (0,), flavour="fast")
        t2 = time.perf_counter()
        row["cpu_oracle_ms_per_step"] = round(max((t1 - t0) - (t2 - t1), 1e-9) * 1e3, 2)
        row["speedup_f64_vs_cpu"] = round(row["cpu_oracle_ms_per_step"] / row["f64"]["ms_per_step"], 1)
        out[name] = row
    out["matmul_tc"] = run_matmul_tc()
    out["note"] = ("one step at the suite's problem size; KG_F64 bitwise equal to the oracle; CPU: the oracle's "
                   "fast-math build on the host cores (step time = program time minus its init)")
    return out


def run_matmul_tc(sizes=((512, 256, 256), (4096, 4096, 4096)), reps=5):
    """kg_matmul_tc (FP32 arrays on the tensor cores, three TF32 MMAs per
    product) at the suite's size and at 4096^3, beside kg_matmul's FP32 SIMT
    kernel at the suite's size; FP32-accurate TFLOP/s count 2 nx ny ns, the
    TF32 MMA rate three times that, against half the measured dense BF16
    rate (the TF32 tensor rate)."""
    import torch

    lib = kgb200.load()
    bf16 = None
    try:
        with open(PEAKS_FILE) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
    except Exception:
        pass
    out = {}
    for nx, ny, ns in sizes:
        g = torch.Generator(device="cuda")
        g.manual_seed(nx + ny + ns)
        A = torch.rand(nx * ny, generator=g, device="cuda") * 2 - 1
        B = torch.rand(ny * ns, generator=g, device="cuda") * 2 - 1
        C = torch.zeros(nx * ns, device="cuda")
        calls = {"tc": lambda: lib.kg_matmul_tc(nx, ny, ns, A.data_ptr(), B.data_ptr(), C.data_ptr(), None)}
        if nx * ny * ns <= 512 * 256 * 256:
            calls["simt_f32"] = lambda: lib.kg_matmul(kgb200.KG_F32, nx, ny, ns, A.data_ptr(), B.data_ptr(),
                                                       C.data_ptr(), None)
        row = {}
        for key, f in calls.items():
            for _ in range(2):
                kgb200.check(f())
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                kgb200.check(f())
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            flops = 2.0 * nx * ny * ns
            r = {"ms": round(ms, 4), "tflops_fp32_accurate": round(flops / ms / 1e9, 1)}
            if key == "tc":
                r["tf32_mma_tflops"] = round(3 * flops / ms / 1e9, 1)
                if bf16:
                    r["tf32_frac_of_half_measured_bf16"] = round(3 * flops / ms / 1e9 / (bf16 / 2), 3)
            row[key] = r
        kgb200.engine_status()
        out["x".join(map(str, (nx, ny, ns)))] = row
        del A, B, C
        torch.cuda.empty_cache()
    return out


# ---- CPU baseline (the oracle built with the suite's flags) ---------------

class CpuSuite:
    """The suite's programs on the host cores: the oracle's C restatement of
    the reference kernels built with the suite's -O3 -ffast-math flags and
    OpenMP (liboracle_fast.so), its inputs drawn by the oracle itself as the
    reference main() draws them (glibc rand(), default seed), so that no
    product library is loaded.  A step is the same as the GPU arm's: ten
    sweeps of each of the eleven programs with the reference's rotation, each
    program restarted from its initial inputs (restored outside the timing)."""

    def __init__(self):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib as ol

        self.lib = ol.load("fast")
        self.cases, self.pristine, self.roles = {}, {}, {}
        for name in SUITE:
            c = ol.Case(name, shape_of(name), flavour="fast")
            self.cases[name] = c
            self.pristine[name] = [b.copy() for b in c.buffers]
            self.roles[name] = ([c.c.arr[q] for q in range(6)], [c.c.order[q] for q in range(6)])

    def restore(self, name):
        import numpy as np
        c = self.cases[name]
        for b, p0 in zip(c.buffers, self.pristine[name]):
            np.copyto(b, p0)
        arr, order = self.roles[name]
        for q in range(6):
            c.c.arr[q] = arr[q]
            c.c.order[q] = order[q]

    def threads(self):
        return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    def step(self, sweeps=NT):
        """Seconds of one step (sweeps per program, every program)."""
        dt = 0.0
        for name in SUITE:
            self.restore(name)
            c = self.cases[name]
            t0 = time.perf_counter()
            self.lib.or_run(ctypes.byref(c.c), sweeps)
            dt += time.perf_counter() - t0
        return dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    cpu = CpuSuite()
    for _ in range(args.warmup):
        cpu.step()
    total = 0.0
    for _ in range(args.steps):
        total += cpu.step()
    value = 11 * NT * NPTS * args.steps / total / 1e9
    threads = cpu.threads()
    sample = ("every step whole: 10 sweeps of each of the 11 programs from their initial inputs "
              "(512x256x256 / 512x65536, FP64), inputs restored between steps outside the timing")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Gpts/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": dict(CONFIG, sample=sample,
                       implementation="the reference kernels' C restatement (oracle) with the suite's gcc "
                                      "flags -O3 -ffast-math and OpenMP over %d host threads; tricubic and "
                                      "tricubic2 evaluate their weights in every sweep, as the reference "
                                      "does" % threads),
        "cpu_baseline": {"value": round(value, 4), "unit": "Gpts/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


METRIC = "Gpts/s, full suite plain FP64 (11 stencils x 10 sweeps, 512x256x256; 2D 512x65536)"
DATA = "synthetic: the reference main()'s glibc rand() draws, default seed"
CONFIG = {"workload": "suite-fp64 benchmark 512 256 256 10 (11 stencils x 10 sweeps per step, "
                      "each program restarted from its initial inputs by a device copy and run as one CUDA "
                      "graph; tricubic/tricubic2 programs evaluate their loop-invariant weight products once "
                      "per run, inside the step)",
          "shape_3d": list(SHAPE3), "shape_2d": list(SHAPE2), "sweeps_per_step": 11 * NT,
          "points_per_sweep": NPTS, "l2": "no flush: every array (268 MB) is larger than L2 (129 MB)",
          "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dtype", default="f64", choices=["f64", "f64fma"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the precision-sweep summary")
    ap.add_argument("--workload", default="suite", choices=["suite", "precision", "batched", "ir", "bandwidth"])
    ap.add_argument("--ir-shape", default="768,768,512")
    ap.add_argument("--batch-config", default="",
                    help="--workload batched: 'configuration,ctas_per_sm' instead of tuning the FP32 batch")
    ap.add_argument("--ir-fp64-cap", type=int, default=0, help="sweep cap of the FP64 SOR run (0: none)")
    ap.add_argument("--ir-jacobi-cap", type=int, default=0,
                    help="sweep cap of the refinement run with FP32 Jacobi sweeps (0: not run)")
    ap.add_argument("--ir-sor-cap", type=int, default=0,
                    help="sweep cap of the refinement run with FP32 red-black SOR sweeps (0: none)")
    args = ap.parse_args()
    args.world, args.rank, args.local_rank = dist_env()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    if args.world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(args.local_rank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    kgb200.check(kgb200.load().kg_device_check())
    dtype = kgb200.DTYPES[args.dtype]
    if args.workload == "ir":
        shape = tuple(int(v) for v in args.ir_shape.split(","))
        kinds = [("fp64_sor", kgb200.KG_SOLVE_SOR_F64, args.ir_fp64_cap or None),
                 ("ir_fp32_sor", kgb200.KG_SOLVE_IR_SOR_F32, args.ir_sor_cap or None)]
        if args.ir_jacobi_cap:
            kinds.append(("ir_fp32_jacobi", kgb200.KG_SOLVE_IR_JACOBI_F32, args.ir_jacobi_cap))
        res = run_ir(shape, kinds=kinds)
        if args.rank == 0:
            print(json.dumps({"workload": "mixed-precision iterative refinement, Poisson 7-point", "forms": res}))
        return 0
    if args.workload == "batched":
        res = run_batched(tune_cache=os.environ.get("KG_TUNE_CACHE"),
                          config=tuple(int(v) for v in args.batch_config.split(",")) if args.batch_config else None)
        if args.rank == 0:
            print(json.dumps({"workload": "batched: 256 problems, log-uniform sizes in [32,256], "
                              "{laplacian, divergence, wave13pt, gaussblur}, FP32, 50 steps", "forms": res}))
        return 0
    if args.workload == "bandwidth":
        res = run_bandwidth_forms()
        if args.rank == 0:
            print(json.dumps({"workload": "FP32 and BF16 storage, one sweep per stencil", "forms": res}))
        return 0
    if args.workload == "precision":
        res = run_precision()
        if args.rank == 0:
            print(json.dumps({"workload": "precision sweep wave13pt/uxx1 1024x512x512, 100 steps, "
                              "Gaussian pulse sigma 16 + 1e-3 noise", "forms": res}))
        return 0

    inputs = make_inputs(SUITE)
    dtype_of = {n: dtype for n in SUITE}
    total_ms, per, clocks, launches, finite, means, state, inline_ms = run_device(
        args, inputs, dtype_of, want_state=not args.no_forms)
    ref_means = reference_final_means()
    checks = {n: {"gpu": means[n], "reference": ref_means.get(n), "match": means[n] == ref_means.get(n)}
              for n in SUITE if n in ref_means}
    ff_form = None
    if not args.no_forms:
        # the same steps with float-float arithmetic (gameoflife stays strict:
        # it must be bit-exact), and its error against the strict arrays
        ff_of = {n: (kgb200.KG_F64 if n == "gameoflife" else kgb200.KG_F64_FF) for n in SUITE}
        fms, fper, _, _, ffinite, fmeans, fstate, _ = run_device(args, inputs, ff_of, want_state=True)
        stats = torch.zeros(4, dtype=torch.float64, device="cuda")
        errs = {}
        for n in SUITE:
            worst = 0.0
            for a, b in zip(fstate[n], state[n]):
                kgb200.error_stats(kgb200.KG_F64, a.numel(), a.data_ptr(), b.data_ptr(), stats.data_ptr())
                mx, _, mref, _ = stats.tolist()
                worst = max(worst, mx / mref if mref else mx)
            errs[n] = float("%.3g" % worst)
        ff_form = {
            "what": "the same suite steps with FP64 storage and float-float arithmetic on the FP32 pipes "
                    "(KG_F64_FF; gameoflife strict FP64)",
            "value": round(11 * NT * NPTS * args.steps / (fms * 1e-3) / 1e9, 4), "unit": "Gpts/s",
            "speedup_vs_strict": round(total_ms / fms, 2),
            "max_normwise_err_vs_strict_fp64": errs,
            "ms_per_sweep": {n: round(fper[n], 4) for n in SUITE},
            "final_means_match_reference": sum(1 for n in SUITE if n in ref_means and fmeans[n] == ref_means[n]),
            "finite": ffinite}
        del fstate
    del inputs, state
    torch.cuda.empty_cache()
    total_ms = replica_max(total_ms, args.world)

    pts_per_step = 11 * NT * NPTS
    value = replica_value(args.world, pts_per_step, args.steps, total_ms * 1e-3)
    ms_per_step = total_ms / args.steps

    # dominant kernel: the largest share of the step
    share = {n: per[n] * NT for n in SUITE}
    dom = max(share, key=share.get)
    hbm, hbm_kind = peaks()
    dur = per[dom] * 1e-3
    achieved = BYTES_PER_PT[dom] * NPTS / dur / 1e9
    fp64_ops = FP64_OPS_PER_PT[dom] * NPTS / dur
    fp64_peak = kgb200.measure_peaks().fp64_ops
    roofline = {
        "kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
        "unit": "GB/s", "frac": round(achieved / hbm, 4), "peak_kind": hbm_kind,
        "traffic": NCU_TRAFFIC.get(dom),
        "bytes_per_launch": BYTES_PER_PT[dom] * NPTS, "launch_ms": round(per[dom], 4),
        "fp64_alu": {"achieved_tops": round(fp64_ops / 1e12, 4), "peak_tops": round(fp64_peak / 1e12, 4),
                     "frac": round(fp64_ops / fp64_peak, 4), "peak_kind": "measured live (kg_measure_peaks, DFMA)",
                     "note": "the FP64 sweeps are bound by GB300's FP64 issue rate, not HBM; achieved_tops counts "
                             "the operations of the reference's per-sweep expression, and tricubic programs "
                             "evaluate their loop-invariant weights once per program (their sweeps read 64 "
                             "precomputed planes, which is the DRAM traffic above), so it exceeds the unit's peak"},
    }
    per_stencil = {n: {"ms_per_sweep": round(per[n], 4), "gpts": round(NPTS / (per[n] * 1e-3) / 1e9, 2),
                       "hbm_gbs": round(BYTES_PER_PT[n] * NPTS / (per[n] * 1e-3) / 1e9, 1),
                       "fp64_tops": round(FP64_OPS_PER_PT[n] * NPTS / (per[n] * 1e-3) / 1e12, 4),
                       "share": round(share[n] / sum(share.values()), 4)} for n in SUITE}

    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "Gpts/s", "n_gpus": args.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.dtype, "data": DATA, "config": CONFIG, "roofline": roofline,
        "gpu_launches": launches, "clocks": clocks, "finite": finite, "per_stencil": per_stencil,
        "final_means_vs_reference": {"matched": sum(1 for c in checks.values() if c["match"]),
                                     "of": len(checks), "lines": checks},
        "weights_per_sweep": {
            "value": round(pts_per_step / (inline_ms * 1e-3) / 1e9, 4), "unit": "Gpts/s",
            "ms_per_step": round(inline_ms, 3),
            "note": "the same step with every sweep a kg_sweep call: tricubic and tricubic2 evaluate their "
                    "weights in every sweep instead of once per program run (a, b, c are constant during the "
                    "time loop; the timed steps above evaluate them once per run, inside the timed step, and "
                    "produce the same bits)"},
    }
    if not args.no_e2e:
        dt, h2d, d2h, each, once, slowest = run_e2e(args, dtype)
        dt = replica_max(dt, args.world)
        line["e2e"] = {"value": round(replica_value(args.world, pts_per_step, args.steps, dt), 4), "unit": "Gpts/s",
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "step_ms": [round(t * 1e3, 1) for t in each], "tricubic_weights_once": once,
                       "slowest_step_ms_by_program": {"fields": ["call", "load", "compute", "save"], **(slowest or {})},
                       "path": "kg_program_run per stencil (stream-ordered alloc, H2D, 10 sweeps, D2H of the "
                               "checksum arrays, free) on pinned host arrays; the 11 programs on %d host threads with a "
                               "stream each (tricubic/tricubic2 on %d normal-priority, the rest on %d high-priority)"
                               % (sum(E2E_LANES), E2E_LANES[0], E2E_LANES[1])}
    if not args.no_forms:
        line["forms"] = {"fp64_float_float": ff_form, "precision_sweep": dict(
            workload="wave13pt and uxx1, 1024x512x512, 100 steps from a Gaussian pulse (sigma 16) + 1e-3 noise; "
                     "FP64 strict vs float-float (f64ff), FP64 state with FP32 increments (f64mix), FP32 and "
                     "BF16 storage (FP32 arithmetic); errors relative to FP64 every 10 steps",
            **run_precision())}
        line["forms"]["batched"] = run_batched(tune_cache=os.environ.get("KG_TUNE_CACHE"))
        line["project_inits"] = run_project_inits()
        line["forms"]["bandwidth"] = run_bandwidth_forms()
        line["forms"]["iterative_refinement"] = dict(
            note="measured to tolerance on 192x192x128; the 768x768x512 run is bench.py --workload ir",
            **run_ir(IR_SMALL, kinds=[("fp64_sor", kgb200.KG_SOLVE_SOR_F64, None),
                                      ("ir_fp32_sor", kgb200.KG_SOLVE_IR_SOR_F32, None),
                                      ("ir_fp32_jacobi", kgb200.KG_SOLVE_IR_JACOBI_F32, 400000)]))
        line["other_tests"] = run_other()
    if args.rank == 0 and args.world == 1 and not args.no_cpu:
        cpu = CpuSuite()
        cpu.step()                       # warm-up
        dt = cpu.step()
        g = 11 * NT * NPTS / dt / 1e9
        threads = cpu.threads()
        line["cpu_baseline"] = {"value": round(g, 4), "unit": "Gpts/s", "cores": threads, "kind": "port",
                                "sample": "one step: 10 sweeps of each of the 11 programs (110 full-size "
                                          "sweeps), after one warm-up step"}
        # the suite's gcc target runs serially: one sweep of each stencil on one core
        cpu.lib.or_set_threads(1)
        dt1 = cpu.step(sweeps=1)
        cpu.lib.or_set_threads(threads)
        line["cpu_baseline_1core"] = {"value": round(11 * NPTS / dt1 / 1e9, 4), "unit": "Gpts/s", "cores": 1,
                                      "kind": "port", "sample": "one full-size sweep of each of the 11 stencils"}
        line["weights_per_sweep"]["vs_cpu_baseline"] = round(line["weights_per_sweep"]["value"] / g, 2)
        line["value_vs_cpu_baseline"] = round(line["value"] / g, 2)
        del cpu
    if args.rank == 0:
        print(json.dumps(line))
    if args.world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
