"""Benchmark: GIAO shell-quartet ERIs on one GB300 (and N independent ranks).

Workload: the 12-atom seeded molecule (seed 2026, atoms uniform in a 10-bohr
cube, min separation 1.8 bohr, shells s(6) s(1) s(1) p(3) p(1) d(1), exponents
log-uniform in [0.1, 5000]) at a seeded field |B| <= 0.2, every canonical
shell quartet (all classes up to (dd|dd)): 6,722,352 quartets,
262,790,892 complex128 ERIs per step.  A step evaluates all of them into
device memory (``value``: inputs resident in HBM) or, for ``e2e``, through the
host-buffer C ABI call gx_eri_batch with the quartet list and the 4.2 GB of
results crossing host<->device inside the timed region.

Under torchrun each rank runs the same job at its own field of a seeded
field grid (the path shards into independent field evaluations; no
collective on the data path) and ``value`` is all ranks' ERIs over the
slowest rank's time.

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement in oracle/ (the reference's own compiled library does
not travel to the GPU host), with all host threads, on a bounded seeded
sample of the same quartets per step.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GIAO ERIs/s & Cholesky time, mixed vs FP64 GPU @1e-10; p50/p99 req latency"
UNIT = "ERIs/s"
WORKLOAD = "12-atom s6 s1 s1 p3 p1 d1 molecule, seed 2026, |B|<=0.2, all 6722352 canonical quartets, complex128"
DTYPE = "f64+f32 (mixed: FP32 primitive quartets under the cutoff, FP64 elsewhere and for every sum)"


# DRAM bytes (read + write) of one plan execution of this workload, from one
# ncu capture of every launch of one step (dram__bytes_read.sum +
# dram__bytes_write.sum summed over the 116 (mixed) / 81 (FP64) class
# launches, L2 kept across launches; pair-record kernels excluded: they run
# once per field):
#   ncu --nvtx --nvtx-include "step/" --cache-control none --clock-control none
#       --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
#       python bench.py --profile-step {mixed,fp64} --no-autotune --warmup 0 --no-cpu
TRAFFIC_PER_STEP: dict = {"mixed": 914.9e6 + 4949.6e6, "fp64": 778.4e6 + 4782.2e6}
TRAFFIC_BASIS = ("ncu dram__bytes_read.sum + dram__bytes_write.sum over every class launch of one step "
                 "(untuned launch configurations, L2 kept across launches); algorithmic output 4.20 GB per step")


def _measured_peaks() -> dict:
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


MEASURED = _measured_peaks()


def config_block(natoms: int) -> dict:
    """The workload description shared by both arms (same keys and values)."""
    return {"workload": WORKLOAD if natoms == 12 else WORKLOAD.replace("12-atom", f"{natoms}-atom"),
            "molecule_seed": 2026, "field": "seeded, |B| <= 0.2", "quartets": "all canonical",
            "l2": "flushed (256 MB write) between timed GPU steps; the 4.2 GB output is also larger than L2"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    p.add_argument("--mixed-cutoff", type=float, default=1e-6)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-cholesky", action="store_true")
    p.add_argument("--no-autotune", action="store_true", help="keep the default per-class launch configurations")
    p.add_argument("--natoms", type=int, default=12)
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-derivatives", action="store_true")
    p.add_argument("--derivatives-only", action="store_true",
                   help="run only the centre-derivative leg and print its JSON (profiling)")
    p.add_argument("--derivative-quartets", type=int, default=200000)
    p.add_argument("--cholesky-only", action="store_true",
                   help="run only the Cholesky leg (no CPU port) and print its JSON (profiling)")
    p.add_argument("--serving-requests", type=int, default=32)
    p.add_argument("--serving-request-gib", type=float, default=6.0,
                   help="per-request device-memory limit of the serving leg (estimated footprint; GiB)")
    p.add_argument("--profile-e2e", action="store_true",
                   help="three gx_eri_batch host-output calls, the third inside an NVTX range 'call', then exit")
    p.add_argument("--profile-step", default="", choices=["", "fp64", "mixed", "fp64_exact"],
                   help="run warm-up steps and one step of this mode inside an NVTX range, then exit (profiling)")
    p.add_argument("--sweep", type=int, default=64,
                   help="field sweep: evaluate the molecule at this many fields |B| <= 0.5 in FP64 and mixed")
    p.add_argument("--sweep-oracle-quartets", type=int, default=4000,
                   help="seeded canonical quartets per sweep field compared with the CPU oracle")
    p.add_argument("--sweep-cholesky", type=int, default=2, help="fields of the sweep that also run Cholesky 1e-6")
    p.add_argument("--sweep-cholesky-pivots", type=int, default=48,
                   help="leading pivots of each sweep Cholesky compared with the CPU oracle's")
    return p.parse_args()


def dist_env():
    from giaoint_gb300.replicas import dist_env as env

    return env()


def workload(natoms: int, rank: int):
    """The 12-atom molecule (seed 2026) and this rank's field (replicas: one
    field per rank, no data-path collective)."""
    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.replicas import field_for_rank

    recs = syn.random_molecule(2026, natoms=natoms)
    return recs, field_for_rank(rank)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, flag in zip(names, f[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample_rate(recs, B, quartets, target_seconds: float, seed: int = 1, threads: int | None = None,
                    keep: bool = False):
    """Oracle (CPU port of the reference) on a bounded seeded quartet sample.
    With ``keep``, the sample's quartet indices and ERI values are returned
    too (for the full-size parity check of the GPU outputs)."""
    from oracle import oracle as O

    orc = O.Oracle()
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    probe_n = min(len(quartets), 2000 if threads > 1 else 300)
    probe = quartets[np.sort(rng.choice(len(quartets), probe_n, replace=False))]
    t0 = time.perf_counter()
    orc.eri_batch(recs, probe, B, None, threads)
    rate = probe_n / max(time.perf_counter() - t0, 1e-6)
    count = int(min(len(quartets), max(probe_n, rate * target_seconds)))
    idx = np.sort(rng.choice(len(quartets), count, replace=False))
    t0 = time.perf_counter()
    vals, _ = orc.eri_batch(recs, quartets[idx], B, None, threads)
    dt = time.perf_counter() - t0
    out = {"value": len(vals) / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{count} seeded canonical quartets ({len(vals)} ERIs) of the same molecule and field, "
                     f"{dt:.2f} s on {threads} threads (oracle/giao_oracle.c, OpenMP)",
           "quartets_per_s": count / dt}
    if keep:
        return out, idx, vals
    return out


def gather_blocks(out_c, offsets, idx):
    """Packed values of quartets ``idx`` (sorted indices into the plan's
    quartet list) from the device output ``out_c`` (complex128), in order."""
    import torch

    starts = offsets[idx]
    lens = offsets[idx + 1] - starts
    firsts = np.concatenate(([0], np.cumsum(lens)[:-1]))
    pos = np.repeat(starts - firsts, lens) + np.arange(int(lens.sum()), dtype=np.int64)
    return out_c.index_select(0, torch.from_numpy(pos).to(out_c.device)).cpu().numpy()


def pivot_agreement(recs, field_int, gpu_pivots, gpu_vectors, ref, threads: int, gap: float = 1e-10) -> dict:
    """Pivots of the GPU factorisation against the oracle's: the common
    prefix, and at the first divergence the residual-diagonal gap of the two
    choices from the oracle's own factors (pivots must agree wherever that
    gap exceeds 1e-10); the largest factor difference over the common prefix."""
    from oracle import oracle as O

    n = gpu_vectors.shape[1]
    m = min(len(ref.pivots), len(gpu_pivots))
    k = 0
    while k < m and tuple(ref.pivots[k]) == tuple(gpu_pivots[k]):
        k += 1
    out = {"compared_pivots": m, "pivots_equal_prefix": k,
           "max_abs_vector_diff_prefix": float(np.abs(gpu_vectors[:k] - ref.vectors[:k]).max()) if k else 0.0}
    if k < m:
        L = ref.vectors[:k].reshape(k, n * n)
        pairs = [(a_, b_) for a_ in range(len(recs)) for b_ in range(a_, len(recs))]
        diag = O.Oracle().cholesky_diagonal(recs, pairs, tuple(field_int), (0.0, 0.0, 0.0), threads).ravel()
        rk = diag - (np.abs(L) ** 2).sum(axis=0)  # the residual diagonal before pivot k
        a = int(ref.pivots[k][0]) * n + int(ref.pivots[k][1])
        b = int(gpu_pivots[k][0]) * n + int(gpu_pivots[k][1])
        out["first_divergence_residual_gap"] = float(abs(rk[a] - rk[b]))
        out["first_divergence_is_tie"] = bool(abs(rk[a] - rk[b]) <= gap)
    else:
        out["first_divergence_is_tie"] = True
    return out


def reconstruction_error(res, basis, field, ctx, count: int = 24, seed: int = 11) -> float:
    """Largest |(mu nu|lam sig) - sum_P L[P,mu,nu] conj(L[P,sig,lam])| over
    seeded shell quartets, against FP64-exact GPU ERI blocks (size-independent
    check: bounded by the final residual diagonal)."""
    from giaoint_gb300.eri import _eri_batch

    rng = np.random.default_rng(seed)
    ns = len(basis.shells)
    qs = rng.integers(0, ns, size=(count, 4))
    _, shapes, offs, vals, _, _ = _eri_batch(basis, qs, field=field, precision="fp64_exact", context=ctx)
    off = basis.ao_offsets
    err = 0.0
    for i, q in enumerate(qs):
        sl = tuple(slice(off[x], off[x] + basis.shells[x].ao_count) for x in q)
        blk = vals[offs[i]:offs[i + 1]].reshape(tuple(shapes[i]))
        err = max(err, float(np.abs(res.reconstruct(sl) - blk).max()))
    return err


def cholesky_roofline(stats: dict, peak64: float) -> dict:
    """Rooflines of one factorisation: the column evaluations against the
    FP64 peak (FLOP model of the primitive quartets evaluated), the factor
    update against HBM (algorithmic bytes: L read once per pivot) and FP64."""
    col_s = stats["column_ms"] * 1e-3
    upd_s = stats["update_ms"] * 1e-3
    hbm = float(MEASURED.get("hbm_gbs") or 6800.0)
    col_tf = stats["column_model_flops"] / col_s / 1e12 if col_s > 0 else 0.0
    upd_gbs = stats["update_bytes"] / upd_s / 1e9 if upd_s > 0 else 0.0
    upd_tf = stats["update_flops"] / upd_s / 1e12 if upd_s > 0 else 0.0
    return {"columns": {"bound": "fp64", "achieved": col_tf, "peak": peak64, "unit": "TFLOP/s",
                        "frac": col_tf / peak64 if peak64 else None, "ms": stats["column_ms"],
                        "block_evaluations": stats["block_evaluations"]},
            "update": {"bound": "hbm", "achieved": upd_gbs, "peak": hbm, "unit": "GB/s", "frac": upd_gbs / hbm,
                       "fp64_tflops": upd_tf, "fp64_frac": upd_tf / peak64 if peak64 else None,
                       "ms": stats["update_ms"], "bytes": stats["update_bytes"], "flops": stats["update_flops"],
                       "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"}}


def cholesky_leg(gi, nat, ctx, run_cpu: bool, peak64: float):
    """Streamed pivoted Cholesky of the 140-AO atom (10s 8p 6d 4f 2g, ratio
    2.5 from 0.05) at B = (0, 0, 0.1), threshold 1e-8: device driver time,
    rank, residual, rooflines of the column evaluations and the factor
    update, and the reconstruction error on seeded blocks; the oracle port on
    all host cores beside it with the pivot agreement."""
    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.cholesky import _cholesky_device

    recs = syn.cholesky_atom()
    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    field = gi.MagneticField((0.0, 0.0, 0.1))
    _cholesky_device(basis, field, 1e-4, 0.0, None, 32, context=ctx)  # warm-up (pairs, plans, pools)
    stats: dict = {}
    t0 = time.perf_counter()
    res = _cholesky_device(basis, field, 1e-8, 0.0, None, 32, context=ctx, stats=stats)
    gpu_s = time.perf_counter() - t0
    out = {"workload": "140-AO atom 10s8p6d4f2g, B=(0,0,0.1), threshold 1e-8", "seconds": gpu_s,
           "rank": int(len(res.pivots)), "max_residual_diagonal": res.max_residual_diagonal,
           "stats": stats, "roofline": cholesky_roofline(stats, peak64),
           "update_gbs": stats["update_bytes"] / max(stats["update_ms"], 1e-9) / 1e6,
           "reconstruction_max_abs_error": reconstruction_error(res, basis, field, ctx)}
    if run_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = O.cholesky_eri(O.Oracle(), recs, (0.0, 0.0, 0.1), None, threshold=1e-8, threads=threads)
        cpu_s = time.perf_counter() - t0
        out["cpu_port_seconds"] = cpu_s
        out["cpu_port_threads"] = threads
        out["cpu_port_rank"] = int(len(ref.pivots))
        out["cpu_port_max_residual_diagonal"] = ref.max_residual_diagonal
        # single centre: the oracle's diagonal at zero field
        out.update(pivot_agreement(recs, (0.0, 0.0, 0.0), res.pivots, res.vectors, ref, threads))
        out["speedup_vs_cpu_port"] = cpu_s / gpu_s
    return out


def sweep_cholesky_leg(args, gi, ctx, fields, run_cpu: bool, peak64: float) -> list:
    """Cholesky (threshold 1e-6) of the 12-atom molecule at the first sweep
    fields: device time, rank, residual, rooflines and reconstruction error;
    against the oracle port, the first ``--sweep-cholesky-pivots`` pivots and
    factors (the oracle's full factorisation of this molecule takes minutes
    per field on the host)."""
    from giaoint_gb300.cholesky import _cholesky_device

    recs, _ = workload(args.natoms, 0)
    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    out = []
    for b in fields[: args.sweep_cholesky]:
        field = gi.MagneticField(tuple(b))
        stats: dict = {}
        t0 = time.perf_counter()
        res = _cholesky_device(basis, field, 1e-6, 0.0, None, 32, context=ctx, stats=stats)
        rec = {"B": list(b), "threshold": 1e-6, "seconds": time.perf_counter() - t0, "rank": int(len(res.pivots)),
               "max_residual_diagonal": res.max_residual_diagonal, "roofline": cholesky_roofline(stats, peak64),
               "block_evaluations": stats["block_evaluations"],
               "reconstruction_max_abs_error": reconstruction_error(res, basis, field, ctx)}
        if run_cpu and args.sweep_cholesky_pivots > 0:
            from oracle import oracle as O

            threads = os.cpu_count() or 1
            t0 = time.perf_counter()
            ref = O.cholesky_eri(O.Oracle(), recs, tuple(b), None, threshold=1e-6, threads=threads,
                                 max_pivots=args.sweep_cholesky_pivots)
            rec["cpu_port_prefix_seconds"] = time.perf_counter() - t0
            rec["cpu_port_threads"] = threads
            rec.update(pivot_agreement(recs, tuple(b), res.pivots, res.vectors, ref, threads))
        out.append(rec)
    return out


def full_tensor_leg(ctx, run_cpu: bool):
    """Plain FP64 full unscreened tensor of the 19-AO atom (4s 3p 1d, B = (0,
    0, 0.1)): latency of one gi.eri(storage="full") call through the C ABI
    (gx_eri_full, host output, every primitive quartet evaluated), with the
    oracle port's time beside it."""
    import giaoint_gb300 as gi
    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.eri import _eri_full

    recs = syn.full_tensor_atom()
    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    field = gi.MagneticField((0.0, 0.0, 0.1))
    for _ in range(3):
        full = _eri_full(basis, field=field, context=ctx, precision="fp64_exact")
    times = []
    for _ in range(20):
        t0 = time.perf_counter()
        full = _eri_full(basis, field=field, context=ctx, precision="fp64_exact")
        times.append(time.perf_counter() - t0)
    out = {"workload": "19-AO atom 4s3p1d, B=(0,0,0.1), full complex128 tensor 19^4",
           "ms_per_call_p50": 1e3 * statistics.median(times), "ms_per_call_min": 1e3 * min(times)}
    if run_cpu:
        from oracle import oracle as O

        orc = O.Oracle()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = orc.eri_full(recs, (0.0, 0.0, 0.1), None, threads)
        out["cpu_port_ms"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_port_threads"] = threads
        out["max_abs_diff_vs_cpu_port"] = float(np.max(np.abs(full - ref)))
    return out


def derivative_leg(ctx, recs, B, quartets, run_cpu: bool, count: int = 200000, seed: int = 5):
    """ERI centre derivatives (4, 3, na, nb, nc, nd) of a seeded sample of
    canonical quartets of the same molecule and field: device time of
    gx_eri_center_derivatives_device (derived-basis integrals + combine,
    output resident in HBM) and of the host-output call, with the oracle port
    (single thread) on a bounded sub-sample beside it."""
    import ctypes

    import torch

    import giaoint_gb300 as gi
    from giaoint_gb300 import _native as nat

    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    rng = np.random.default_rng(seed)
    q = np.ascontiguousarray(quartets[np.sort(rng.choice(len(quartets), min(count, len(quartets)), replace=False))],
                             dtype=np.uint32)
    sizes = np.array([gi.Shell.from_record(r).ao_count for r in recs], dtype=np.int64)
    total = int(12 * np.prod(sizes[q.astype(np.int64)], axis=1).sum())
    Bv = np.ascontiguousarray(B, dtype=np.float64)
    Ov = np.zeros(3)
    dev = torch.empty(total, dtype=torch.complex128, device="cuda:0")
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    ms = ctypes.c_float()
    lib = nat.lib()
    h = basis._device(ctx)

    def device_call():
        nat.check(lib.gx_eri_center_derivatives_device(ctx.handle, h, nat.dptr(Bv), nat.dptr(Ov), nat.u32ptr(q),
                                                       len(q), nat.i64ptr(offsets), ctypes.c_void_p(dev.data_ptr()),
                                                       total, ctypes.byref(ms)))

    for _ in range(2):
        device_call()
    times, kms = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        device_call()
        times.append(time.perf_counter() - t0)
        kms.append(ms.value)
    host = torch.empty(total, dtype=torch.complex128).pin_memory()
    hv = host.numpy()
    t0 = time.perf_counter()
    nat.check(lib.gx_eri_center_derivatives(ctx.handle, h, nat.dptr(Bv), nat.dptr(Ov), nat.u32ptr(q), len(q),
                                            nat.i64ptr(offsets), nat.dptr(hv.view(np.float64)), total,
                                            ctypes.byref(ms)))
    host_s = time.perf_counter() - t0
    dev_s = statistics.median(times)
    out = {"workload": f"{len(q)} seeded canonical quartets of the 12-atom molecule, same field, "
                       f"{total} derivative components (4 slots x 3 axes per ERI)",
           "quartets": int(len(q)), "components": total, "seconds_device": dev_s,
           "derived_integral_kernel_ms": statistics.median(kms),
           "quartets_per_s": len(q) / dev_s, "components_per_s": total / dev_s,
           "seconds_host_output": host_s, "host_output_components_per_s": total / host_s}
    if run_cpu:
        from oracle import oracle as O

        sub = q[np.sort(rng.choice(len(q), 400, replace=False))]
        t0 = time.perf_counter()
        ref, roff = O.Oracle().eri_center_derivatives(recs, sub, tuple(B), (0.0, 0.0, 0.0))
        cpu_s = time.perf_counter() - t0
        idx = {tuple(x): i for i, x in enumerate(q.tolist())}
        got = np.concatenate([hv[offsets[idx[tuple(x)]]:offsets[idx[tuple(x)] + 1]] for x in sub.tolist()])
        out["cpu_port"] = {"components_per_s": len(ref) / cpu_s, "cores": 1,
                           "sample": f"400 of the quartets ({len(ref)} components), {cpu_s:.2f} s, "
                                     "oracle/giao_oracle.c single thread"}
        out["max_abs_diff_vs_cpu_port"] = float(np.abs(got - ref).max())
        out["speedup_vs_cpu_port_1_thread"] = (total / dev_s) / (len(ref) / cpu_s)
    del dev
    return out


def serving_cpu_baseline(reqs, budget_s: float = 20.0) -> dict:
    """The same request list served sequentially by the CPU oracle port (all
    host threads), bounded: requests are run in arrival order until
    ``budget_s`` of CPU service time is spent (a Cholesky request only when
    its molecule has at most 4 atoms: larger ones take minutes on the port).
    The service time of every other request is modelled from the measured
    rates (ERI requests: ERIs/s; Cholesky: seconds per pivot-block column
    entry are not modelled, the request is reported as not run), and the
    sequential schedule start = max(arrival, previous finish) gives the
    latencies."""
    from oracle import oracle as O

    orc = O.Oracle()
    threads = os.cpu_count() or 1
    spent = 0.0
    service = [None] * len(reqs)
    entries = [0] * len(reqs)
    measured = 0
    for i, r in enumerate(reqs):
        sizes = np.array([(s_.angular_momentum + 1) * (s_.angular_momentum + 2) // 2 * len(s_.raw_coefficients)
                          for s_ in r.shells])
        if r.kind == "eri":
            q = np.asarray(r.quartets, dtype=np.uint32).reshape(-1, 4)
            entries[i] = int(np.prod(sizes[q.astype(np.int64)], axis=1).sum()) if len(q) else 0
            if spent < budget_s:
                t0 = time.perf_counter()
                orc.eri_batch(list(r.shells), q, tuple(r.field), None, threads)
                service[i] = time.perf_counter() - t0
                spent += service[i]
                measured += 1
        elif spent < budget_s and len(r.shells) <= 4 * len(syn_recipe()):
            t0 = time.perf_counter()
            O.cholesky_eri(orc, list(r.shells), tuple(r.field), None, threshold=float(r.threshold), threads=threads)
            service[i] = time.perf_counter() - t0
            spent += service[i]
            measured += 1
    eri_meas = [(service[i], entries[i]) for i, r in enumerate(reqs) if r.kind == "eri" and service[i] is not None]
    rate = sum(e for _, e in eri_meas) / max(sum(t for t, _ in eri_meas), 1e-9) if eri_meas else None
    modelled = 0
    for i, r in enumerate(reqs):
        if service[i] is None and r.kind == "eri" and rate:
            service[i] = entries[i] / rate
            modelled += 1
    t = 0.0
    lat, kinds = [], []
    served = 0
    for i, r in enumerate(reqs):
        if service[i] is None:
            continue
        start = max(t, r.arrival)
        t = start + service[i]
        lat.append(t - r.arrival)
        kinds.append(r.kind)
        served += 1
    lat_ms = np.array(lat) * 1e3
    makespan = t - min(r.arrival for r in reqs) if served else 0.0
    served_entries = sum(entries[i] for i in range(len(reqs)) if service[i] is not None)
    return {"threads": threads, "kind": "port", "requests": len(reqs), "measured": measured,
            "modelled_from_rate": modelled, "not_run": len(reqs) - served,
            "cpu_seconds_measured": spent,
            "p50_ms": float(np.percentile(lat_ms, 50)) if served else None,
            "p99_ms": float(np.percentile(lat_ms, 99)) if served else None,
            "eris_per_s": served_entries / makespan if makespan > 0 else None,
            "requests_per_s": served / makespan if makespan > 0 else None,
            "eri_rate_measured": rate,
            "note": "sequential service on the host in arrival order; requests beyond the measured budget are "
                    "modelled from the measured ERI rate; Cholesky requests above 4 atoms are not run"}


def syn_recipe():
    from giaoint_gb300 import synthetic as syn

    return syn.MOLECULE_RECIPE


def serving_leg(args, run_cpu: bool):
    """Serving mix (config 5 as specified): Poisson arrivals at 200 req/s; each
    request a seeded molecule of 3-40 atoms (the 12-atom recipe), |B| <= 0.3,
    either an ERI block of up to 2^24 complex entries (seeded canonical
    quartet subset) or Cholesky at threshold 1e-6/1e-7/1e-8.  Four
    overlapping slots admit requests by estimated device footprint; a request
    estimated above the per-request limit (--serving-request-gib) is refused
    with MemoryError and counted.  Then the same list at a load the GPU
    sustains, and the CPU port serving the list sequentially."""
    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.serving import Server, latency_summary

    limit = int(args.serving_request_gib * (1 << 30))

    def requests(rate, count, seed):
        return syn.serving_requests(count=count, rate=rate, seed=seed, atoms=(3, 40), max_entries=1 << 24,
                                    cholesky_fraction=0.25, cholesky_atoms=(3, 40))

    def trace(reqs, rate):
        with Server(slots=4, precision=args.precision, mixed_cutoff=args.mixed_cutoff,
                    max_request_bytes=limit) as srv:
            done = srv.run(reqs)
            summary = latency_summary(done)
            summary.update(load={"rate_req_s": rate, "requests": len(reqs), "slots": 4,
                                 "hbm_budget_bytes": srv.hbm_budget, "max_inflight": srv.max_inflight,
                                 "per_request_limit_bytes": limit, "refused": srv.refused,
                                 "eri_requests": sum(r.kind == "eri" for r in reqs),
                                 "cholesky_requests": sum(r.kind == "cholesky" for r in reqs),
                                 "cholesky_atoms": sorted(len(r.shells) // len(syn.MOLECULE_RECIPE)
                                                          for r in reqs if r.kind == "cholesky")},
                           precision=args.precision)
            errors = [repr(c.error) for c in done if c.error is not None and not isinstance(c.error, MemoryError)]
            if errors:
                summary["errors"] = errors[:3]
        return summary

    # the specified load (200 req/s offered: beyond one GPU, latency is mostly
    # queueing), then a load the GPU sustains (service latency)
    reqs = requests(200.0, args.serving_requests, 2026)
    out = trace(reqs, 200.0)
    out["sustained_load"] = trace(requests(4.0, max(8, args.serving_requests // 2), 2027), 4.0)
    if run_cpu:
        out["cpu_sequential"] = serving_cpu_baseline(reqs)
    return out


def sweep_leg(args, lib, nat, plan, outp, out, stream, torch, ctx, recs, quartets, offsets, peak64: float,
              run_cpu: bool):
    """Field sweep on the same molecule (config 4): every field evaluated in
    FP64 and in mixed precision through the plan (all 262.8M ERIs per field,
    kept on the device); per field the times, max |mixed - FP64| over every
    ERI, and max |GPU - oracle| of both modes on a seeded subset of canonical
    quartets; then the Cholesky (1e-6) of the first fields."""
    from giaoint_gb300 import synthetic as syn
    from oracle import oracle as O

    fields = syn.field_grid(args.sweep, 0.5)
    nat.check(lib.gx_context_set_stream(ctx.handle, ctypes.c_void_p(stream.cuda_stream)))
    ref = torch.empty_like(out)
    out_c, ref_c = out.view(torch.complex128), ref.view(torch.complex128)
    orc = O.Oracle() if run_cpu else None
    threads = os.cpu_count() or 1
    per_field = []
    t64 = tmx = 0.0
    Ov = np.zeros(3)
    nq = len(quartets)
    with torch.cuda.stream(stream):
        for k, b in enumerate(fields):
            Bv = np.ascontiguousarray(b, dtype=np.float64)
            # the pair records of a new field are built outside the timed region
            nat.check(lib.gx_eri_plan_execute(plan, nat.dptr(Bv), nat.dptr(Ov), 0, args.mixed_cutoff, outp))
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record(stream)
            nat.check(lib.gx_eri_plan_execute(plan, nat.dptr(Bv), nat.dptr(Ov), 0, args.mixed_cutoff, outp))
            e[1].record(stream)
            ref.copy_(out)
            e[2].record(stream)
            nat.check(lib.gx_eri_plan_execute(plan, nat.dptr(Bv), nat.dptr(Ov), 1, args.mixed_cutoff, outp))
            e[3].record(stream)
            d = (out - ref).view(-1, 2)
            err = float(torch.sqrt((d * d).sum(dim=1)).max().item())
            del d
            ms64, msmx = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
            t64 += ms64
            tmx += msmx
            rec = {"B": list(b), "B_norm": float(np.linalg.norm(b)), "fp64_ms": ms64, "mixed_ms": msmx,
                   "max_abs_err_mixed_vs_fp64": err}
            if orc is not None and args.sweep_oracle_quartets > 0:
                rng = np.random.default_rng(500 + k)
                idx = np.sort(rng.choice(nq, min(nq, args.sweep_oracle_quartets), replace=False))
                vals, _ = orc.eri_batch(recs, quartets[idx], tuple(b), None, threads)
                stream.synchronize()
                rec["oracle_quartets"] = int(len(idx))
                rec["max_abs_err_fp64_vs_oracle"] = float(np.abs(gather_blocks(ref_c, offsets, idx) - vals).max())
                rec["max_abs_err_mixed_vs_oracle"] = float(np.abs(gather_blocks(out_c, offsets, idx) - vals).max())
            per_field.append(rec)
    nat.check(lib.gx_context_synchronize(ctx.handle))
    nat.check(lib.gx_context_set_stream(ctx.handle, None))
    del ref
    eris = int(offsets[-1])
    out_d = {"workload": "12-atom molecule (seed 2026) at 64 seeded fields |B| <= 0.5 sorted by |B|; all canonical "
                         "quartets per field in FP64 and mixed (cutoff %g)" % args.mixed_cutoff,
             "fields": len(fields), "bmax": 0.5, "fp64_ms_total": t64, "mixed_ms_total": tmx,
             "fp64_eris_per_s": eris * len(fields) / (t64 * 1e-3), "mixed_eris_per_s": eris * len(fields) / (tmx * 1e-3),
             "speedup_mixed_vs_fp64": t64 / max(tmx, 1e-9),
             "max_abs_err_mixed_vs_fp64": max(f["max_abs_err_mixed_vs_fp64"] for f in per_field),
             "per_field": per_field}
    if per_field and "max_abs_err_mixed_vs_oracle" in per_field[0]:
        out_d["max_abs_err_mixed_vs_oracle"] = max(f["max_abs_err_mixed_vs_oracle"] for f in per_field)
        out_d["max_abs_err_fp64_vs_oracle"] = max(f["max_abs_err_fp64_vs_oracle"] for f in per_field)
    if args.sweep_cholesky > 0:
        import giaoint_gb300 as gi

        out_d["cholesky_1e-6"] = sweep_cholesky_leg(args, gi, ctx, fields, run_cpu, peak64)
    return out_d


def run_reference(args):
    """The reference algorithm on the host cores: the oracle port (a C
    restatement of the reference library) with all host threads, on a
    bounded seeded sample of the same quartets per step.  Nothing of the GPU
    library is loaded on this path."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.replicas import field_for_rank
    from oracle import oracle as O

    recs = syn.random_molecule(2026, natoms=args.natoms)
    B = field_for_rank(0)
    quartets = O.Oracle().canonical_quartets(len(recs))
    per_step = []
    info = None
    for i in range(args.warmup + args.steps):
        info = cpu_sample_rate(recs, B, quartets, target_seconds=4.0, seed=100 + i)
        if i >= args.warmup:
            per_step.append(info["value"])
    value = float(statistics.mean(per_step))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_block(args.natoms),
            "arm": "CPU reference algorithm (oracle port of the reference library, FP64, every primitive quartet)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import giaoint_gb300 as gi
    from giaoint_gb300 import _native as nat

    lib = nat.lib()
    ctx = nat.Context(local)
    recs, B = workload(args.natoms, rank)
    if args.cholesky_only:
        pk = ctypes.c_double()
        nat.check(lib.gx_measure_fp64_peak(ctx.handle, ctypes.byref(pk)))
        print(json.dumps({"cholesky": cholesky_leg(gi, nat, ctx, run_cpu=False, peak64=pk.value)}), flush=True)
        return
    if args.derivatives_only:
        quartets = gi.canonical_quartets(len(recs))
        leg = derivative_leg(ctx, recs, B, quartets, run_cpu=False, count=args.derivative_quartets)
        print(json.dumps({"center_derivatives": leg}), flush=True)
        return
    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    bh = basis._device(ctx)
    quartets = gi.canonical_quartets(len(recs))
    nq = len(quartets)
    offsets = np.zeros(nq + 1, dtype=np.int64)
    plan = ctypes.c_void_p()
    nat.check(lib.gx_eri_plan_create(ctx.handle, bh, nat.u32ptr(quartets), nq, nat.i64ptr(offsets),
                                     ctypes.byref(plan)))
    total = int(offsets[-1])
    ntask, nprim = ctypes.c_int64(), ctypes.c_int64()
    model = ctypes.c_double()
    launches = ctypes.c_int()
    nat.check(lib.gx_eri_plan_info(plan, ctypes.byref(ntask), ctypes.byref(nprim), ctypes.byref(model),
                                   ctypes.byref(launches)))
    out = torch.empty(2 * total, dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2
    stream = torch.cuda.Stream(device=local)
    nat.check(lib.gx_context_set_stream(ctx.handle, ctypes.c_void_p(stream.cuda_stream)))
    Bv = np.ascontiguousarray(B, dtype=np.float64)
    Ov = np.zeros(3)
    outp = ctypes.c_void_p(out.data_ptr())

    def step(prec):
        nat.check(lib.gx_eri_plan_execute(plan, nat.dptr(Bv), nat.dptr(Ov), prec, args.mixed_cutoff, outp))

    tuning = {}

    def autotune(prec):
        # one-time plan setup: per-class launch configurations (not timed)
        before, after = ctypes.c_double(), ctypes.c_double()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            nat.check(lib.gx_eri_plan_autotune(plan, nat.dptr(Bv), nat.dptr(Ov), prec, args.mixed_cutoff, outp, 2,
                                               ctypes.byref(before), ctypes.byref(after)))
        tuning[prec] = {"seconds": time.perf_counter() - t0, "class_ms_default": before.value,
                        "class_ms_tuned": after.value}

    def timed(prec):
        if not args.no_autotune:
            autotune(prec)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                step(prec)
            torch.cuda.synchronize()
            nat.check(lib.gx_context_synchronize(ctx.handle))
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            clocks = ClockSampler(local)
            clocks.start()
            evs = []
            for _ in range(args.steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step(prec)
                e1.record(stream)
                evs.append((e0, e1))
            torch.cuda.synchronize()
            clock_info = clocks.stop()
        nat.check(lib.gx_context_synchronize(ctx.handle))
        ms = float(sum(a.elapsed_time(b) for a, b in evs) / len(evs))
        if world > 1:
            t = torch.tensor([ms], device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        n64, n32 = ctypes.c_int64(), ctypes.c_int64()
        f64, f32 = ctypes.c_double(), ctypes.c_double()
        nat.check(lib.gx_eri_plan_counts(plan, ctypes.byref(n64), ctypes.byref(n32), ctypes.byref(f64),
                                         ctypes.byref(f32)))
        return ms, clock_info, (n64.value, n32.value, f64.value, f32.value)

    if args.profile_e2e:
        # three host-output calls through the C ABI into page-locked memory,
        # the third inside an NVTX range "call" (for an ncu capture of every
        # launch of one end-to-end call: --nvtx --nvtx-include "call/")
        nat.check(lib.gx_context_set_stream(ctx.handle, None))
        host = torch.empty(2 * total, dtype=torch.float64, pin_memory=True)
        hq = torch.from_numpy(quartets.view(np.int32)).pin_memory()
        off2 = np.zeros(nq + 1, dtype=np.int64)
        prec = {"fp64": 0, "mixed": 1}[args.precision]

        def call():
            nat.check(lib.gx_eri_batch(ctx.handle, bh, nat.dptr(Bv), nat.dptr(Ov),
                                       ctypes.cast(hq.data_ptr(), ctypes.POINTER(ctypes.c_uint32)), nq, prec,
                                       args.mixed_cutoff, 0.0, None, nat.i64ptr(off2),
                                       ctypes.cast(host.data_ptr(), ctypes.POINTER(ctypes.c_double)), total, None))

        call()
        call()
        torch.cuda.nvtx.range_push("call")
        call()
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"profile_e2e": args.precision}), flush=True)
        lib.gx_eri_plan_destroy(plan)
        return
    if args.profile_step:
        # one step of one mode inside an NVTX range "step" (for an ncu capture
        # of every class launch of the step: --nvtx --nvtx-include "step/")
        prec = {"fp64": 0, "mixed": 1, "fp64_exact": 2}[args.profile_step]
        if not args.no_autotune:
            autotune(prec)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                step(prec)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push("step")
            step(prec)
            torch.cuda.nvtx.range_pop()
            torch.cuda.synchronize()
        nat.check(lib.gx_context_synchronize(ctx.handle))
        print(json.dumps({"profile_step": args.profile_step, "classes": int(lib.gx_eri_plan_class_count(plan))}),
              flush=True)
        lib.gx_eri_plan_destroy(plan)
        return
    ms_ex, clocks_ex, cnt_ex = timed(2)
    exact = out.clone()
    ms64, clocks64, cnt64 = timed(0)
    d64 = (out - exact).view(-1, 2)
    err64 = float(torch.sqrt((d64 * d64).sum(dim=1)).max().item())
    del d64
    fp64_out = out.clone()
    ms_mx, clocks_mx, cnt_mx = timed(1)
    diff = (out - exact).view(-1, 2)
    max_err = float(torch.sqrt((diff * diff).sum(dim=1)).max().item())
    del diff
    mixed_out = out.clone()  # out is reused by the e2e leg
    headline_mixed = args.precision == "mixed"
    ms = ms_mx if headline_mixed else ms64
    clock_info = clocks_mx if headline_mixed else clocks64
    value = world * total / (ms * 1e-3)
    # live roofline denominators: FP64 and FP32 FMA probes
    peak, peak32 = ctypes.c_double(), ctypes.c_double()
    nat.check(lib.gx_measure_fp64_peak(ctx.handle, ctypes.byref(peak)))
    nat.check(lib.gx_measure_fp32_peak(ctx.handle, ctypes.byref(peak32)))
    achieved64 = cnt64[2] / (ms64 * 1e-3) / 1e12
    # mixed: FLOPs_fp64 / (t P64) + FLOPs_fp32 / (t P32) (FLOP model per primitive quartet)
    mx_tf64 = cnt_mx[2] / (ms_mx * 1e-3) / 1e12
    mx_tf32 = cnt_mx[3] / (ms_mx * 1e-3) / 1e12
    frac_mixed = mx_tf64 / peak.value + mx_tf32 / peak32.value
    prec = {"fp64": 0, "mixed": 1}[args.precision]
    # e2e through the host-buffer C ABI call (pinned host memory)
    e2e = None
    if not args.no_e2e:
        nat.check(lib.gx_context_set_stream(ctx.handle, None))
        host = torch.empty(2 * total, dtype=torch.float64, pin_memory=True)
        hq = torch.from_numpy(quartets.view(np.int32)).pin_memory()
        kept = np.empty((nq, 4), dtype=np.uint32)
        off2 = np.zeros(nq + 1, dtype=np.int64)
        stats = nat.GxStats()
        times, kernel_ms, prepare_ms, copy_ms = [], [], [], []
        reps = max(1, min(args.steps, 5))
        warm = max(3, args.warmup)  # the first call is the cold one, reported separately
        for i in range(warm + reps):
            t0 = time.perf_counter()
            nat.check(lib.gx_eri_batch(ctx.handle, bh, nat.dptr(Bv), nat.dptr(Ov),
                                       ctypes.cast(hq.data_ptr(), ctypes.POINTER(ctypes.c_uint32)), nq, prec, 1e-6,
                                       0.0, nat.u32ptr(kept), nat.i64ptr(off2),
                                       ctypes.cast(host.data_ptr(), ctypes.POINTER(ctypes.c_double)), total,
                                       ctypes.byref(stats)))
            dt = time.perf_counter() - t0
            if i >= warm:
                times.append(dt)
                kernel_ms.append(stats.kernel_ms)
                prepare_ms.append(round(stats.prepare_ms, 2))
                copy_ms.append(round(stats.copy_ms, 2))
            elif i == 0:
                cold_s = dt  # builds and caches the class-sorted plan on the host
        # breakdown: the same call with device output (no host copy)
        dev_times = []
        for i in range(reps):
            t0 = time.perf_counter()
            nat.check(lib.gx_eri_batch_device(ctx.handle, bh, nat.dptr(Bv), nat.dptr(Ov),
                                              ctypes.cast(hq.data_ptr(), ctypes.POINTER(ctypes.c_uint32)), nq, prec,
                                              1e-6, 0.0, None, nat.i64ptr(off2), ctypes.c_void_p(out.data_ptr()),
                                              total, None))
            dev_times.append(time.perf_counter() - t0)
        e2e_s = float(statistics.mean(times))
        if world > 1:
            t = torch.tensor([e2e_s], device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(t.item())
        # spot check: the host result equals the device-resident result (the
        # autotuned plan groups primitive sums differently: last-bit differences)
        dev_sample = out[: 2 * min(total, 1 << 20)].cpu().numpy()
        e2e_diff = float(np.max(np.abs(dev_sample - host[: len(dev_sample)].numpy()), initial=0.0))
        assert e2e_diff <= 1e-11, f"e2e and device results differ by {e2e_diff}"
        # the device-to-host leg alone, for the breakdown: pinned copies
        # (the first one warms the mapping)
        d2h = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            host.copy_(out.view(-1)[: 2 * total])
            torch.cuda.synchronize()
            d2h.append(time.perf_counter() - t0)
        d2h_s = min(d2h[1:])
        e2e = {"value": world * total / e2e_s, "unit": UNIT,
               # per warm call: the field (B, O); the quartet list is read and
               # hashed on the host, its plan is cached on the device
               "h2d_bytes_per_step": 48, "d2h_bytes_per_step": int(total * 16), "seconds_per_step": e2e_s,
               "cold_call_seconds": cold_s, "cold_h2d_bytes": int(ntask.value * 48 + 48),
               "d2h_copy_seconds": d2h_s, "d2h_gb_per_s": total * 16 / d2h_s / 1e9,
               "api": "gx_eri_batch (C ABI, pinned host buffers)", "max_abs_diff_vs_device_path": e2e_diff,
               "copy": "each class's blocks copied by the SMs to the page-locked output as the class finishes",
               "call_seconds": times, "call_seconds_median": float(statistics.median(times)),
               "call_kernel_ms": kernel_ms,
               "call_prepare_ms": prepare_ms,
               "call_copy_ms": copy_ms,
               "device_output_call_seconds": dev_times}
    cpu = None
    parity = {"bar": {"fp64": 1e-12, "fp64_exact": 1e-12, "mixed": 1e-10}}
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, cpu_idx, cpu_vals = cpu_sample_rate(recs, B, quartets, target_seconds=10.0, keep=True)
        # the same port on one thread (a smaller sample), the figure beside the all-core one
        single = cpu_sample_rate(recs, B, quartets, target_seconds=4.0, seed=2, threads=1)
        cpu["single_thread"] = {"value": single["value"], "cores": 1, "sample": single["sample"]}
        # full-size parity: every mode's output against the oracle on the sample
        for name, t in (("fp64_exact", exact), ("fp64", fp64_out), ("mixed", mixed_out)):
            got = gather_blocks(t.view(torch.complex128), offsets, cpu_idx)
            parity[name] = float(np.abs(got - cpu_vals).max())
        parity["quartets"] = int(len(cpu_idx))
        parity["eris"] = int(len(cpu_vals))
        parity["ok"] = all(parity[k] <= parity["bar"][k] for k in ("fp64", "fp64_exact", "mixed"))
        del cpu_vals
    del exact, fp64_out, mixed_out
    sweep = None
    if args.sweep > 0:
        sweep = sweep_leg(args, lib, nat, plan, outp, out, stream, torch, ctx, recs, quartets, offsets, peak.value,
                          run_cpu=(rank == 0 and world == 1 and not args.no_cpu))
    chol = None
    if rank == 0 and not args.no_cholesky:
        nat.check(lib.gx_context_set_stream(ctx.handle, None))
        chol = cholesky_leg(gi, nat, ctx, run_cpu=(world == 1 and not args.no_cpu), peak64=peak.value)
    full_tensor = None
    if rank == 0:
        nat.check(lib.gx_context_set_stream(ctx.handle, None))
        full_tensor = full_tensor_leg(ctx, run_cpu=(world == 1 and not args.no_cpu))
    derivatives = None
    if rank == 0 and not args.no_derivatives:
        nat.check(lib.gx_context_set_stream(ctx.handle, None))
        derivatives = derivative_leg(ctx, recs, B, quartets, run_cpu=(world == 1 and not args.no_cpu),
                                     count=args.derivative_quartets)
    serving = None
    if rank == 0 and not args.no_serving:
        serving = serving_leg(args, run_cpu=(world == 1 and not args.no_cpu))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE if headline_mixed else "f64", "data": "synthetic",
            "config": config_block(args.natoms),
            "run": {"precision": args.precision, "quartets_per_step": nq, "eris_per_step": total,
                    "primitive_quartets_per_step": int(nprim.value), "mixed_cutoff": args.mixed_cutoff,
                    "parallelism": f"replicas{world} (one field per rank)"},
            "quartets_per_s": world * nq / (ms * 1e-3),
            "fp64_exact": {"ms_per_step": ms_ex, "eris_per_s": world * total / (ms_ex * 1e-3),
                           "primitive_quartets_evaluated": cnt_ex[0], "clocks": clocks_ex,
                           "note": "every primitive quartet, as the reference evaluates them"},
            "fp64": {"ms_per_step": ms64, "eris_per_s": world * total / (ms64 * 1e-3),
                     "max_abs_error_vs_fp64_exact": err64,
                     "primitive_quartets_evaluated": cnt64[0], "primitive_quartets_skipped": int(nprim.value) - cnt64[0],
                     "clocks": clocks64},
            "mixed": {"ms_per_step": ms_mx, "eris_per_s": world * total / (ms_mx * 1e-3),
                      "fp64_primitive_quartets": cnt_mx[0], "fp32_primitive_quartets": cnt_mx[1],
                      "max_abs_error_vs_fp64_exact": max_err, "speedup_vs_fp64": ms64 / ms_mx,
                      "speedup_vs_fp64_exact": ms_ex / ms_mx, "clocks": clocks_mx},
            "roofline": {"bound": "fp64", "unit": "TFLOP/s",
                         # FP64-equivalent rate: FLOPs_fp64 + FLOPs_fp32 * P64 / P32 per second of the
                         # headline step, so that achieved / peak is the two-term fraction
                         "achieved": (frac_mixed if headline_mixed else achieved64 / peak.value) * peak.value,
                         "peak": peak.value,
                         "frac": frac_mixed if headline_mixed else achieved64 / peak.value,
                         "terms": {"fp64": {"achieved": mx_tf64, "peak": peak.value,
                                            "frac": mx_tf64 / peak.value, "flops": cnt_mx[2]},
                                   "fp32": {"achieved": mx_tf32, "peak": peak32.value,
                                            "frac": mx_tf32 / peak32.value, "flops": cnt_mx[3]}},
                         "fp64_mode": {"achieved": achieved64, "frac": achieved64 / peak.value,
                                       "ms_per_step": ms64},
                         "traffic": TRAFFIC_PER_STEP.get(args.precision) if args.natoms == 12 else None,
                         "traffic_basis": TRAFFIC_BASIS,
                         "kernel": "one plan execution: quartet_kernel, small_kernel and (mixed) lane32_kernel launches of the 81 classes",
                         "achieved_basis": "FLOP model per primitive quartet (reference-structured MD count) x "
                                           "primitive quartets evaluated per precision / event-timed step; "
                                           "frac = FLOPs_fp64/(t P64) + FLOPs_fp32/(t P32)",
                         "model_flops_all_primitive_quartets": model.value,
                         "peak_source": "measured live: FP64 and FP32 FMA-chain probe kernels "
                                        "(gx_measure_fp64_peak, gx_measure_fp32_peak); MEASURED_PEAKS.json holds "
                                        "no FP64/FP32 CUDA-core peak",
                         "peak32": peak32.value},
            "parity": parity,
            # one kernel per (la, lb, lc, ld) class per step; the pair records
            # are computed once per field, before the timed steps
            "gpu_launches": int(lib.gx_eri_plan_class_count(plan)) * args.steps,
            "autotune": {str({0: "fp64", 1: "mixed", 2: "fp64_exact"}[k]): v for k, v in tuning.items()} or None,
            "graph_replays": int(lib.gx_eri_plan_graph_replays(plan)),
            "clocks": clock_info,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "cholesky": chol,
            "field_sweep": sweep,
            "full_tensor": full_tensor,
            "center_derivatives": derivatives,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    lib.gx_eri_plan_destroy(plan)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0 and parity.get("ok") is False:
        print(f"parity failure against the oracle sample: {parity}", file=sys.stderr, flush=True)
        sys.exit(1)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
