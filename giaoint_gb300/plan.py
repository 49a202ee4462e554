"""Device-resident evaluation plans (gx_eri_plan).

An ``EriPlan`` fixes a shell-quartet list of a basis once: its class-sorted
task list, packed output offsets and warp work units live on the device, so
that the same list can be evaluated for many magnetic fields without host
work.  This is the persistent, batched form of the reference's
``evaluate_eri_shell_quartets`` (src/eri.cpp:644-767) with three additions:

* ``autotune`` times every (la, lb, lc, ld) class over its launch
  configurations (work-unit size, warps per block, phase-1 batch) and keeps
  the fastest per precision mode;
* repeated executions on the same stream and output replay one CUDA graph of
  all class launches;
* ``profile`` reports the event-timed kernel duration and the FP64 / FP32
  primitive-quartet counts of every class.

Outputs are device memory owned by the caller: any object with
``data_ptr()`` (a torch tensor of ``2 * total`` float64 or ``total``
complex128 values) or a raw device address.
"""

from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _native as nat
from ._types import Basis, MagneticField, field_arrays
from .eri import DEFAULT_MIXED_CUTOFF, _precision, canonical_quartets

__all__ = ["EriPlan"]


def _address(out) -> ctypes.c_void_p:
    if hasattr(out, "data_ptr"):
        return ctypes.c_void_p(out.data_ptr())
    if isinstance(out, int):
        return ctypes.c_void_p(out)
    raise TypeError("out must be a device tensor (data_ptr()) or a device address")


class EriPlan:
    """Evaluation plan for ``quartets`` (default: all canonical quartets)."""

    def __init__(self, basis: Basis, quartets=None, *, context: nat.Context | None = None):
        if not isinstance(basis, Basis):
            raise TypeError("basis must be a Basis")
        self._ctx = context or nat.default_context()
        self._basis = basis
        q = canonical_quartets(len(basis.shells)) if quartets is None else quartets
        self.quartets = np.ascontiguousarray(np.asarray(q, dtype=np.uint32).reshape(-1, 4))
        self.offsets = np.zeros(len(self.quartets) + 1, dtype=np.int64)
        handle = ctypes.c_void_p()
        lib = nat.lib()
        nat.check(lib.gx_eri_plan_create(self._ctx.handle, basis._device(self._ctx), nat.u32ptr(self.quartets),
                                         len(self.quartets), nat.i64ptr(self.offsets), ctypes.byref(handle)))
        self._handle = handle
        tasks, prims = ctypes.c_int64(), ctypes.c_int64()
        flops, launches = ctypes.c_double(), ctypes.c_int()
        nat.check(lib.gx_eri_plan_info(handle, ctypes.byref(tasks), ctypes.byref(prims), ctypes.byref(flops),
                                       ctypes.byref(launches)))
        self.tasks = tasks.value
        self.primitive_quartets = prims.value
        self.model_flops = flops.value
        self.launches = launches.value

    @property
    def total(self) -> int:
        """Complex entries of the packed output."""
        return int(self.offsets[-1])

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._handle

    def execute(self, out, field: MagneticField | None = None, *, precision: str = "fp64",
                mixed_cutoff: float = DEFAULT_MIXED_CUTOFF) -> None:
        """Enqueue the evaluation into device memory ``out`` (asynchronous)."""
        B, O = field_arrays(field)
        nat.check(nat.lib().gx_eri_plan_execute(self._handle, nat.dptr(B), nat.dptr(O), _precision(precision),
                                                float(mixed_cutoff), _address(out)))

    def synchronize(self) -> None:
        nat.check(nat.lib().gx_context_synchronize(self._ctx.handle))

    def counts(self) -> dict:
        """Primitive quartets evaluated by the last execution (waits for it)."""
        n64, n32 = ctypes.c_int64(), ctypes.c_int64()
        f64, f32 = ctypes.c_double(), ctypes.c_double()
        nat.check(nat.lib().gx_eri_plan_counts(self._handle, ctypes.byref(n64), ctypes.byref(n32),
                                               ctypes.byref(f64), ctypes.byref(f32)))
        return {"fp64_quartets": n64.value, "fp32_quartets": n32.value, "fp64_model_flops": f64.value,
                "fp32_model_flops": f32.value}

    @property
    def graph_replays(self) -> int:
        return int(nat.lib().gx_eri_plan_graph_replays(self._handle))

    def profile(self, out, field: MagneticField | None = None, *, precision: str = "fp64",
                mixed_cutoff: float = DEFAULT_MIXED_CUTOFF) -> list[dict]:
        """Per-class event-timed kernel durations of one execution."""
        lib = nat.lib()
        n = lib.gx_eri_plan_class_count(self._handle)
        if n < 0:
            nat.check(n)
        arr = (nat.GxClassProfile * max(n, 1))()
        B, O = field_arrays(field)
        nat.check(lib.gx_eri_plan_profile(self._handle, nat.dptr(B), nat.dptr(O), _precision(precision),
                                          float(mixed_cutoff), _address(out), arr))
        return [{name: getattr(arr[i], name) for name, _ in nat.GxClassProfile._fields_} for i in range(n)]

    def autotune(self, out, field: MagneticField | None = None, *, precision: str = "fp64",
                 mixed_cutoff: float = DEFAULT_MIXED_CUTOFF, repeats: int = 2) -> tuple[float, float]:
        """Tune every class's launch configuration for ``precision``; returns
        the summed class times (ms) before and after."""
        before, after = ctypes.c_double(), ctypes.c_double()
        B, O = field_arrays(field)
        nat.check(nat.lib().gx_eri_plan_autotune(self._handle, nat.dptr(B), nat.dptr(O), _precision(precision),
                                                 float(mixed_cutoff), _address(out), int(repeats),
                                                 ctypes.byref(before), ctypes.byref(after)))
        return before.value, after.value

    def get_config(self, precision: str = "fp64") -> list[dict]:
        """Launch configuration of every class for ``precision`` (zeros: default)."""
        lib = nat.lib()
        n = lib.gx_eri_plan_class_count(self._handle)
        if n < 0:
            nat.check(n)
        arr = (nat.GxClassConfig * max(n, 1))()
        nat.check(lib.gx_eri_plan_get_config(self._handle, _precision(precision), arr))
        keys = [name for name, _ in nat.GxClassConfig._fields_]
        return [{k: getattr(arr[i], k) for k in keys} for i in range(n)]

    def set_config(self, configs: list[dict], precision: str = "fp64") -> None:
        """Pin the launch configuration of every class for ``precision``."""
        n = nat.lib().gx_eri_plan_class_count(self._handle)
        if len(configs) != n:
            raise ValueError(f"expected {n} class configurations")
        arr = (nat.GxClassConfig * max(n, 1))()
        for i, c in enumerate(configs):
            for k, v in c.items():
                setattr(arr[i], k, int(v))
        nat.check(nat.lib().gx_eri_plan_set_config(self._handle, _precision(precision), arr))

    def close(self) -> None:
        if getattr(self, "_handle", None):
            nat.lib().gx_eri_plan_destroy(self._handle)
            self._handle = None

    def __del__(self):  # pragma: no cover
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def _main(argv=None) -> None:
    """Evaluate one (la, lb, lc, ld) class of the seeded synthetic molecule
    through a plan, once per precision mode, and print the counts: a small,
    self-contained workload for profiling one kernel launch per mode.

        python -m giaoint_gb300.plan --atoms 12 --class 1111 --precision fp64,mixed [--stream] [--min-blocks 4]
    """
    import argparse

    import torch

    from . import synthetic as syn
    from ._types import Shell

    p = argparse.ArgumentParser(prog="python -m giaoint_gb300.plan")
    p.add_argument("--atoms", type=int, default=12)
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--class", dest="cls", default="1111", help="four digits la lb lc ld")
    p.add_argument("--precision", default="fp64,mixed")
    p.add_argument("--stream", action="store_true", help="stream mode (per-entry recurrences) for the class")
    p.add_argument("--min-blocks", type=int, default=0, choices=[0, 2, 4])
    a = p.parse_args(argv)
    key = tuple(int(c) for c in a.cls)
    recs = syn.random_molecule(a.seed, natoms=a.atoms)
    basis = Basis([Shell.from_record(r) for r in recs])
    ls = np.array([r.angular_momentum for r in recs])
    q = canonical_quartets(len(recs))
    sel = q[np.all(ls[q.astype(np.int64)] == np.array(key), axis=1)]
    plan = EriPlan(basis, sel)
    out = torch.empty(max(plan.total, 1), dtype=torch.complex128, device="cuda:0")
    field = MagneticField(syn.random_field(a.seed))
    for prec in a.precision.split(","):
        if a.stream or a.min_blocks:
            plan.set_config([dict(c, stream=int(a.stream), min_blocks=a.min_blocks) for c in plan.get_config(prec)],
                            prec)
        plan.execute(out, field, precision=prec)
        plan.synchronize()
        print(prec, {"class": key, "quartets": len(sel), **plan.counts()}, flush=True)


if __name__ == "__main__":
    _main()
