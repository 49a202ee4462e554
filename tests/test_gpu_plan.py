"""Plans on the GPU: per-class profile, autotuned launch configurations and
CUDA-graph replay give the same integrals as the default eager launches."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300.plan import EriPlan

from helpers import molecule

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_autotune_profile_and_graph_replay_match_eager():
    torch = _torch()
    recs, basis = molecule(seed=7, natoms=3)
    field = gi.MagneticField((0.05, -0.1, 0.12))
    plan = EriPlan(basis)
    out = torch.empty(plan.total, dtype=torch.complex128, device="cuda:0")
    plan.execute(out, field, precision="fp64")
    plan.synchronize()
    ref = out.clone()
    base_counts = plan.counts()

    prof = plan.profile(out, field, precision="fp64")
    keys = {(p["la"], p["lb"], p["lc"], p["ld"]) for p in prof}
    assert len(keys) == len(prof) >= 1
    assert sum(p["fp64_quartets"] for p in prof) == base_counts["fp64_quartets"]
    assert sum(p["primitive_quartets"] for p in prof) == plan.primitive_quartets
    assert all(p["ms"] >= 0.0 for p in prof)

    before, after = plan.autotune(out, field, precision="fp64", repeats=1)
    assert after <= before * 1.0001
    out.zero_()
    for _ in range(4):  # eager, capture, replays
        plan.execute(out, field, precision="fp64")
    plan.synchronize()
    assert plan.graph_replays >= 2
    # regrouping changes only the order of the FP64 primitive sums
    assert float((out - ref).abs().max()) <= 1e-13
    assert plan.counts()["fp64_quartets"] == base_counts["fp64_quartets"]

    # a new field through the replayed graph equals a fresh eager plan
    field2 = gi.MagneticField((-0.2, 0.03, 0.07))
    plan.execute(out, field2, precision="fp64")
    plan.synchronize()
    fresh = EriPlan(basis)
    out2 = torch.empty_like(out)
    fresh.execute(out2, field2, precision="fp64")
    fresh.synchronize()
    assert float((out - out2).abs().max()) <= 1e-13


def test_mixed_precision_autotuned_within_1e10_of_fp64():
    torch = _torch()
    recs, basis = molecule(seed=11, natoms=4)
    field = gi.MagneticField((0.1, 0.1, -0.15))
    plan = EriPlan(basis)
    out = torch.empty(plan.total, dtype=torch.complex128, device="cuda:0")
    plan.execute(out, field, precision="fp64_exact")
    plan.synchronize()
    exact = out.clone()
    plan.autotune(out, field, precision="mixed", repeats=1)
    for _ in range(3):
        plan.execute(out, field, precision="mixed")
    plan.synchronize()
    counts = plan.counts()
    assert counts["fp32_quartets"] > 0
    err = float((out - exact).abs().max())
    assert err <= 1e-10, err
    prof = plan.profile(out, field, precision="mixed")
    assert sum(p["fp32_quartets"] for p in prof) == counts["fp32_quartets"]


def test_pinned_stream_mode_matches_exact_and_batched():
    """Every generic class pinned to stream mode (per-entry recurrences into
    a two-column buffer), over its register variants, staging and batch
    sizes: FP64 within 1e-13 of the batched launches and 1e-12 of the
    FP64-exact path; mixed precision within 1e-10 of FP64-exact."""
    torch = _torch()
    recs, basis = molecule(seed=13, natoms=4)
    field = gi.MagneticField((0.08, -0.12, 0.05))
    plan = EriPlan(basis)
    out = torch.empty(plan.total, dtype=torch.complex128, device="cuda:0")
    plan.execute(out, field, precision="fp64_exact")
    plan.synchronize()
    exact = out.clone()
    # the untuned configuration runs stream mode from L = 5 on: pin every
    # class to the batched launches for the reference
    default = plan.get_config("fp64")
    assert any(c["stream"] == 1 for c in default)
    plan.set_config([dict(c, stream=0) for c in default], "fp64")
    plan.execute(out, field, precision="fp64")
    plan.synchronize()
    batched = out.clone()
    for minb in (2, 4):
        for nostage in (0, 1):
            for b1 in (32, 8):
                cfg = [dict(c, stream=1, min_blocks=minb, nostage=nostage, batch=b1) for c in default]
                plan.set_config(cfg, "fp64")
                assert plan.get_config("fp64") == cfg
                out.zero_()
                plan.execute(out, field, precision="fp64")
                plan.synchronize()
                assert float((out - batched).abs().max()) <= 1e-13, (minb, nostage, b1)
                assert float((out - exact).abs().max()) <= 1e-12, (minb, nostage, b1)
    plan.set_config([dict(c, stream=1, min_blocks=4) for c in plan.get_config("mixed")], "mixed")
    plan.execute(out, field, precision="mixed")
    plan.synchronize()
    assert plan.counts()["fp32_quartets"] > 0
    assert float((out - exact).abs().max()) <= 1e-10
    with pytest.raises(ValueError, match="out of range"):
        plan.set_config([dict(c, stream=2) for c in default], "fp64")
    with pytest.raises(ValueError, match="class configurations"):
        plan.set_config(default[:-1], "fp64")
