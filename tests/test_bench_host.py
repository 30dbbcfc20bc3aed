"""Host-side pieces of bench.py (CPU): the work model behind the roofline lines and one complete
oracle G0W0 step of the reference arm on a small system.

The reference arm times `oracle_g0w0_full` on the benchmark system; here it runs on the N=24
synthetic system (seconds), and its breakdown must carry the QP gap and the branch it took for
the second Casida (RG0W0.f90:222-225: with an open gap the oracle's phRLR runs; with a closed
one EcRPA is NaN and the step skips the eigenproblem, as the GPU tiers do).
"""
import numpy as np

import bench
from quack_gb300 import synth


def test_stage_work_double_float_tridiagonalisation():
    w = bench.stage_work(200, 3600)
    kind, amount, desc = w["tridiag_df"]
    assert kind == "fp32_ops"
    assert abs(amount - 49.0 * 3600 ** 3 / 6.0) < 1.0
    assert "49" in desc
    # the FP64 tier's count stays LAPACK's
    assert abs(w["tridiag"][1] - 4.0 / 3.0 * 3600 ** 3) < 1.0


def test_oracle_full_g0w0_step_open_gap():
    s = synth.gen_system(24, 3, 72, np.random.default_rng(1))
    E = synth.eri_phys_numpy(s["L"])
    total, tb = bench.oracle_g0w0_full(s, E)
    assert total > 0.0
    assert tb["qp_gap"] > 0.0
    assert "casida2" in tb and not tb.get("casida2_skipped_closed_gap", False)
    for k in ("casida", "rho", "sigma", "qp"):
        assert tb[k] >= 0.0
