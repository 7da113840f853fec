"""Parity at the benchmark's own sizes, against the C restatement.

- The 3D64 operator (N = 1,310,720, 1,810,432 5x5 blocks, k = 10, Nw = 32):
  two forced RK4 steps of all test vectors through rsvdt_rk4_steps, on the
  stage kernels the benchmark times (k_rstage<z128,10,*> and, in the
  precision form, k_bstage<z64,10,2,*>), from a seeded state, across the
  wrap of the forcing index (SourceCode/TSRK4.c:18-47). These are the
  forcing-slab offsets at N*k = 13.1M and the step counter at Ns = 384 that
  the small cases never reach.
- The 48-problem batching family (N log-uniform in [200, 20000]): six
  problems, including the one where the complex64 batch is furthest from
  the complex128 batch, solved whole (SourceCode/main.c:134-144) by the
  oracle with the batch's own sketches.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def test_rk4_steps_at_3d64_match_oracle(built_lib):
    import rsvdt
    from rsvdt import workloads

    bench = _bench()
    wl = workloads.make_3d(n=64)
    ctxs = []
    for prec in (rsvdt.PREC_C128, rsvdt.PREC_C64):
        c = rsvdt.Context(wl.params(precision=prec))
        c.set_operator_bcsr(*wl.bcsr)
        c.random_sketch(1234)
        ctxs.append(c)
    res = bench.parity_steps(wl, ctxs[0], ctxs[1], os.cpu_count() or 1)
    for c in ctxs:
        c.close()
    print(res)
    assert res["same_sketch_in_both_contexts"]
    for name in ("c128_direct", "c128_adjoint"):
        assert res[name]["y_rel_err_max"] < 1e-11, (name, res[name])
        assert res[name]["F3_rel_err_max"] < 1e-11, (name, res[name])
    assert res["c64_direct"]["y_rel_err_max"] < 1e-5, res["c64_direct"]
    assert res["c64_direct"]["F3_rel_err_max"] < 1e-5, res["c64_direct"]
    assert res["pass"]


def test_batch_family_problems_match_oracle(built_lib):
    import rsvdt
    from rsvdt import synth

    bench = _bench()
    fam = synth.gl_family(48, seed=2024)
    T = 2 * np.pi / 0.1
    dt = T / 4096 * (1 + 1e-12)

    def params(pr, prec):
        return rsvdt.default_params(k=pr["k"], q=0, Nw=pr["Nw"], w=0.1, dt=dt, TransientLength=T,
                                    DiscFlg=int(pr["beta"] > 0), beta=pr["beta"], precision=prec, Display=0)

    sketches = [synth.complex_normal(pr["N"], pr["k"] * pr["Nw"], 2024 + 1 + i) for i, pr in enumerate(fam)]
    S = {}
    for name, prec in (("batched_c128", rsvdt.PREC_C128), ("batched_c64", rsvdt.PREC_C64)):
        b = rsvdt.Batch(prec)
        for pr in fam:
            b.add(params(pr, prec), pr["A"])
        for i, F in enumerate(sketches):
            b.set_sketch(i, F)
        b.run()
        S[name] = [b.get_results(i)[2] for i in range(len(fam))]
        b.close()
    errs = [float((np.abs(a[:3] - c[:3]) / c[:3]).max()) for a, c in zip(S["batched_c64"], S["batched_c128"])]
    S["worst_c64"] = int(np.argmax(errs))
    res = bench.parity_batch(fam, sketches, lambda pr: params(pr, rsvdt.PREC_C128), S, os.cpu_count() or 1, 0)
    print(res)
    assert res["problems"][0]["index"] == S["worst_c64"]
    assert res["batched_c128"]["gain_rel_err_max"] < 1e-9
    # The complex64 batch on the same problems: FP32 rounding amplified by
    # the operators' non-normality (the worst problem's sigma_1 is 4e5).
    assert res["batched_c64"]["gain_rel_err_max_j<=3"] < 1e-2
