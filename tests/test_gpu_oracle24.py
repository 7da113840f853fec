"""The precision form of the 3D operator family against the exact resolvent
on a 24^3 subproblem: N = 69,120 (5x5 blocks), k = 16, 64 frequencies, two
transient periods, diagonal W_q = W_f from cell volumes, the spectral shift
from the RK4 propagator's growth rate.

Variant 1 = complex64 stages with the FP64 sweep (RSVDT_PREC_C64_REFINE),
variant 2 = plain complex128, both with q = 1. The oracle is a sparse LU of
(i w I - A) with Lanczos on W_q^{1/2} (i w I - A)^{-1} W_f^{-1/2}
(oracle.sparse_resolvent_svd) at w = 0 and w = 0.1, where sigma_1 /
sigma_2 is about 1.17. With q = 1 neither variant has converged there (the
random sketch, not the arithmetic, sets the error: both variants agree with
each other to the complex64 rounding); with q = 6 the same path reaches the
exact leading gain to within the RK4 truncation and transient errors.
"""
import numpy as np
import pytest

import oracle
from rsvdt import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def chord_angle(u, v):
    u = u / np.linalg.norm(u)
    v = v / np.linalg.norm(v)
    c = np.vdot(v, u)
    ph = c / abs(c) if abs(c) > 0 else 1.0
    return float(2 * np.arcsin(min(1.0, np.linalg.norm(u - ph * v) / 2)))


def test_3d24_precision_forms_against_the_sparse_oracle(built_lib):
    import rsvdt
    from rsvdt import workloads

    k, Nw = 16, 64
    wl = workloads.make_3d(n=24, k=k, Nw=Nw, q=1)
    A = synth.bcsr_to_csr(*wl.bcsr)
    wq = wl.weights["W_sqrt"].diagonal()
    wqi = wl.weights["W_sqrt_inv"].diagonal()
    iws = [0, 1]
    S, U1, V1 = {}, {}, {}
    for name, prec, q in (("v1_q1", rsvdt.PREC_C64_REFINE, 1), ("v2_q1", rsvdt.PREC_C128, 1),
                          ("v1_q6", rsvdt.PREC_C64_REFINE, 6)):
        p = rsvdt.default_params(k=k, q=q, Nw=Nw, w=wl.w, dt=wl.dt_in, TransientLength=wl.transient_length,
                                 TransientRemoval=0, precision=prec, Display=0)
        ctx = rsvdt.Context(p)
        ctx.set_operator_bcsr(*wl.bcsr)
        ctx.set_weight(rsvdt.W_Q_SQRT, wl.weights["W_sqrt"])
        ctx.set_weight(rsvdt.W_F_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.set_weight(rsvdt.W_Q_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.random_sketch(99)
        ctx.run()
        S[name] = ctx.get_results(U=False, V=False)[2]
        U1[name], V1[name] = ctx.get_result_cols([iw * k for iw in iws], U=True, V=True)
        ctx.close()
    So, Uo, Vo = oracle.sparse_resolvent_svd(A, [oracle.freq_of(iw, Nw, wl.w) for iw in iws], 3, wq=wq,
                                             wf_inv=wqi, procs=2)
    # Variant 1 against variant 2 (q = 1): the complex64 arithmetic's share.
    rel12 = np.abs(S["v1_q1"] - S["v2_q1"]) / S["v2_q1"]
    print("24^3: variant 1 vs 2 gain error (j <= 3):", rel12[:3].max())
    assert rel12[:3].max() < 1e-5
    for name in S:
        for j, iw in enumerate(iws):
            e = abs(S[name][0, iw] - So[0, j]) / So[0, j]
            au = chord_angle(U1[name][:, j], wqi * Uo[j][:, 0])
            av = chord_angle(V1[name][:, j], wqi * Vo[j][:, 0])
            print(f"24^3 {name} w={oracle.freq_of(iw, Nw, wl.w):+.1f}: sigma_1 {S[name][0, iw]:.6f} "
                  f"oracle {So[0, j]:.6f} rel err {e:.3e}, angle U {au:.3e} V {av:.3e}")
            if name == "v1_q6":
                # Measured: 3.4e-4 / 7.4e-5 gain error, V angles 1.7e-4 / 1.7e-3.
                assert e < 1e-3 and av < 1e-2
