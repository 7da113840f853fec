"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle
(the C restatement of the reference) on the same seeded inputs.

Tolerances (floating point, complex128 plain form): the target is a
relative gain error <= 1e-9 and subspace angles <= 1e-7 rad against the
reference's own run; against the restatement, which performs the same
operations in the same order up to FMA contraction and summation order, the
tests demand more where the mathematics allows it (see each test).
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from rsvdt import synth

pytestmark = pytest.mark.gpu

GAIN_TOL = 1e-9
ANGLE_TOL = 1e-7


def small_gl(N=64, w=0.1, Nw=16, dt_in=0.15, TL_periods=1.0):
    """Stable 64-node Ginzburg-Landau operator (mu0 = 0.2: max Re(lambda) =
    -0.108, |lambda| <= 12.3, RK4-stable at dt = 0.145)."""
    A = synth.gl_operator(N, mu0=0.2)
    T = 2 * np.pi / w
    return A, dict(w=w, Nw=Nw, dt=dt_in, TransientLength=TL_periods * T)


def make_ctx(A, cfg, k, q=0, tr=False, prec=0, bcsr=None):
    import rsvdt
    p = rsvdt.default_params(k=k, q=q, Nw=cfg["Nw"], w=cfg["w"], dt=cfg["dt"],
                             TransientLength=cfg["TransientLength"], TransientRemoval=int(tr),
                             precision=prec, Display=0)
    ctx = rsvdt.Context(p)
    if bcsr is not None:
        ctx.set_operator_bcsr(*bcsr)
    else:
        ctx.set_operator(A)
    return ctx


def make_oracle(A, cfg, tr=False):
    return oracle.Oracle(A, cfg["Nw"], cfg["w"], cfg["dt"], cfg["TransientLength"], transient_removal=tr)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def angles(U, Uref, k, nw, jmax):
    """Angle between u and u_ref (unit vectors after the best unit-modulus
    phase) per (frequency, mode j < jmax); columns iw*k + j. Computed from
    the chord 2 sin(theta/2) = |u - e^{i phi} u_ref|, which stays accurate
    below 1e-8 where arccos|<u, u_ref>| does not."""
    out = np.zeros((jmax, nw))
    for iw in range(nw):
        for j in range(jmax):
            u = U[:, iw * k + j] / np.linalg.norm(U[:, iw * k + j])
            v = Uref[:, iw * k + j] / np.linalg.norm(Uref[:, iw * k + j])
            c = np.vdot(v, u)
            ph = c / abs(c) if abs(c) > 0 else 1.0
            out[j, iw] = 2 * np.arcsin(min(1.0, np.linalg.norm(u - ph * v) / 2))
    return out


def test_grid_matches_oracle(built_lib):
    A, cfg = small_gl()
    ctx = make_ctx(A, cfg, k=2)
    g = ctx.grid()
    dt, Ns, Nt, R = oracle.setup_grid(cfg["w"], cfg["Nw"], cfg["dt"], cfg["TransientLength"])
    assert (g.Ns, g.Nt, g.ResRatio) == (Ns, Nt, R)
    assert g.dt == dt
    ctx.close()


@pytest.mark.parametrize("direction", [1, 0])
def test_rk4_steps_match_oracle(built_lib, direction):
    """A window of forced RK4 steps (SourceCode/TSRK4.c) from a random
    state, past the period wrap of the forcing index."""
    A, cfg = small_gl()
    k = 3
    ctx = make_ctx(A, cfg, k=k)
    g = ctx.grid()
    N, nwe = A.shape[0], g.Nw_eff
    F = synth.complex_normal(N, k * nwe, 5)
    y0 = synth.complex_normal(N, k, 6)
    F30 = synth.complex_normal(N, k, 7)
    ctx.set_sketch(F)
    i0 = 2 * g.Ns - 7  # crosses jt = 2Ns -> 0
    y, F3 = ctx.rk4_steps(direction, i0, 20, y0.copy(), F30.copy())
    orc = make_oracle(A, cfg)
    for ik in range(k):
        Fk = F[:, [iw * k + ik for iw in range(nwe)]]
        yo, F3o = orc.rk4_steps(direction, Fk, i0, 20, y0[:, ik], F30[:, ik])
        # The GPU takes each negative frequency's phasor as the exact
        # conjugate of the positive one; the reference evaluates it from an
        # argument up to 2*pi*2Ns, which carries ~|arg| * 1.1e-16 of its own
        # rounding (here < 1e-12).
        assert rel(y[:, ik], yo) < 1e-11
        assert rel(F3[:, ik], F3o) < 1e-11
    ctx.close()


def test_rk4_steps_continue_and_restage(built_lib):
    """Two calls of 10 steps equal one call of 20 (the staged forcing is
    reused between calls), and a new sketch is restaged (results follow
    the new forcing, against the oracle)."""
    A, cfg = small_gl()
    k = 2
    ctx = make_ctx(A, cfg, k=k)
    g = ctx.grid()
    N, nwe = A.shape[0], g.Nw_eff
    y0 = synth.complex_normal(N, k, 16)
    F30 = synth.complex_normal(N, k, 17)
    for seed in (18, 19):
        F = synth.complex_normal(N, k * nwe, seed)
        ctx.set_sketch(F)
        y1, F31 = ctx.rk4_steps(1, 5, 20, y0.copy(), F30.copy())
        ya, F3a = ctx.rk4_steps(1, 5, 10, y0.copy(), F30.copy())
        yb, F3b = ctx.rk4_steps(1, 15, 10, ya, F3a)
        assert np.array_equal(yb, y1) and np.array_equal(F3b, F31)
        orc = make_oracle(A, cfg)
        for ik in range(k):
            Fk = F[:, [iw * k + ik for iw in range(nwe)]]
            yo, _ = orc.rk4_steps(1, Fk, 5, 20, y0[:, ik], F30[:, ik])
            assert rel(y1[:, ik], yo) < 1e-11, seed
    ctx.close()


@pytest.mark.parametrize("nsteps", [1, 9])
def test_rk4_steps_with_row_kernels_match_oracle(built_lib, nsteps):
    """rsvdt_rk4_steps on the one-lane-per-row kernels, whose last step reads
    F3 back on a second stream while stages 2-4 run: y and F3 against the
    oracle, for a single step and for several."""
    A, cfg = small_gl()
    k = 3
    ctx = make_ctx(A, cfg, k=k)
    ctx.set_lanes_per_row(1)
    g = ctx.grid()
    N, nwe = A.shape[0], g.Nw_eff
    F = synth.complex_normal(N, k * nwe, 25)
    y0 = synth.complex_normal(N, k, 26)
    F30 = synth.complex_normal(N, k, 27)
    ctx.set_sketch(F)
    y, F3 = ctx.rk4_steps(0, 11, nsteps, y0.copy(), F30.copy())
    orc = make_oracle(A, cfg)
    for ik in range(k):
        Fk = F[:, [iw * k + ik for iw in range(nwe)]]
        yo, F3o = orc.rk4_steps(0, Fk, 11, nsteps, y0[:, ik], F30[:, ik])
        assert rel(y[:, ik], yo) < 1e-11 and rel(F3[:, ik], F3o) < 1e-11
    ctx.close()


@pytest.mark.parametrize("nsteps", [1, 9])
def test_rk4_steps_block_rows_match_oracle(built_lib, nsteps):
    """rsvdt_rk4_steps on the complex128 block-row kernels (k_rstage), whose
    last step runs stage 4 in row slabs, each slab's rows of y downloaded
    while the next computes: y and F3 against the oracle."""
    import rsvdt
    bcsr = synth.op3d_blocks(n=4, shift=0.5, seed=8)
    A = synth.bcsr_to_csr(*bcsr)
    cfg = dict(w=0.5, Nw=8, dt=0.05, TransientLength=2 * np.pi / 0.5)
    k = 10
    p = rsvdt.default_params(k=k, q=0, Nw=cfg["Nw"], w=cfg["w"], dt=cfg["dt"],
                             TransientLength=cfg["TransientLength"], Display=0)
    ctx = rsvdt.Context(p)
    ctx.set_operator_bcsr(*bcsr)
    ctx.set_step_engine(rsvdt.ENGINE_STAGES)
    ctx.set_lanes_per_row(1)
    N, nwe = A.shape[0], ctx.grid().Nw_eff
    F = synth.complex_normal(N, k * nwe, 31)
    y0 = synth.complex_normal(N, k, 32)
    F30 = synth.complex_normal(N, k, 33)
    ctx.set_sketch(F)
    orc = oracle.Oracle(A, cfg["Nw"], cfg["w"], cfg["dt"], cfg["TransientLength"])
    for d in (1, 0):
        y, F3 = ctx.rk4_steps(d, 3, nsteps, y0.copy(), F30.copy())
        for ik in range(k):
            Fk = F[:, [iw * k + ik for iw in range(nwe)]]
            yo, F3o = orc.rk4_steps(d, Fk, 3, nsteps, y0[:, ik], F30[:, ik])
            assert rel(y[:, ik], yo) < 1e-11 and rel(F3[:, ik], F3o) < 1e-11, (d, ik)
    orc.close()
    ctx.close()


@pytest.mark.parametrize("direction,tr", [(1, False), (0, False), (1, True), (0, True)])
def test_action_matches_oracle(built_lib, direction, tr):
    """One resolvent action (TSActionRK4 + DFT or transient removal)."""
    A, cfg = small_gl()
    k = 3
    ctx = make_ctx(A, cfg, k=k, tr=tr)
    g = ctx.grid()
    F = synth.complex_normal(A.shape[0], k * g.Nw_eff, 21)
    ctx.set_sketch(F)
    ctx.action(direction)
    Y = ctx.get_block()
    Yo = make_oracle(A, cfg, tr=tr).ts_action(direction, F)
    # Per frequency block relative error.
    for iw in range(g.Nw_eff):
        blk = slice(iw * k, (iw + 1) * k)
        assert rel(Y[:, blk], Yo[:, blk]) < (1e-10 if not tr else 1e-9), iw
    ctx.close()


@pytest.mark.parametrize("case", ["odd_nw", "real_operator"])
def test_plain_forcing_paths_match_oracle(built_lib, case):
    """Forcing without the +-f pairing: an odd number of frequencies, and a
    real operator (positive frequencies only, Nw_eff = Nw/2,
    SourceCode/LNSStructure.c:37-44)."""
    if case == "odd_nw":
        A, cfg = small_gl(Nw=15)
    else:
        A = synth.gl_operator(64, nu=2.0, gamma=1.0, mu0=0.2)  # real-valued
        T = 2 * np.pi / 0.1
        cfg = dict(w=0.1, Nw=16, dt=0.15, TransientLength=T)
    k = 2
    for direction in (1, 0):
        ctx = make_ctx(A, cfg, k=k)
        g = ctx.grid()
        if case == "real_operator":
            assert g.Nw_eff == 8
        F = synth.complex_normal(A.shape[0], k * g.Nw_eff, 31)
        ctx.set_sketch(F)
        ctx.action(direction)
        Y = ctx.get_block()
        Yo = make_oracle(A, cfg).ts_action(direction, F)
        assert rel(Y, Yo) < 1e-11
        ctx.close()


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_lane_split_stepping_matches_oracle(built_lib, lanes):
    """The stepping of one context with 1 lane per (row, test vector) (the
    CSR stage kernels) and with 2, 4, 8 lanes splitting the nonzeros and
    forcing slabs (the batched stage kernel as a batch of one): both
    directions, transient removal on, against the oracle."""
    A, cfg = small_gl()
    k = 3
    for direction in (1, 0):
        ctx = make_ctx(A, cfg, k=k, tr=True)
        ctx.set_lanes_per_row(lanes)
        assert ctx.lanes_per_row() == lanes
        g = ctx.grid()
        F = synth.complex_normal(A.shape[0], k * g.Nw_eff, 41)
        ctx.set_sketch(F)
        ctx.action(direction)
        Y = ctx.get_block()
        Yo = make_oracle(A, cfg, tr=True).ts_action(direction, F)
        assert rel(Y, Yo) < 1e-9
        ctx.close()


def test_qr_and_svd_match_oracle(built_lib):
    A, cfg = small_gl()
    k = 4
    ctx = make_ctx(A, cfg, k=k)
    g = ctx.grid()
    Y = synth.complex_normal(A.shape[0], k * g.Nw_eff, 3)
    # Make some blocks ill-conditioned (kappa ~ 1e4).
    Y[:, 0] *= 1e-4
    ctx.set_sketch(Y)
    ctx.qr_all_freqs()
    Q = ctx.get_block()
    Qo = oracle.qr_all_freqs(Y, k)
    assert rel(Q, Qo) < 1e-11
    for iw in range(g.Nw_eff):
        b = Q[:, iw * k:(iw + 1) * k]
        assert np.abs(b.conj().T @ b - np.eye(k)).max() < 1e-13
    # SVD before the adjoint: the block becomes the left singular vectors.
    ctx.set_sketch(Y)
    ctx.svd_all_freqs(True)
    U = ctx.get_block()
    Uo, So = oracle.svd_all_freqs(Y, k)
    ang = angles(U, Uo, k, g.Nw_eff, k)
    assert ang.max() < 1e-9
    ctx.close()


@pytest.mark.parametrize("q,tr", [(0, False), (1, True)])
def test_run_matches_oracle(built_lib, q, tr):
    """The whole main.c sequence (SourceCode/main.c:134-144)."""
    A, cfg = small_gl()
    k = 3
    ctx = make_ctx(A, cfg, k=k, q=q, tr=tr)
    g = ctx.grid()
    F = synth.complex_normal(A.shape[0], k * g.Nw_eff, 14)
    ctx.set_sketch(F)
    ctx.run()
    U, V, S = ctx.get_results()
    Uo, Vo, So = make_oracle(A, cfg, tr=tr).run(F, q)
    # Per (frequency, j) relative error of every gain.
    rel_gain = np.abs(S - So) / So
    assert rel_gain.max() < GAIN_TOL, rel_gain.max(axis=1)
    assert angles(U, Uo, k, g.Nw_eff, 1).max() < ANGLE_TOL
    assert angles(V, Vo, k, g.Nw_eff, 1).max() < ANGLE_TOL
    ctx.close()


def test_weights_match_oracle(built_lib):
    """Diagonal W_q^{1/2}, W_f^{-1/2}, W_q^{-1/2} and rectangular B, C
    (SourceCode/ApplyWeightMats.c, SourceCode/SVDAllFreqs.c:63-64)."""
    import rsvdt
    A, cfg = small_gl()
    N = A.shape[0]
    k = 2
    rng = np.random.default_rng(3)
    Nb, Nc = 40, 30
    Bm = sp.random(N, Nb, density=0.1, random_state=1, dtype=np.float64).astype(np.complex128) + \
        sp.eye(N, Nb, dtype=np.complex128)
    Cm = sp.random(Nc, N, density=0.1, random_state=2, dtype=np.float64).astype(np.complex128) + \
        sp.eye(Nc, N, dtype=np.complex128)
    wf = rng.uniform(0.5, 1.5, Nb)
    wq = rng.uniform(0.5, 1.5, Nc)
    Wf_inv = sp.diags(1 / np.sqrt(wf) + 0j, format="csr")
    Wq = sp.diags(np.sqrt(wq) + 0j, format="csr")
    Wq_inv = sp.diags(1 / np.sqrt(wq) + 0j, format="csr")
    ctx = make_ctx(A, cfg, k=k, q=1)
    orc = make_oracle(A, cfg)
    for which, M in [(rsvdt.W_F_SQRT_INV, Wf_inv), (rsvdt.B, Bm), (rsvdt.C_OUT, Cm), (rsvdt.W_Q_SQRT, Wq),
                     (rsvdt.W_Q_SQRT_INV, Wq_inv)]:
        ctx.set_weight(which, M)
        orc.set_weight(which, M)
    g = ctx.grid()
    assert (g.Nb, g.Nc) == (Nb, Nc)
    F = synth.complex_normal(Nb, k * g.Nw_eff, 8)
    ctx.set_sketch(F)
    ctx.run()
    U, V, S = ctx.get_results()
    Uo, Vo, So = orc.run(F, 1)
    assert U.shape == (Nc, k * g.Nw_eff) and V.shape == (Nb, k * g.Nw_eff)
    assert (np.abs(S - So) / So).max() < 1e-8
    assert angles(U, Uo, k, g.Nw_eff, 1).max() < ANGLE_TOL
    assert angles(V, Vo, k, g.Nw_eff, 1).max() < ANGLE_TOL
    ctx.close()


@pytest.mark.parametrize("lanes", [1, 0])
def test_bcsr_matches_csr_and_oracle(built_lib, lanes):
    """Block-CSR operator (3D five-field shape, 4^3 grid) against the same
    operator as CSR on the GPU and in the oracle; lanes = 1 runs the 5x5
    block-row kernels, 0 the automatic choice (the lane-split kernel at this
    size)."""
    br, bc, bl = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    Acsr = synth.bcsr_to_csr(br, bc, bl)
    cfg = dict(w=0.5, Nw=8, dt=0.05, TransientLength=2 * np.pi / 0.5)
    k = 2
    ctx_b = make_ctx(None, cfg, k=k, bcsr=(br, bc, bl))
    ctx_c = make_ctx(Acsr, cfg, k=k)
    ctx_b.set_lanes_per_row(lanes)
    ctx_c.set_lanes_per_row(lanes)
    assert ctx_b.lanes_per_row() == (1 if lanes == 1 else 4)
    g = ctx_b.grid()
    F = synth.complex_normal(Acsr.shape[0], k * g.Nw_eff, 9)
    for d in (1, 0):
        ctx_b.set_sketch(F)
        ctx_c.set_sketch(F)
        ctx_b.action(d)
        ctx_c.action(d)
        Yb, Yc = ctx_b.get_block(), ctx_c.get_block()
        Yo = make_oracle(Acsr, cfg).ts_action(d, F)
        assert rel(Yb, Yc) < 1e-12
        assert rel(Yb, Yo) < 1e-11
    ctx_b.close()
    ctx_c.close()


@pytest.mark.parametrize("op,prec", [("csr", 0), ("csr", 1), ("bcsr", 0), ("bcsr", 1)])
def test_cluster_engine_is_bit_identical(built_lib, op, prec):
    """The cluster engine (forcing of 64 steps over the GPU, then the steps'
    stages on one thread-block cluster) against the one-lane stage kernels:
    identical bits after whole actions in both directions, with and without
    transient removal, and through rsvdt_rk4_steps from an arbitrary step.
    CSR: the 64-node Ginzburg-Landau operator, k = 3; block CSR: the 4^3
    five-field operator, k = 2."""
    import rsvdt
    if op == "csr":
        A, cfg = small_gl()
        bcsr, k = None, 3
    else:
        bcsr = synth.op3d_blocks(n=4, shift=0.5, seed=3)
        A = synth.bcsr_to_csr(*bcsr)
        cfg, k = dict(w=0.5, Nw=8, dt=0.05, TransientLength=2 * np.pi / 0.5), 2
    out = {}
    for engine in (rsvdt.ENGINE_STAGES, rsvdt.ENGINE_CLUSTER):
        res = []
        for tr in (False, True):
            ctx = make_ctx(A, cfg, k=k, tr=tr, prec=prec, bcsr=bcsr)
            ctx.set_lanes_per_row(1)
            ctx.set_step_engine(engine)
            assert ctx.step_engine() == engine
            F = synth.complex_normal(A.shape[0], k * ctx.grid().Nw_eff, 6)
            for d in (1, 0):
                ctx.set_sketch(F)
                ctx.action(d)
                res.append(ctx.get_block())
            if prec == 0 and not tr:
                y0 = synth.complex_normal(A.shape[0], k, 7)
                f0 = synth.complex_normal(A.shape[0], k, 8)
                res.extend(ctx.rk4_steps(1, 37, 70, y0, f0))
            ctx.close()
        out[engine] = res
    for a, b in zip(out[rsvdt.ENGINE_STAGES], out[rsvdt.ENGINE_CLUSTER]):
        assert np.isfinite(a).all() and np.array_equal(a, b)


def test_c64_form_close_to_c128(built_lib):
    """Precision form: complex64 operator/state/stages with FP32 accumulation,
    FP64 DFT/QR/SVD. Gains within 1e-3 of the complex128 plain form."""
    A, cfg = small_gl()
    k = 3
    g128 = make_ctx(A, cfg, k=k, q=1, tr=True)
    g64 = make_ctx(A, cfg, k=k, q=1, tr=True, prec=1)
    F = synth.complex_normal(A.shape[0], k * g128.grid().Nw_eff, 14)
    for c in (g128, g64):
        c.set_sketch(F)
        c.run()
    _, _, S128 = g128.get_results()
    _, _, S64 = g64.get_results()
    assert (np.abs(S64 - S128) / S128)[0].max() < 1e-3
    g128.close()
    g64.close()


def test_refine_form_recovers_fp64_gains(built_lib):
    """Precision form with one FP64 sweep (the last adjoint action in
    complex128): on the non-normal Ginzburg-Landau operator its gains are
    closer to the complex128 plain form than the all-complex64 form's for
    the leading mode."""
    import rsvdt
    A, cfg = small_gl()
    k = 4
    F = None
    S = {}
    for prec in (rsvdt.PREC_C128, rsvdt.PREC_C64, rsvdt.PREC_C64_REFINE):
        ctx = make_ctx(A, cfg, k=k, q=1, tr=True, prec=prec)
        if F is None:
            F = synth.complex_normal(A.shape[0], k * ctx.grid().Nw_eff, 15)
        ctx.set_sketch(F)
        ctx.run()
        S[prec] = ctx.get_results()[2]
        # The context keeps its precision form across runs.
        ctx.set_sketch(F)
        ctx.run()
        assert np.array_equal(ctx.get_results()[2], S[prec])
        ctx.close()
    e64 = (np.abs(S[rsvdt.PREC_C64] - S[rsvdt.PREC_C128]) / S[rsvdt.PREC_C128])
    eref = (np.abs(S[rsvdt.PREC_C64_REFINE] - S[rsvdt.PREC_C128]) / S[rsvdt.PREC_C128])
    print("refine vs c64 gain errors, mode 1:", eref[0].max(), e64[0].max(), "modes<=3:", eref[:3].max(),
          e64[:3].max())
    assert eref[0].max() < e64[0].max() and eref[:3].max() < 1e-3


def test_progress_output_and_phase_timings(built_lib, capfd):
    """Display = 2 prints the reference's progress lines
    (SourceCode/DisplayProgress.c:18-50, SourceCode/TSActionRK4.c:150-160);
    rsvdt_get_timings counts the actions and steps of the run and splits
    its wall time into phases."""
    import rsvdt
    A, cfg = small_gl()
    k = 2
    p = rsvdt.default_params(k=k, q=1, Nw=cfg["Nw"], w=cfg["w"], dt=cfg["dt"],
                             TransientLength=cfg["TransientLength"], Display=2)
    ctx = rsvdt.Context(p)
    ctx.set_operator(A)
    g = ctx.grid()
    ctx.set_sketch(synth.complex_normal(A.shape[0], k * g.Nw_eff, 2))
    capfd.readouterr()
    ctx.run()
    out = capfd.readouterr().out
    assert out.count("Progress percentage: 50%") == 4 and out.count("Progress percentage: 100%") == 4
    assert out.count("*** Direct action elapsed time = ") == 2
    assert out.count("*** Adjoint action elapsed time = ") == 2
    assert f"(k = {k} out of {k})" in out
    t = ctx.timings()
    assert t["actions"] == {"direct": 2, "adjoint": 2}
    assert t["steps"] == 4 * (g.Nt + g.Ns)
    assert all(v >= 0 for v in t["seconds"].values()) and t["seconds"]["stepping"] > 0
    ctx.reset_timings()
    assert ctx.timings()["steps"] == 0
    ctx.close()


def test_nan_in_the_operator_is_reported(built_lib):
    """A NaN injected into A on the host propagates through the stepping and
    the action returns RSVDT_ERR_DIVERGED with a message (the context stays
    usable: a clean operator afterwards runs normally)."""
    import rsvdt
    A, cfg = small_gl()
    Abad = A.tolil()
    Abad[10, 11] = np.nan
    ctx = make_ctx(Abad.tocsr(), cfg, k=2)
    F = synth.complex_normal(A.shape[0], 2 * ctx.grid().Nw_eff, 3)
    ctx.set_sketch(F)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.action(1)
    assert e.value.status == rsvdt.ERR_DIVERGED and "NaN" in str(e.value)
    ctx.set_operator(A)
    ctx.set_sketch(F)
    ctx.action(1)
    assert np.isfinite(ctx.get_block()).all()
    ctx.close()


def test_3d_gains_match_the_dense_resolvent(built_lib):
    """The 3D five-field operator (6^3 grid, N = 1080, block-CSR), shifted so
    that its rightmost eigenvalue (dense eigensolver) sits at -0.05, diagonal
    W_q = W_f, k = 8, q = 4, transient removal: the leading gain of the whole
    sequence in the plain and the refinement forms against a dense FP64 SVD
    of W_q^{1/2} (i w I - A)^{-1} W_f^{-1/2} wherever sigma_1 / sigma_2 > 1.5
    (the oracle's own run of this case agrees to 1.3e-5 there)."""
    import rsvdt
    from rsvdt import workloads
    br, bc, bl = synth.op3d_blocks(n=6, seed=7, shift=0.0)
    abscissa = np.linalg.eigvals(synth.bcsr_to_csr(br, bc, bl).toarray()).real.max()
    br, bc, bl = synth.op3d_blocks(n=6, seed=7, shift=abscissa + 0.05)
    A = synth.bcsr_to_csr(br, bc, bl)
    N = A.shape[0]
    w, Nw, k, q = 0.1, 8, 8, 4
    dt = 1.0 / workloads.gershgorin_bound_bcsr(br, bc, bl)
    Wq, Wq_inv = synth.diag_weights(N, seed=11)
    F = synth.complex_normal(N, k * Nw, 17)
    res = {}
    for prec in (rsvdt.PREC_C128, rsvdt.PREC_C64_REFINE):
        p = rsvdt.default_params(k=k, q=q, Nw=Nw, w=w, dt=dt, TransientLength=2 * 2 * np.pi / w,
                                 TransientRemoval=1, precision=prec, Display=0)
        ctx = rsvdt.Context(p)
        ctx.set_operator_bcsr(br, bc, bl)
        for which, M in [(rsvdt.W_F_SQRT_INV, Wq_inv), (rsvdt.W_Q_SQRT, Wq), (rsvdt.W_Q_SQRT_INV, Wq_inv)]:
            ctx.set_weight(which, M)
        ctx.set_sketch(F)
        ctx.run()
        res[prec] = ctx.get_results()[2]
        ctx.close()
    om = [oracle.freq_of(i, Nw, w) for i in range(Nw)]
    Sd, _, _ = oracle.dense_resolvent_svd(A, om, 2, Wq=Wq, Wf_inv=Wq_inv)
    good = Sd[0] / Sd[1] > 1.5
    assert good.sum() >= 3
    for prec, S in res.items():
        err = (np.abs(S[0, good] - Sd[0, good]) / Sd[0, good]).max()
        print("3D gains vs dense resolvent, precision form", prec, "max rel err", err)
        assert err < 1e-4, (prec, err)


def test_checkpoint_resumes_exactly(built_lib):
    """rsvdt_set_checkpoint: the block read at power sweep j, set as the
    sketch of a run with q - j sweeps, reproduces the uninterrupted run's
    gains and modes bit for bit; a callback returning true stops the run."""
    import rsvdt
    A, cfg = small_gl()
    k, q = 3, 2
    ctx = make_ctx(A, cfg, k=k, q=q, tr=True)
    F = synth.complex_normal(A.shape[0], k * ctx.grid().Nw_eff, 23)
    saved = {}

    def keep(sweep):
        saved[sweep] = ctx.get_block()
        return False

    ctx.set_checkpoint(keep)
    ctx.set_sketch(F)
    ctx.run()
    U, V, S = ctx.get_results()
    assert sorted(saved) == [1, 2]
    ctx.set_checkpoint(lambda sweep: sweep == 1)
    ctx.set_sketch(F)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.run()
    assert e.value.status == rsvdt.ERR_STATE and "checkpoint" in str(e.value)
    ctx.close()
    for sweep, Q in saved.items():
        c2 = make_ctx(A, cfg, k=k, q=q - sweep, tr=True)
        c2.set_sketch(Q)
        c2.run()
        U2, V2, S2 = c2.get_results()
        c2.close()
        assert np.array_equal(S2, S) and np.array_equal(U2, U) and np.array_equal(V2, V), sweep


def test_diverged_and_state_errors(built_lib):
    import rsvdt
    A, cfg = small_gl()
    # Strongly unstable operator: the response overflows to Inf/NaN.
    Abad = A + sp.eye(A.shape[0]) * 40.0
    ctx = make_ctx(Abad, cfg, k=1)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.action(1)  # no sketch yet
    assert e.value.status == rsvdt.ERR_STATE
    F = synth.complex_normal(A.shape[0], ctx.grid().Nw_eff, 1)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.set_sketch(F[:, :-1])
    assert e.value.status == rsvdt.ERR_ARG
    ctx.set_sketch(F)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.action(1)
    assert e.value.status == rsvdt.ERR_DIVERGED
    ctx.close()


@pytest.mark.parametrize("q,tr", [(0, False), (1, True)])
def test_gl1_config_matches_oracle(built_lib, q, tr):
    """The Ginzburg-Landau benchmark configuration at full size: N=500,
    k=10, 64 frequencies j*0.1 (j=-32..31), dt=T/4096, one transient
    period, q in {0, 1}."""
    A = synth.gl_operator(500)
    dt, T = synth.gl_time_grid(0.1, 4096)
    cfg = dict(w=0.1, Nw=64, dt=dt, TransientLength=T)
    k = 10
    ctx = make_ctx(A, cfg, k=k, q=q, tr=tr)
    g = ctx.grid()
    assert (g.Ns, g.Nt, g.ResRatio) == (4096, 4096, 64)
    F = synth.gl_sketch(500, k, 64, seed=14)
    ctx.set_sketch(F)
    ctx.run()
    U, V, S = ctx.get_results()
    Uo, Vo, So = make_oracle(A, cfg, tr=tr).run(F, q)
    assert (np.abs(S - So) / So)[:3].max() < GAIN_TOL
    assert angles(U, Uo, k, 64, 1).max() < ANGLE_TOL
    assert angles(V, Vo, k, 64, 1).max() < ANGLE_TOL
    ctx.close()


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 1e-5)])  # complex128, complex64 form
@pytest.mark.parametrize("direction", [1, 0])
def test_actions_are_the_rk4_transfer_function(built_lib, prec, tol, direction):
    """The actions of a diagonal operator on the GPU against the closed
    form of forced RK4 (oracle.rk4_tone_response: each row a scalar ODE),
    independently of the C restatement, once the transient has decayed:
    direct Y[:, iw k + j] = e^{i w (Nt + R) dt} H(lam, w) F[:, iw k + j],
    adjoint (A^H, time-reversed forcing, samples in reverse slot order)
    e^{-i w Nt dt} conj(H) F; complex128 to rounding, the complex64 form to
    its FP32 state."""
    import rsvdt
    N, w, Nw, k = 12, 0.1, 16, 2
    rng = np.random.default_rng(8)
    lam = -1.0 - 2.0 * rng.random(N) + 1j * rng.uniform(-3, 3, N)
    A = sp.diags(lam).tocsr()
    cfg = dict(w=w, Nw=Nw, dt=0.15, TransientLength=2 * np.pi / w)
    ctx = make_ctx(A, cfg, k=k, prec=prec)
    g = ctx.grid()
    z = lam * g.dt
    assert g.Nt == g.Ns and (np.abs(1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24) ** g.Nt < 1e-15).all()
    F = synth.complex_normal(N, k * Nw, 10)
    ctx.set_sketch(F)
    ctx.action(direction)
    Y = ctx.get_block()
    ctx.close()
    for iw in range(Nw):
        om = oracle.freq_of(iw, Nw, w)
        H = oracle.rk4_tone_response(lam, om, g.dt)
        if direction == rsvdt.DIRECT:
            resp = np.exp(1j * om * (g.Nt + g.ResRatio) * g.dt) * H
        else:
            resp = np.exp(-1j * om * g.Nt * g.dt) * np.conj(H)
        for j in range(k):
            c = iw * k + j
            expect = resp * F[:, c]
            assert np.abs(Y[:, c] - expect).max() / np.abs(expect).max() < tol, (iw, j)


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 1e-5)])  # complex128, complex64 form
def test_real_operator_action_is_the_rk4_transfer_function(built_lib, prec, tol):
    """A real diagonal operator (the real-operator branch: Nw/2 non-negative
    frequencies) on the GPU against the closed form of forced RK4."""
    import rsvdt
    N, w, Nw, k = 12, 0.1, 16, 2
    lam = -1.0 - 2.0 * np.random.default_rng(8).random(N) + 0j
    cfg = dict(w=w, Nw=Nw, dt=0.15, TransientLength=2 * np.pi / w)
    ctx = make_ctx(sp.diags(lam).tocsr(), cfg, k=k, prec=prec)
    g = ctx.grid()
    assert g.Nw_eff == Nw // 2
    F = synth.complex_normal(N, k * g.Nw_eff, 11)
    ctx.set_sketch(F)
    ctx.action(rsvdt.DIRECT)
    Y = ctx.get_block()
    ctx.close()
    for iw in range(g.Nw_eff):
        om = oracle.freq_of(iw, Nw, w, real_op=True)
        resp = np.exp(1j * om * (g.Nt + g.ResRatio) * g.dt) * oracle.rk4_tone_response(lam, om, g.dt)
        for j in range(k):
            c = iw * k + j
            expect = resp * F[:, c]
            assert np.abs(Y[:, c] - expect).max() / np.abs(expect).max() < tol, (iw, j)


# complex128 to rounding; the complex64 form to its FP32 state (mode errors
# up to about 1e-4 after a power iteration, where two gains are close).
@pytest.mark.parametrize("prec,q,gtol,mtol", [(0, 0, 1e-10, 1e-8), (0, 1, 1e-10, 1e-8), (1, 0, 1e-5, 1e-4),
                                              (1, 1, 1e-5, 1e-3)])
def test_whole_run_of_a_diagonal_operator_is_exact(built_lib, prec, q, gtol, mtol):
    """The whole sequence on the GPU with a full sketch (k = N) on a
    diagonal operator with diagonal weights, against the closed form rather
    than the restatement: gains = the sorted |a_n H_n b_n| (H the forced-RK4
    answer, a = W_q^{1/2}, b = W_f^{-1/2}), V's columns e_n b_n, U's
    columns e_n / a_n from q = 1 on (U is taken before the adjoint: at q = 0
    it is the left singular basis of R F, which depends on the sketch)."""
    import rsvdt
    N, w, Nw = 12, 0.1, 16
    rng = np.random.default_rng(8)
    lam = -1.0 - 2.0 * rng.random(N) + 1j * rng.uniform(-3, 3, N)
    vol = rng.uniform(0.5, 1.5, N)
    a, b = np.sqrt(vol), 1 / np.sqrt(vol)
    cfg = dict(w=w, Nw=Nw, dt=0.15, TransientLength=2 * np.pi / w)
    ctx = make_ctx(sp.diags(lam).tocsr(), cfg, k=N, q=q, prec=prec)
    ctx.set_weight(rsvdt.W_Q_SQRT, sp.diags(a + 0j).tocsr())
    ctx.set_weight(rsvdt.W_F_SQRT_INV, sp.diags(b + 0j).tocsr())
    ctx.set_weight(rsvdt.W_Q_SQRT_INV, sp.diags(1 / a + 0j).tocsr())
    ctx.set_sketch(synth.complex_normal(N, N * Nw, 9))
    ctx.run()
    U, V, S = ctx.get_results()
    dt = ctx.grid().dt
    ctx.close()
    for iw in range(Nw):
        g = np.abs(a * oracle.rk4_tone_response(lam, oracle.freq_of(iw, Nw, w), dt) * b)
        order = np.argsort(-g)
        assert (np.abs(S[:, iw] - g[order]) / g[order]).max() < gtol, iw
        for j in range(3):
            n = order[j]
            for M, scale, check in ((V, b[n], True), (U, 1 / a[n], q >= 1)):
                if not check:
                    continue
                col = M[:, iw * N + j]
                e = np.zeros(N)
                e[n] = scale
                c = np.vdot(e, col) / np.vdot(e, e)
                assert abs(abs(c) - 1) < mtol and np.linalg.norm(col - c * e) / scale < mtol, (iw, j)
