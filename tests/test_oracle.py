"""The CPU oracle against closed forms, the dense FP64 resolvent and the
reference's tutorial known answer (tests/golden/, made by make_golden.py)."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from rsvdt import petsc_io, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_time_grid_follows_setup_time_freq_grid():
    # SourceCode/SetupTimeFreqGrid.c:16-21 on the two configurations used.
    dt, T = synth.gl_time_grid(0.1, 4096)
    assert oracle.setup_grid(0.1, 64, dt, T)[1:] == (4096, 4096, 64)
    d, Ns, Nt, R = oracle.setup_grid(0.05, 42, 0.003, 10.0)
    T = 2 * math.pi / 0.05
    assert Ns == 42 * math.ceil((T / 42) / 0.003)
    assert (Ns, Nt, R) == (41916, 3336, 998)
    assert abs(d - (T / 42) / math.ceil((T / 42) / 0.003)) < 1e-18


@pytest.mark.parametrize("Nw", [8, 7, 16])
def test_idft_and_dft_tables(Nw):
    """idft[iw, jt] = exp(+2 pi i f jt / (2 Ns)) / Ns with f = iw for the
    first half and iw - Nw for the rest (SourceCode/CreateDFTiDFTMats.c:42-59),
    dft[j, iw] = exp(-2 pi i j iw / Nw) (:61-85)."""
    Ns = 5 * Nw
    idft = np.zeros(2 * Nw * 2 * Ns)
    oracle.lib().orc_build_idft(Nw, Ns, 0, oracle._d(idft))
    idft = idft.view(complex).reshape(Nw, 2 * Ns)
    half = Nw // 2 - 1 if Nw % 2 == 0 else (Nw - 1) // 2
    f = np.array([i if i <= half else i - Nw for i in range(Nw)])
    jt = np.arange(2 * Ns)
    ref = np.exp(2j * np.pi * np.outer(f, jt) / (2 * Ns)) / Ns
    assert np.abs(idft - ref).max() < 1e-13
    dft = np.zeros(2 * Nw * Nw)
    oracle.lib().orc_build_dft(Nw, Nw, 0, oracle._d(dft))
    dft = dft.view(complex).reshape(Nw, Nw)  # [iw][j]
    j = np.arange(Nw)
    assert np.abs(dft - np.exp(-2j * np.pi * np.outer(np.arange(Nw), j) / Nw)).max() < 1e-13


def _small():
    A = synth.gl_operator(64, mu0=0.2)
    w, Nw = 0.1, 16
    return A, w, Nw, 0.15, 2 * np.pi / w


def test_direct_action_is_the_resolvent_up_to_a_phase():
    """Y[:, iw] = e^{i w (Nt+R) dt} R(w) F[:, iw] to RK4 / transient accuracy
    with transient removal (the reference's phase convention)."""
    A, w, Nw, dt, T = _small()
    o = oracle.Oracle(A, Nw, w, dt, T, transient_removal=True)
    F = synth.complex_normal(64, Nw, 3)
    Y = o.ts_action(1, F)
    Ad = A.toarray()
    for iw in range(Nw):
        om = oracle.freq_of(iw, Nw, w)
        x = np.linalg.solve(1j * om * np.eye(64) - Ad, F[:, iw])
        ph = np.exp(1j * om * (o.Nt + o.R) * o.dt)
        assert np.linalg.norm(Y[:, iw] - ph * x) / np.linalg.norm(x) < 1e-4


def test_real_operator_action_is_the_resolvent_up_to_a_phase():
    """A real-valued operator keeps the Nw/2 non-negative frequencies; the
    DFT over the Nw snapshots of one period then picks frequency iw * w
    (SourceCode/CreateDFTiDFTMats.c:79, alpha = -2 pi i / (2 Nw_eff))."""
    A = synth.gl_operator(64, nu=2.0, gamma=1.0, mu0=0.2)
    w, Nw, dt, T = 0.1, 16, 0.15, 2 * np.pi / 0.1
    o = oracle.Oracle(A, Nw, w, dt, T, transient_removal=True)
    assert o.real_op and o.Nw_eff == Nw // 2
    F = synth.complex_normal(64, Nw // 2, 13)
    Y = o.ts_action(1, F)
    Ad = A.toarray()
    for iw in range(Nw // 2):
        om = oracle.freq_of(iw, Nw, w, real_op=True)
        x = np.linalg.solve(1j * om * np.eye(64) - Ad, F[:, iw])
        ph = np.exp(1j * om * (o.Nt + o.R) * o.dt)
        assert np.linalg.norm(Y[:, iw] - ph * x) / np.linalg.norm(x) < 1e-4, iw


def test_adjoint_action_is_the_adjoint_resolvent_up_to_a_phase():
    A, w, Nw, dt, T = _small()
    o = oracle.Oracle(A, Nw, w, dt, T, transient_removal=True)
    F = synth.complex_normal(64, Nw, 4)
    Y = o.ts_action(0, F)
    Ad = A.toarray()
    for iw in range(Nw):
        om = oracle.freq_of(iw, Nw, w)
        x = np.linalg.solve((1j * om * np.eye(64) - Ad).conj().T, F[:, iw])
        c = np.vdot(x, Y[:, iw]) / np.vdot(x, x)
        assert abs(abs(c) - 1) < 1e-4
        assert np.linalg.norm(Y[:, iw] - c * x) / np.linalg.norm(x) < 1e-4


def test_rsvd_gains_match_the_dense_resolvent():
    A, w, Nw, dt, T = _small()
    o = oracle.Oracle(A, Nw, w, dt, T, transient_removal=True)
    k = 4
    F = synth.complex_normal(64, k * Nw, 5)
    _, _, S = o.run(F, 1)
    om = [oracle.freq_of(i, Nw, w) for i in range(Nw)]
    Sd, _, _ = oracle.dense_resolvent_svd(A, om, k)
    gap = Sd[0] / Sd[1]
    good = gap > 3
    assert good.sum() >= 4
    # RK4 truncation error at |lambda| dt ~ 1.8 bounds the agreement here.
    assert (np.abs(S[0, good] - Sd[0, good]) / Sd[0, good]).max() < 1e-3


def test_qr_and_svd_helpers():
    Y = synth.complex_normal(50, 12, 6)
    Q = oracle.qr_all_freqs(Y, 4)
    for iw in range(3):
        b = Q[:, iw * 4:(iw + 1) * 4]
        assert np.abs(b.conj().T @ b - np.eye(4)).max() < 1e-14
        R = b.conj().T @ Y[:, iw * 4:(iw + 1) * 4]
        assert np.allclose(np.tril(R, -1), 0, atol=1e-12)
        assert (np.diag(R).real > 0).all() and np.abs(np.diag(R).imag).max() < 1e-12
    U, S = oracle.svd_all_freqs(Y, 4)
    for iw in range(3):
        s = np.linalg.svd(Y[:, iw * 4:(iw + 1) * 4], compute_uv=False)
        assert np.abs(S[:, iw] - s).max() / s[0] < 1e-14


def test_golden_tutorial_known_answer():
    """The reference's own known answer (Tutorial/Ginzburg-Landau: sigma_1
    peaks near 1.6e3 at omega = -0.65, gains.png) holds for the dense
    resolvent of the shipped operator and for the oracle's RSVD-dt run of the
    full tutorial configuration stored in the fixture."""
    g = json.load(open(os.path.join(GOLDEN, "gl_tutorial.json")))
    om = np.array(g["omega"])
    Sd = np.array(g["dense_gains"])
    So = np.array(g["oracle_gains"])
    ka = g["known_answer"]
    iw = int(np.argmax(Sd[0]))
    assert abs(om[iw] - ka["omega_peak"]) < 1e-12
    assert abs(Sd[0, iw] - ka["sigma1_peak"]) / ka["sigma1_peak"] < 0.06
    assert int(np.argmax(So[0])) == iw
    assert abs(So[0, iw] - Sd[0, iw]) / Sd[0, iw] < 1e-6
    # Leading gains of the RSVD-dt run against the dense oracle wherever the
    # singular-value gap lets k=10, q=1 converge.
    good = Sd[0] / Sd[1] > 2
    assert (np.abs(So[0, good] - Sd[0, good]) / Sd[0, good]).max() < 1e-3
    assert g["grid"] == {"dt": g["grid"]["dt"], "Ns": 41916, "Nt": 3336, "ResRatio": 998}


@pytest.mark.slow
def test_oracle_reproduces_the_tutorial_peak():
    """Re-runs the oracle on the shipped A_GL (k=2, q=0, transient removal)
    and recovers the published peak gain at omega = -0.65."""
    A = petsc_io.read_mat(os.path.join(GOLDEN, "A_GL"))
    o = oracle.Oracle(A, 42, 0.05, 0.003, 10.0, transient_removal=True)
    F = synth.gl_sketch(500, 2, 42, seed=14)
    _, _, S = o.run(F, 0)
    g = json.load(open(os.path.join(GOLDEN, "gl_tutorial.json")))
    Sd = np.array(g["dense_gains"])
    iw = int(np.argmax(Sd[0]))
    assert abs(S[0, iw] - Sd[0, iw]) / Sd[0, iw] < 1e-4


def test_row_threads_do_not_change_the_result():
    """The RK4 step's row loops on several threads (the CPU baseline's
    setting) give bit-identical results: rows are independent and each sum
    keeps its order."""
    A, w, Nw, dt, T = _small()
    o = oracle.Oracle(A, Nw, w, dt, T)
    F = synth.complex_normal(64, Nw, 9)
    y0 = synth.complex_normal(64, 1, 10)[:, 0]
    f0 = synth.complex_normal(64, 1, 11)[:, 0]
    ya, fa = o.rk4_steps(1, F, 3, 25, y0.copy(), f0.copy())
    o.set_row_threads(4)
    yb, fb = o.rk4_steps(1, F, 3, 25, y0.copy(), f0.copy())
    assert np.array_equal(ya, yb) and np.array_equal(fa, fb)


def test_sparse_resolvent_oracle_matches_the_dense_one():
    """oracle.sparse_resolvent_svd (sparse LU + Lanczos, the exact-resolvent
    oracle for sizes a dense inverse cannot hold) against the dense SVD on
    the 4^3 five-field operator with diagonal weights, serially and in a
    spawned pool."""
    br, bc, bl = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    A = synth.bcsr_to_csr(br, bc, bl)
    Wq, Wqi = synth.diag_weights(A.shape[0], seed=5)
    om = [0.0, 0.3, -0.6]
    Sd, Ud, Vd = oracle.dense_resolvent_svd(A, om, 3, Wq=Wq, Wf_inv=Wqi)
    for procs in (1, 2):
        S, U, V = oracle.sparse_resolvent_svd(A, om, 3, wq=Wq.diagonal(), wf_inv=Wqi.diagonal(), procs=procs)
        assert np.abs(S - Sd).max() / Sd.max() < 1e-10
        for j in range(len(om)):
            for X, Xd in ((U, Ud), (V, Vd)):
                c = abs(np.vdot(Xd[j][:, 0], X[j][:, 0]))
                assert abs(c - 1) < 1e-8


@pytest.mark.parametrize("Nw", [16, 7])
def test_actions_are_the_rk4_transfer_function(Nw):
    """For a diagonal operator the direct action is known in closed form:
    each row is a scalar ODE y' = lam y + f(t), and forced RK4 with the
    forcing at t, t + dt/2 (twice) and t + dt (SourceCode/TSRK4.c:18-47)
    answers a tone e^{i w t} in steady state with y_n = H e^{i w n dt},
        H = dt G / (e^{i w dt} - P(z)),  z = lam dt,
        P(z) = 1 + z + z^2/2 + z^3/6 + z^4/24,
        G = (k1 + 2 k2 + 2 k3 + k4) / 6,  k1 = 1, k2 = z/2 + a,
        k3 = (z/2) k2 + a,  k4 = z k3 + b,  a = e^{i w dt/2}, b = e^{i w dt}.
    The idft's 1/Ns, the DFT's ResRatio and the sample times Nt + R (p + 1)
    of SaveSnapshots (SourceCode/SaveSnapshots.c:19-29) then give
    Y[:, iw] = e^{i w (Nt + R) dt} H F[:, iw] exactly, once the transient
    (a factor |P(z)| per step) has decayed: the whole forcing, stepping,
    sampling and DFT chain of the oracle to rounding, not to RK4 accuracy."""
    import scipy.sparse as sp

    N, w, dt_in = 12, 0.1, 0.15
    T = 2 * np.pi / w
    rng = np.random.default_rng(8)
    lam = -1.0 - 2.0 * rng.random(N) + 1j * rng.uniform(-3, 3, N)
    A = sp.diags(lam).tocsr()
    o = oracle.Oracle(A, Nw, w, dt_in, T)
    z = lam * o.dt
    # One transient period: the homogeneous part has decayed below rounding.
    assert o.Nt == o.Ns and (np.abs(1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24) ** o.Nt < 1e-15).all()
    F = synth.complex_normal(N, Nw, 9)
    Y = o.ts_action(1, F)
    dt = o.dt
    for iw in range(Nw):
        om = oracle.freq_of(iw, Nw, w)
        H = oracle.rk4_tone_response(lam, om, dt)
        expect = np.exp(1j * om * (o.Nt + o.R) * dt) * H * F[:, iw]
        err = np.abs(Y[:, iw] - expect).max() / np.abs(expect).max()
        assert err < 1e-12, (iw, om, err)
    # The adjoint action steps A^H with the forcing time-reversed (indices
    # (-1 - m) mod 2 Ns, SourceCode/TSRK4.c:21-26) and stores the samples in
    # reverse slot order (SourceCode/SaveSnapshots.c:24-26): the same
    # algebra gives e^{-i w Nt dt} conj(H) F.
    Ya = o.ts_action(0, F)
    for iw in range(Nw):
        om = oracle.freq_of(iw, Nw, w)
        H = oracle.rk4_tone_response(lam, om, dt)
        expect = np.exp(-1j * om * o.Nt * dt) * np.conj(H) * F[:, iw]
        err = np.abs(Ya[:, iw] - expect).max() / np.abs(expect).max()
        assert err < 1e-12, (iw, om, err)
    o.close()


def test_real_operator_action_is_the_rk4_transfer_function():
    """A real diagonal operator takes the reference's real-operator branch
    (Nw/2 non-negative frequencies, SourceCode/LNSStructure.c:37-44 and
    CreateDFTiDFTMats.c:46-47,63-76); its direct action is the same closed
    form, e^{i w (Nt + R) dt} H F, to rounding."""
    import scipy.sparse as sp

    N, w, Nw, dt_in = 12, 0.1, 16, 0.15
    lam = -1.0 - 2.0 * np.random.default_rng(8).random(N) + 0j
    o = oracle.Oracle(sp.diags(lam).tocsr(), Nw, w, dt_in, 2 * np.pi / w)
    assert o.real_op and o.Nw_eff == Nw // 2
    F = synth.complex_normal(N, Nw // 2, 9)
    Y = o.ts_action(1, F)
    for iw in range(Nw // 2):
        om = oracle.freq_of(iw, Nw, w, real_op=True)
        H = oracle.rk4_tone_response(lam, om, o.dt)
        expect = np.exp(1j * om * (o.Nt + o.R) * o.dt) * H * F[:, iw]
        assert np.abs(Y[:, iw] - expect).max() / np.abs(expect).max() < 1e-12, iw
    o.close()


def _diag_run_expectation(lam, a, b, om, dt, k):
    """Gains and mode rows of W_q^{1/2} R(w) W_f^{-1/2} for a diagonal
    operator and diagonal weights, R the forced-RK4 answer diag(H): the
    singular values are |a_n H_n b_n| sorted, the singular vectors unit
    vectors e_n; after the inverse weights of SourceCode/SVDAllFreqs.c:63-64
    the j-th U and V columns are e_n / a_n and e_n b_n (up to a phase)."""
    g = np.abs(a * oracle.rk4_tone_response(lam, om, dt) * b)
    order = np.argsort(-g)[:k]
    return g[order], order


def test_whole_run_of_a_diagonal_operator_is_exact():
    """The whole sequence of SourceCode/main.c:134-144 (actions, QR, SVD
    before the adjoint, StoreU, adjoint action, SVD, inverse weights) with a
    full sketch (k = N) on a diagonal operator with diagonal weights: the
    gains are the sorted |a_n H_n b_n| to rounding at q = 0 and 1, V's
    columns are e_n b_n; U (taken before the adjoint, SourceCode/StoreU.c:15)
    is the left singular basis of R F, which is e_n / a_n once the sketch
    is orthonormal, from q = 1 on."""
    import scipy.sparse as sp

    N, w, Nw, dt_in = 12, 0.1, 16, 0.15
    rng = np.random.default_rng(8)
    lam = -1.0 - 2.0 * rng.random(N) + 1j * rng.uniform(-3, 3, N)
    vol = rng.uniform(0.5, 1.5, N)
    a, b = np.sqrt(vol), 1 / np.sqrt(vol)  # W_q^{1/2} = W_f^{1/2} = diag(sqrt(vol))
    for q in (0, 1):
        o = oracle.Oracle(sp.diags(lam).tocsr(), Nw, w, dt_in, 2 * np.pi / w)
        o.set_weight(3, sp.diags(a + 0j).tocsr())      # W_q^{1/2}
        o.set_weight(0, sp.diags(b + 0j).tocsr())      # W_f^{-1/2}
        o.set_weight(4, sp.diags(1 / a + 0j).tocsr())  # W_q^{-1/2}
        F = synth.complex_normal(N, N * Nw, 9)
        U, V, S = o.run(F, q)
        for iw in range(Nw):
            g, order = _diag_run_expectation(lam, a, b, oracle.freq_of(iw, Nw, w), o.dt, N)
            assert (np.abs(S[:, iw] - g) / g).max() < 1e-12, (q, iw)
            for j in range(3):
                n = order[j]
                for M, scale, check in ((V, b[n], True), (U, 1 / a[n], q >= 1)):
                    if not check:
                        continue
                    col = M[:, iw * N + j]
                    e = np.zeros(N)
                    e[n] = scale
                    c = np.vdot(e, col) / np.vdot(e, e)
                    assert abs(abs(c) - 1) < 1e-9 and np.linalg.norm(col - c * e) / scale < 1e-9, (q, iw, j)
        o.close()
