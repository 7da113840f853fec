"""The transient-simulation oracle (oracle/trans_ref.py) against closed
forms: RK4 of a diagonal operator is y_n = P(lambda dt)^n y_0, and the DFT
of geometric snapshot sequences is a geometric sum. Also the run loop's
stopping rules (SourceCode/TransientRunRK4.c:137-158)."""
import math

import numpy as np
import scipy.sparse as sp

from oracle import trans_ref


def _diag(lams):
    return sp.diags(np.asarray(lams, dtype=np.complex128)).tocsr()


def test_time_grid_follows_the_reference_rule():
    w, Nw = 0.1, 8
    dt_g = trans_ref.grid_dt(w, Nw, 0.15)
    dt, Ntp, Rd, rend, n_saved = trans_ref.trans_grid(w, Nw, dt_g, periods=3, save_mod=7)
    T = 2 * math.pi / w
    assert abs(dt - (T / Nw) / math.ceil((T / Nw) / dt_g)) == 0
    assert Ntp == round(T / dt) and Ntp % Nw == 0 and Rd == Ntp // Nw
    assert rend == 3 * Ntp and n_saved == rend // 7 + 1


def test_diagonal_operator_matches_the_rk4_amplification():
    rng = np.random.default_rng(0)
    lam = -rng.uniform(0.01, 0.3, 12) + 1j * rng.uniform(-1, 1, 12)
    q0 = rng.standard_normal(12) + 1j * rng.standard_normal(12)
    w, Nw = 0.1, 8
    dt_g = trans_ref.grid_dt(w, Nw, 0.2)
    out = trans_ref.trans_run(_diag(lam), q0, w, Nw, dt_g, periods=2, save_mod=25, con_val=0.0)
    dt = out["dt"]
    P = trans_ref.rk4_amplification(lam * dt)
    assert out["stop"] == 0 and out["steps"] == out["rend"]
    ref = P ** out["rend"] * q0
    assert np.linalg.norm(out["q"] - ref) <= 1e-12 * np.linalg.norm(ref)
    for pos in range(out["norms"].size):
        ref_n = np.linalg.norm(P ** (pos * 25) * q0)
        assert abs(out["norms"][pos] - ref_n) <= 1e-12 * ref_n
        assert np.allclose(out["snapshots"][pos], P ** (pos * 25) * q0, rtol=1e-12, atol=0)


def test_removal_estimate_initial_norms_are_geometric_sums():
    """First period, diagonal operator: snapshot column j = r^j q0 with
    r = P(lambda dt)^R, so column iw of Q dft / Nw is
    q0 (1 - r^Nw) / (1 - r e^{-2 pi i iw / Nw}) / Nw."""
    rng = np.random.default_rng(1)
    n = 10
    lam = -rng.uniform(0.02, 0.1, n) + 1j * rng.uniform(-0.5, 0.5, n)
    q0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    w, Nw = 0.1, 8
    dt_g = trans_ref.grid_dt(w, Nw, 0.25)
    out = trans_ref.trans_run(_diag(lam), q0, w, Nw, dt_g, periods=1, save_mod=10 ** 6, con_val=0.0,
                              removal_est_flag=True)
    assert len(out["estimates"]) == 1
    period, initial, updated = out["estimates"][0]
    assert period == 1 and initial.size == Nw // 2
    R = out["Nt_period"] // Nw
    r = trans_ref.rk4_amplification(lam * out["dt"]) ** R
    for iw in range(Nw // 2):
        col = q0 * (1 - r ** Nw) / (1 - r * np.exp(-2j * np.pi * iw / Nw)) / Nw
        assert abs(initial[iw] - np.linalg.norm(col)) <= 1e-12 * np.linalg.norm(col)
    assert np.all(updated >= 0) and np.all(updated <= 1 + 1e-12)


def test_stopping_rules():
    w, Nw = 0.1, 8
    dt_g = trans_ref.grid_dt(w, Nw, 0.2)
    q0 = np.ones(4, dtype=np.complex128) / 2
    # Growth: the first check above TransDivVal stops the run.
    out = trans_ref.trans_run(_diag([0.05] * 4), q0, w, Nw, dt_g, periods=5, save_mod=10, div_val=2.0)
    assert out["stop"] == 2
    s = out["steps"]
    assert s % 10 == 0 and np.linalg.norm(out["q"]) > 2.0
    assert out["norms"][s // 10] == 0 and 0 < out["norms"][s // 10 - 1] <= 2.0
    # Decay below TransConVal.
    out = trans_ref.trans_run(_diag([-0.5] * 4), q0, w, Nw, dt_g, periods=5, save_mod=10, con_val=1e-3)
    assert out["stop"] == 3 and np.linalg.norm(out["q"]) < 1e-3
    # A NaN in the initial vector: stopped at the first check.
    qn = q0.copy()
    qn[1] = np.nan
    out = trans_ref.trans_run(_diag([-0.1] * 4), qn, w, Nw, dt_g, periods=1, save_mod=10)
    assert out["stop"] == 1 and out["steps"] == 10
