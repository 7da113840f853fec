"""Oracle for the transient simulation mode (TEST INFRASTRUCTURE).

Only tests and the smoke check import this module, as the checker. It
restates in numpy, step for step:
  - the time grid of SourceCode/TransientRunRK4.c:39-46;
  - the unforced RK4 step of SourceCode/TSTransRK4.c:15-36;
  - the run loop of SourceCode/TransientRunRK4.c:101-186 (norm checks every
    TransSaveMod steps with the NaN / divergence / convergence stops, the
    snapshot columns of the transient-removal estimate every Nt_period/Nw
    steps);
  - TransientRemovalEst (SourceCode/TransientRemovalEst.c:26-117), with
    the reference's QR (SLEPc BVOrthogonalize) restated as a Householder QR
    (numpy.linalg.qr): both give an orthonormal basis of the same span when
    the synthetic snapshots have full numerical rank.

Parity pin: for a diagonal operator the RK4 iterate has the closed form
y_n = P(lambda dt)^n y_0 with P(z) = 1 + z + z^2/2 + z^3/6 + z^4/24, and
the DFT of geometric snapshot sequences is a geometric sum; the CPU tests
check this module against both.
"""
from __future__ import annotations

import math

import numpy as np


def trans_grid(w: float, Nw: int, dt_grid: float, periods: int, save_mod: int):
    """(dt, Nt_period, Nt_saved_delta, rend, n_saved) of
    SourceCode/TransientRunRK4.c:39-46, from the effective base frequency w
    and the time step of SetupTimeFreqGrid (SourceCode/SetupTimeFreqGrid.c:16-18)."""
    TSS = 2 * math.pi / w
    deltaT = TSS / Nw
    dt = deltaT / math.ceil(deltaT / dt_grid)
    Nt_period = int(round(TSS / dt))
    rend = Nt_period * periods
    return dt, Nt_period, Nt_period // Nw, rend, rend // save_mod + 1


def grid_dt(w: float, Nw: int, dt_in: float) -> float:
    """dt of SourceCode/SetupTimeFreqGrid.c:16-18."""
    T = 2 * math.pi / w
    dt_w = T / Nw
    return dt_w / math.ceil(dt_w / dt_in)


def rk4_step(A, y: np.ndarray, dt: float) -> np.ndarray:
    """One unforced RK4 step (SourceCode/TSTransRK4.c:15-36), in the
    reference's order of vector updates."""
    k1 = A @ y
    k2 = A @ (dt / 2 * k1 + y)
    k3 = A @ (dt / 2 * k2 + y)
    k4 = A @ (dt * k3 + y)
    y = y + dt / 6 * k1
    y = y + dt / 6 * 2 * k2
    y = y + dt / 6 * 2 * k3
    y = y + dt / 6 * k4
    return y


def dft_matrix(Nw: int, Nw_eff: int, real_op: bool) -> np.ndarray:
    """dft (Nw x Nw_eff) of SourceCode/CreateDFTiDFTMats.c:61-85."""
    a = -2 * np.pi / (2 * Nw_eff) if real_op else -2 * np.pi / Nw_eff
    j = np.arange(Nw)[:, None]
    iw = np.arange(Nw_eff)[None, :]
    return np.exp(1j * (a * iw) * j)


def removal_est(Q: np.ndarray, qss: np.ndarray, period: int, w: float, dft: np.ndarray):
    """SourceCode/TransientRemovalEst.c:26-117: Q is N x Ns (Ns = Nw
    snapshot columns). Returns (initial, updated), Nw/2 values each."""
    N, Ns = Q.shape
    Nw = Ns
    deltaT = 2 * np.pi / w / Ns
    ns = Ns - (1 if period == 1 else 0)
    Qhat = Q @ dft / Nw
    H = Nw // 2
    initial = np.linalg.norm(Qhat[:, :H], axis=0)
    updated = np.zeros(H)
    nq = np.linalg.norm(qss)
    for iw in range(H):
        wi = w * iw
        cols = []
        for s in range(ns):
            s1 = s + 1 if period == 1 else s
            cols.append(Q[:, s1] + qss * np.exp(1j * wi * s * deltaT))
        U, _ = np.linalg.qr(np.stack(cols, axis=1))
        r = qss - U @ (U.conj().T @ qss)
        updated[iw] = np.linalg.norm(r) / nq
    return initial, updated


def trans_run(A, q0: np.ndarray, w: float, Nw: int, dt_grid: float, periods: int = 1, save_mod: int = 100,
              div_val: float = 1e3, con_val: float = 1e-8, removal_est_flag: bool = False,
              real_op: bool = False):
    """SourceCode/TransientRunRK4.c:101-186. Returns a dict with q (last
    snapshot), norms, steps, stop (0 done, 1 NaN, 2 diverged, 3 converged),
    snapshots {pos: q} and estimates [(period, initial, updated)]."""
    dt, Ntp, Rd, rend, n_saved = trans_grid(w, Nw, dt_grid, periods, save_mod)
    A = A.tocsr()
    q = np.array(q0, dtype=np.complex128)
    norms = np.zeros(n_saved)
    norms[0] = np.linalg.norm(q)
    snaps = {0: q.copy()}
    ests = []
    Nw_eff = Nw // 2 if real_op else Nw
    dft = dft_matrix(Nw, Nw_eff, real_op)
    if removal_est_flag:
        Q = np.zeros((q.size, Nw), dtype=np.complex128)
        Q[:, 0] = q
        qss = -q
    stop, steps = 0, 0
    for i in range(1, rend + 1):
        q = rk4_step(A, q, dt)
        steps = i
        if i % save_mod == 0:
            pos = i // save_mod
            nr = np.linalg.norm(q)
            if np.isnan(nr):
                stop = 1
                break
            if nr > div_val:
                stop = 2
                break
            if nr < con_val:
                stop = 3
                break
            snaps[pos] = q.copy()
            norms[pos] = nr
        if removal_est_flag and i % Rd == 0:
            pos = (i // Rd) % Nw
            if pos == 0:
                ini, upd = removal_est(Q, qss, i // Ntp, w, dft)
                ests.append((i // Ntp, ini, upd))
            Q[:, pos] = q
    return dict(q=q, norms=norms, steps=steps, stop=stop, snapshots=snaps, estimates=ests, dt=dt,
                Nt_period=Ntp, rend=rend)


def rk4_amplification(z):
    """P(z) = 1 + z + z^2/2 + z^3/6 + z^4/24: one RK4 step of dy/dt = lambda y."""
    return 1 + z + z * z / 2 + z ** 3 / 6 + z ** 4 / 24
