"""Oracle for the RSVD-Delta-t time-stepping path (TEST INFRASTRUCTURE).

Only tests, the smoke check and the benchmark's CPU-baseline leg import
this package, as the checker. It holds:
  - a ctypes binding of the C restatement of the reference algorithm
    (rsvdt_oracle.c, built into oracle/_build/liboracle.so);
  - the dense FP64 resolvent oracle: SVD of W_q^{1/2} C (i w I - A)^{-1} B
    W_f^{-1/2} per frequency, for problems small enough to invert.

Parity status: the reference needs PETSc 3.19 + SLEPc 3.19 + MPI, none of
which exist here or on the GPU machine, so the reference itself cannot be run.
The restatement is pinned instead to the reference's own known answer, the
Ginzburg-Landau tutorial (Tutorial/Ginzburg-Landau/A_GL with the parameters
of variables.yaml:16-39 and the gains of gains.png), through the fixtures
and script in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
SRC = os.path.join(HERE, "rsvdt_oracle.c")


def build(force: bool = False) -> str:
    """gcc -O2 -fopenmp -ffp-contract=off rsvdt_oracle.c -> _build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "rsvdt_oracle.h"))):
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               SRC, "-o", LIB, "-lm"]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + res.stdout)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        d = P(C.c_double)
        i64 = C.c_int64
        L.orc_setup_grid.argtypes = [C.c_double, i64, C.c_double, C.c_double, d, P(i64)]
        L.orc_build_idft.argtypes = [i64, i64, C.c_int, d]
        L.orc_build_dft.argtypes = [i64, i64, C.c_int, d]
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [i64, P(i64), P(i64), d, i64, C.c_double, C.c_double, i64, i64, i64,
                                 C.c_int, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_row_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_weight.argtypes = [C.c_void_p, C.c_int, i64, i64, P(i64), P(i64), d]
        L.orc_ts_action.argtypes = [C.c_void_p, C.c_int, i64, d, d]
        L.orc_action.argtypes = [C.c_void_p, C.c_int, i64, d, d]
        L.orc_rk4_steps.argtypes = [C.c_void_p, C.c_int, d, i64, i64, d, d]
        L.orc_qr_all_freqs.argtypes = [i64, i64, i64, d]
        L.orc_svd_all_freqs.argtypes = [i64, i64, i64, d, d, d]
        L.orc_run.argtypes = [C.c_void_p, i64, i64, d, d, d, d]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def setup_grid(w: float, Nw: int, dt: float, transient_length: float):
    """(dt, Ns, Nt, ResRatio) of SourceCode/SetupTimeFreqGrid.c:16-21."""
    out_dt = np.zeros(1)
    ints = np.zeros(3, dtype=np.int64)
    lib().orc_setup_grid(w, Nw, dt, transient_length, _d(out_dt), _i(ints))
    return float(out_dt[0]), int(ints[0]), int(ints[1]), int(ints[2])


class Oracle:
    """CPU restatement of one resolvent problem (same entry points as the
    CUDA library's Context)."""

    def __init__(self, A, Nw: int, w: float, dt: float, transient_length: float,
                 transient_removal: bool = False, real_op: bool | None = None, threads: int = 0):
        A = A.tocsr()
        A.sort_indices()
        self.N = A.shape[0]
        if real_op is None:
            real_op = bool(np.linalg.norm(A.data.imag) < 1e-12)
        self.real_op = real_op
        self.Nw = Nw
        self.Nw_eff = Nw // 2 if real_op else Nw
        self.w = w
        self.dt, self.Ns, self.Nt, self.R = setup_grid(w, Nw, dt, transient_length)
        rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
        ci = np.ascontiguousarray(A.indices, dtype=np.int64)
        va = np.ascontiguousarray(A.data, dtype=np.complex128)
        self._h = lib().orc_create(self.N, _i(rp), _i(ci), _d(va.view(np.float64)), Nw, w, self.dt,
                                   self.Ns, self.Nt, self.R, int(transient_removal), int(real_op))
        if not self._h:
            raise RuntimeError("oracle create failed")
        self.Nb = self.N
        self.Nc = self.N
        if threads:
            lib().orc_set_threads(self._h, threads)

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int):
        lib().orc_set_threads(self._h, n)

    def set_row_threads(self, n: int):
        """Threads for the row loops of each RK4 step (results unchanged)."""
        lib().orc_set_row_threads(self._h, n)

    def set_weight(self, which: int, M):
        M = M.tocsr()
        M.sort_indices()
        rp = np.ascontiguousarray(M.indptr, dtype=np.int64)
        ci = np.ascontiguousarray(M.indices, dtype=np.int64)
        va = np.ascontiguousarray(M.data, dtype=np.complex128)
        rc = lib().orc_set_weight(self._h, which, M.shape[0], M.shape[1], _i(rp), _i(ci),
                                  _d(va.view(np.float64)))
        if rc:
            raise RuntimeError("oracle set_weight failed")
        if which == 1:
            self.Nb = M.shape[1]
        if which == 2:
            self.Nc = M.shape[0]

    def ts_action(self, direction: int, F: np.ndarray) -> np.ndarray:
        F = np.asfortranarray(F, dtype=np.complex128)
        k = F.shape[1] // self.Nw_eff
        Y = np.zeros((self.N, F.shape[1]), dtype=np.complex128, order="F")
        if lib().orc_ts_action(self._h, direction, k, _d(F), _d(Y)):
            raise RuntimeError("oracle action failed")
        return Y

    def action(self, direction: int, Y: np.ndarray) -> np.ndarray:
        Y = np.asfortranarray(Y, dtype=np.complex128)
        k = Y.shape[1] // self.Nw_eff
        rows_out = self.Nc if direction else self.Nb
        out = np.zeros((rows_out, Y.shape[1]), dtype=np.complex128, order="F")
        if lib().orc_action(self._h, direction, k, _d(Y), _d(out)):
            raise RuntimeError("oracle action failed")
        return out

    def rk4_steps(self, direction: int, Fk: np.ndarray, i0: int, nsteps: int, y: np.ndarray,
                  F3: np.ndarray):
        Fk = np.asfortranarray(Fk, dtype=np.complex128)
        y = np.array(y, dtype=np.complex128)
        F3 = np.array(F3, dtype=np.complex128)
        lib().orc_rk4_steps(self._h, direction, _d(Fk), i0, nsteps, _d(y), _d(F3))
        return y, F3

    def run(self, F: np.ndarray, q: int):
        F = np.asfortranarray(F, dtype=np.complex128)
        k = F.shape[1] // self.Nw_eff
        U = np.zeros((self.Nc, F.shape[1]), dtype=np.complex128, order="F")
        V = np.zeros((self.Nb, F.shape[1]), dtype=np.complex128, order="F")
        S = np.zeros((k, self.Nw_eff), order="F")
        if lib().orc_run(self._h, k, q, _d(F), _d(U), _d(V), _d(S)):
            raise RuntimeError("oracle run failed")
        return U, V, S


def qr_all_freqs(Y: np.ndarray, k: int) -> np.ndarray:
    Y = np.array(Y, dtype=np.complex128, order="F")
    lib().orc_qr_all_freqs(Y.shape[0], k, Y.shape[1] // k, _d(Y))
    return Y


def svd_all_freqs(Y: np.ndarray, k: int):
    Y = np.asfortranarray(Y, dtype=np.complex128)
    nw = Y.shape[1] // k
    U = np.zeros_like(Y, order="F")
    S = np.zeros((k, nw), order="F")
    lib().orc_svd_all_freqs(Y.shape[0], k, nw, _d(Y), _d(U), _d(S))
    return U, S


def freq_of(iw: int, Nw: int, w: float, real_op: bool = False) -> float:
    """Angular frequency of column block iw: iw*w up to Nw/2 - 1 (even Nw)
    or (Nw - 1)/2 (odd Nw), (iw - Nw)*w above (the ordering of
    SourceCode/CreateDFTiDFTMats.c:46-52); iw*w for a real operator."""
    half = Nw // 2 - 1 if Nw % 2 == 0 else (Nw - 1) // 2
    if real_op or iw <= half:
        return iw * w
    return (iw - Nw) * w


def rk4_tone_response(lam, om: float, dt: float):
    """Steady-state answer H of forced RK4 (SourceCode/TSRK4.c:18-47: the
    forcing at t, t + dt/2 twice and t + dt) on y' = lam y + e^{i om t}:
    y_n = H e^{i om n dt} with H = dt G / (e^{i om dt} - P(lam dt)), P the
    RK4 amplification polynomial and G the stages' forcing sum. For a
    diagonal operator the direct action is e^{i om (Nt + R) dt} H F
    exactly, once the transient has decayed."""
    z = np.asarray(lam) * dt
    a, b = np.exp(0.5j * om * dt), np.exp(1j * om * dt)
    P = 1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24
    k2 = z / 2 + a
    k3 = z / 2 * k2 + a
    k4 = z * k3 + b
    return dt * (1 + 2 * k2 + 2 * k3 + k4) / 6 / (b - P)


def dense_resolvent_svd(A, omegas, k: int, Wq=None, Wf_inv=None, B=None, Cm=None):
    """Dense FP64 oracle: SVD of W_q^{1/2} C (i w I - A)^{-1} B W_f^{-1/2} for
    each w; returns (S [k, len(omegas)], U list, V list)."""
    Ad = A.toarray() if hasattr(A, "toarray") else np.asarray(A)
    N = Ad.shape[0]
    S = np.zeros((k, len(omegas)))
    Us, Vs = [], []
    for j, om in enumerate(omegas):
        Rm = np.linalg.solve(1j * om * np.eye(N) - Ad, np.eye(N) if B is None else B.toarray())
        if Cm is not None:
            Rm = Cm.toarray() @ Rm
        if Wq is not None:
            Rm = Wq.toarray() @ Rm
        if Wf_inv is not None:
            Rm = Rm @ Wf_inv.toarray()
        u, s, vh = np.linalg.svd(Rm)
        S[:, j] = s[:k]
        Us.append(u[:, :k])
        Vs.append(vh.conj().T[:, :k])
    return S, Us, Vs


def _sparse_resolvent_one(task):
    """One frequency of sparse_resolvent_svd (a module-level function so a
    spawned worker can import it)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    A, om, k, wq, wfi, tol, seed = task
    N = A.shape[0]
    lu = spla.splu((1j * om * sp.eye(N, format="csc") - A).tocsc(), permc_spec="MMD_AT_PLUS_A")
    op = spla.LinearOperator(
        (N, N), dtype=np.complex128,
        matvec=lambda x: wq * lu.solve(wfi * x.ravel()),
        rmatvec=lambda x: np.conj(wfi) * lu.solve(np.conj(wq) * x.ravel(), trans="H"))
    rng = np.random.default_rng(seed)
    v0 = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    u, s, vh = spla.svds(op, k=k, tol=tol, v0=v0 / np.linalg.norm(v0))
    o = np.argsort(-s)
    return s[o], u[:, o], vh[o].conj().T


def sparse_resolvent_svd(A, omegas, k: int, wq=None, wf_inv=None, tol: float = 1e-10, procs: int = 1,
                         seed: int = 3):
    """Exact-resolvent oracle for N too large to invert densely: for each w,
    a sparse LU of (i w I - A) (SuperLU, minimum degree on A^T + A) and
    Lanczos (ARPACK, scipy svds) on M = diag(wq) (i w I - A)^{-1} diag(wf_inv)
    for the k leading singular triplets, M and M^H applied through the LU
    factors. wq, wf_inv: diagonals of W_q^{1/2} and W_f^{-1/2} (None = I).
    procs > 1 runs the frequencies in a spawned process pool. Returns
    (S [k, len(omegas)], U list, V list) in the weighted coordinates, like
    dense_resolvent_svd."""
    import multiprocessing

    A = A.tocsc()
    N = A.shape[0]
    wq = np.ones(N) if wq is None else np.asarray(wq)
    wf_inv = np.ones(N) if wf_inv is None else np.asarray(wf_inv)
    tasks = [(A, float(om), k, wq, wf_inv, tol, seed + j) for j, om in enumerate(omegas)]
    if procs > 1:
        # Each worker's BLAS (used by SuperLU's supernodes) gets its share of
        # the cores: oversubscribed spinning BLAS threads are many times slower.
        procs = min(procs, len(tasks))
        keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {key: os.environ.get(key) for key in keys}
        for key in keys:
            os.environ[key] = str(max(1, (os.cpu_count() or 1) // procs))
        try:
            with multiprocessing.get_context("spawn").Pool(procs) as pool:
                res = pool.map(_sparse_resolvent_one, tasks)
        finally:
            for key, v in saved.items():
                if v is None:
                    os.environ.pop(key, None)
                else:
                    os.environ[key] = v
    else:
        res = [_sparse_resolvent_one(t) for t in tasks]
    S = np.stack([r[0] for r in res], axis=1)
    return S, [r[1] for r in res], [r[2] for r in res]
