"""Learned sketch: a network trained on the method's own forcing modes
predicts the warm-start test matrix of a new problem, replacing the random
sketch (SourceCode/CreateRandomMat.c:33-39) so that fewer power iterations
are needed.

Pipeline (everything heavy runs on the GPU through the C ABI):
  1. the method itself (batched RSVD-Delta-t) computes the top-k forcing
     modes V(p, w) at seeded training points p of a problem family;
  2. a POD basis Phi (N x r) of all those modes (one basis per frequency
     for the 3D family, by the method of snapshots);
  3. each mode block projected on Phi, C = Phi^H V (r x k), column phases
     fixed (largest coefficient real and positive), real and imaginary parts
     standardised;
  4. the network (3 -> hidden^depth GELU -> 2 r k; bf16 weights, FP32
     accumulation; rsvdt_mlp_*) is trained with Adam on inputs
     (p_1, p_2, w) scaled to [-1, 1];
  5. for a new problem the sketch's frequency block iw is Phi C_pred(p, w_iw).
The fallback is the random sketch: after a learned run, one FP64 direct
action on the computed forcing modes checks the gains (| |R v_j| - s_j | /
s_j for the leading modes); above the threshold the problem is re-solved
from a random sketch with one power iteration.

Problem families: Ginzburg-Landau operators with the grid spacing of the
500-node case (synth.gl_stretched), parameters mu0 in [0.2, 0.45] and the
advection speed U = Re(nu) in [1.5, 2.5], discounted where unstable
(Family); and the five-field 3D operator at 48^3 (synth.op3d_blocks) over
the Reynolds number Re in [500, 2000] and a uniform reaction term mu0 in
[0.2, 0.45] added to the diagonal, as mu0 enters the Ginzburg-Landau
operator (Family3D). Each family supplies its points, its network inputs
(three values in [-1, 1]) and a context with its operator.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import synth


@dataclass
class Family:
    N: int = 2000
    k: int = 10
    Nw: int = 16
    w0: float = 0.1
    mu0: tuple = (0.2, 0.45)
    U: tuple = (1.5, 2.5)
    # Discounting places the leading eigenvalue at -margin (or lower): with
    # one transient period the transient left is exp(-margin T) = 3.5e-6.
    margin: float = 0.2

    @property
    def T(self):
        return 2 * np.pi / self.w0

    @property
    def dt(self):
        return self.T / 4096 * (1 + 1e-12)

    def omegas(self):
        return np.array([(i if i <= self.Nw // 2 - 1 else i - self.Nw) * self.w0 for i in range(self.Nw)])

    def points(self, count: int, seed: int):
        rng = np.random.default_rng(seed)
        return [(float(rng.uniform(*self.mu0)), float(rng.uniform(*self.U))) for _ in range(count)]

    def operator(self, pt):
        mu0, U = pt
        nu = U + 0.2j
        A = synth.gl_stretched(self.N, mu0, nu=nu)
        beta = max(0.0, synth.gl_rightmost(self.N, mu0, nu=nu) + self.margin)
        return A, beta

    def params(self, rsvdt, q: int, beta: float, precision: int):
        return rsvdt.default_params(k=self.k, q=q, Nw=self.Nw, w=self.w0, dt=self.dt, TransientLength=self.T,
                                    DiscFlg=int(beta > 0), beta=beta, precision=precision, Display=0)

    batched = True

    def inputs(self, pts) -> np.ndarray:
        """(mu0, U, w) scaled to [-1, 1], one row per (point, frequency)."""
        om = self.omegas()
        rows = []
        for mu0, U in pts:
            for w in om:
                rows.append([2 * (mu0 - self.mu0[0]) / (self.mu0[1] - self.mu0[0]) - 1,
                             2 * (U - self.U[0]) / (self.U[1] - self.U[0]) - 1,
                             w / (self.w0 * self.Nw / 2)])
        return np.asarray(rows, dtype=np.float32)

    def context(self, rsvdt, pt, q: int, precision: int):
        A, beta = self.operator(pt)
        ctx = rsvdt.Context(self.params(rsvdt, q, beta, precision))
        ctx.set_operator(A)
        return ctx


@dataclass
class Family3D:
    """The 3D five-field operator at n^3 (N = 5 n^3) over Re and a uniform
    reaction term mu0: A(Re, mu0) = stencil(Re) + coupling + (mu0 - s) I,
    with s fixed for the family so that the least stable corner (Re = 2000,
    mu0 = 0.45) has its rightmost eigenvalue at `target` (estimated with the
    unforced RK4 propagator, workloads.rk4_growth_rate); every other member
    is more damped. One time grid for the family: dt from the Gershgorin
    bound of the stiffest member (Re = 500)."""
    n: int = 48
    k: int = 4
    Nw: int = 16
    w0: float = 0.1
    Re: tuple = (500.0, 2000.0)
    mu0: tuple = (0.2, 0.45)
    seed: int = 7
    target: float = -0.05
    periods: float = 2.0

    batched = False
    pod_per_frequency = True

    def __post_init__(self):
        self._shift = None
        self._dt = None

    @property
    def N(self):
        return 5 * self.n ** 3

    @property
    def T(self):
        return 2 * np.pi / self.w0

    def _setup(self):
        if self._shift is not None:
            return
        from . import workloads

        br, bc, bl = synth.op3d_blocks(n=self.n, Re=self.Re[0], seed=self.seed, shift=-self.mu0[0])
        rho = workloads.gershgorin_bound_bcsr(br, bc, bl)
        dt = 2.5 / (rho + 1.0)  # room for the family's shift
        corner = synth.op3d_blocks(n=self.n, Re=self.Re[1], seed=self.seed, shift=-self.mu0[1])
        rate, _ = workloads.rk4_growth_rate(corner, self.w0, self.Nw, dt)
        self._shift = rate - self.target
        self._dt = dt

    @property
    def dt(self):
        self._setup()
        return self._dt

    @property
    def shift(self):
        self._setup()
        return self._shift

    def omegas(self):
        return np.array([(i if i <= self.Nw // 2 - 1 else i - self.Nw) * self.w0 for i in range(self.Nw)])

    def points(self, count: int, seed: int):
        rng = np.random.default_rng(seed)
        return [(float(rng.uniform(*self.Re)), float(rng.uniform(*self.mu0))) for _ in range(count)]

    def operator(self, pt):
        Re, mu0 = pt
        return synth.op3d_blocks(n=self.n, Re=Re, seed=self.seed, shift=self.shift - mu0), 0.0

    def params(self, rsvdt, q: int, beta: float, precision: int):
        return rsvdt.default_params(k=self.k, q=q, Nw=self.Nw, w=self.w0, dt=self.dt,
                                    TransientLength=self.periods * self.T, precision=precision, Display=0)

    def inputs(self, pts) -> np.ndarray:
        """(Re, mu0, w) scaled to [-1, 1] (Re on a log scale)."""
        om = self.omegas()
        lo, hi = np.log(self.Re[0]), np.log(self.Re[1])
        rows = []
        for Re, mu0 in pts:
            for w in om:
                rows.append([2 * (np.log(Re) - lo) / (hi - lo) - 1,
                             2 * (mu0 - self.mu0[0]) / (self.mu0[1] - self.mu0[0]) - 1,
                             w / (self.w0 * self.Nw / 2)])
        return np.asarray(rows, dtype=np.float32)

    def context(self, rsvdt, pt, q: int, precision: int):
        bcsr, _ = self.operator(pt)
        ctx = rsvdt.Context(self.params(rsvdt, q, 0.0, precision))
        ctx.set_operator_bcsr(*bcsr)
        return ctx


def solve_batch(fam, pts, q: int, precision: int, sketches=None, seed: int = 0):
    """RSVD-Delta-t for every point (one batch for a batched family, one
    context after another otherwise); returns ([(U, V, S)], seconds of the
    solves). Random sketches (seeded, CN(0,1)) unless `sketches` are given."""
    import rsvdt

    def sketch(i):
        return sketches[i] if sketches is not None else synth.complex_normal(fam.N, fam.k * fam.Nw, seed + i)

    if fam.batched:
        b = rsvdt.Batch(precision)
        for pt in pts:
            A, beta = fam.operator(pt)
            b.add(fam.params(rsvdt, q, beta, precision), A)
        for i in range(len(pts)):
            b.set_sketch(i, sketch(i))
        t0 = time.perf_counter()
        b.run()
        out = [b.get_results(i) for i in range(len(pts))]
        dt = time.perf_counter() - t0
        b.close()
        return out, dt
    out, dt = [], 0.0
    for i, pt in enumerate(pts):
        ctx = fam.context(rsvdt, pt, q, precision)
        ctx.set_sketch(sketch(i))
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.run()
        out.append(ctx.get_results())
        dt += time.perf_counter() - t0
        ctx.close()
    return out, dt


def _phase_fix(C: np.ndarray) -> np.ndarray:
    """Rotates each column so that its largest coefficient is real positive."""
    idx = np.argmax(np.abs(C), axis=0)
    ph = C[idx, np.arange(C.shape[1])]
    return C * (np.abs(ph) / np.where(ph == 0, 1, ph))[None, :]


def pod_basis(M: np.ndarray, r: int):
    """Leading r left singular vectors of M (N x m) and the fraction of
    |M|_F^2 they hold: from the N x N correlation when N <= m, otherwise by
    the method of snapshots (Phi = M W Lambda^{-1/2} from M^H M = W Lambda W^H),
    whose cost does not grow with N^2."""
    if M.shape[0] <= M.shape[1]:
        ev, vec = np.linalg.eigh(M @ M.conj().T)
        ev = ev[::-1]
        Phi = np.ascontiguousarray(vec[:, ::-1][:, :r])
    else:
        ev, W = np.linalg.eigh(M.conj().T @ M)
        ev, W = ev[::-1], W[:, ::-1]
        Phi = np.ascontiguousarray((M @ W[:, :r]) / np.sqrt(np.maximum(ev[:r], 1e-300)))
    return Phi, float(ev[:r].sum() / ev.sum())


class LearnedSketch:
    def __init__(self, fam: Family, r: int = 64, hidden: int = 256, depth: int = 4, seed: int = 0):
        self.fam = fam
        self.r = r
        self.widths = [3] + [hidden] * depth + [2 * r * fam.k]
        self.seed = seed
        self.net = None
        self.Phi = None
        self.per_frequency = False

    def _inputs(self, pts):
        return self.fam.inputs(pts)

    def _basis(self, iw):
        return self.Phi[iw] if self.per_frequency else self.Phi

    def fit(self, pts, modes, steps: int = 3000, batch: int = 256, lr: float = 1e-3):
        """modes: list of V (N x k*Nw, frequency-major) at the points. One
        POD basis for all frequencies, or one per frequency when the family
        asks for it (3D modes differ too much between frequencies for one
        r = 64 basis)."""
        import rsvdt

        f = self.fam
        self.per_frequency = bool(getattr(f, "pod_per_frequency", False))
        if self.per_frequency:
            self.Phi, energies = [], []
            for iw in range(f.Nw):
                Mw = np.concatenate([V[:, iw * f.k:(iw + 1) * f.k] for V in modes], axis=1)
                P, e = pod_basis(Mw, min(self.r, Mw.shape[1]))
                if P.shape[1] < self.r:  # fewer modes than r: pad with zero columns
                    P = np.concatenate([P, np.zeros((P.shape[0], self.r - P.shape[1]), P.dtype)], axis=1)
                self.Phi.append(P)
                energies.append(e)
            self.pod_energy = float(np.mean(energies))
        else:
            M = np.concatenate([V for V in modes], axis=1)  # N x (points * k * Nw)
            self.Phi, self.pod_energy = pod_basis(M, self.r)
        T = []
        for V in modes:
            for iw in range(f.Nw):
                C = _phase_fix(self._basis(iw).conj().T @ V[:, iw * f.k:(iw + 1) * f.k])
                T.append(np.concatenate([C.real.ravel(), C.imag.ravel()]))
        T = np.asarray(T, dtype=np.float64)
        self.t_mean = T.mean(axis=0)
        self.t_std = T.std(axis=0) + 1e-12
        Tn = ((T - self.t_mean) / self.t_std).astype(np.float32)
        X = self._inputs(pts)
        self.net = rsvdt.Mlp(self.widths, seed=self.seed)
        t0 = time.perf_counter()
        self.final_loss = self.net.train(X, Tn, batch=batch, steps=steps, lr=lr, seed=self.seed)
        self.train_seconds = time.perf_counter() - t0
        return self.final_loss

    def sketch(self, pt) -> np.ndarray:
        f = self.fam
        Y = self.net.forward(self._inputs([pt])).astype(np.float64) * self.t_std + self.t_mean
        F = np.zeros((f.N, f.k * f.Nw), dtype=np.complex128, order="F")
        rk = self.r * f.k
        for iw in range(f.Nw):
            C = (Y[iw, :rk] + 1j * Y[iw, rk:]).reshape(self.r, f.k)
            F[:, iw * f.k:(iw + 1) * f.k] = self._basis(iw) @ C
        return F


def gain_check(fam: Family, pt, result, jmax: int = 3):
    """max over frequencies and j < jmax of | |R v_j| - s_j | / s_j, with R v
    from one complex128 direct action on the computed forcing modes."""
    import rsvdt

    U, V, S = result
    ctx = fam.context(rsvdt, pt, 0, rsvdt.PREC_C128)
    ctx.set_sketch(V)
    ctx.action(rsvdt.DIRECT)
    Y = ctx.get_block()
    ctx.close()
    k = fam.k
    worst = 0.0
    for iw in range(fam.Nw):
        for j in range(min(jmax, k)):
            s = S[j, iw]
            worst = max(worst, abs(np.linalg.norm(Y[:, iw * k + j]) - s) / s)
    return worst


def gain_errors(results, refs, jmax: int = 3):
    """Per problem: max over frequencies of the relative error of s_1, and of
    s_j for j < jmax."""
    e1, ej = [], []
    for (_, _, S), (_, _, Sr) in zip(results, refs):
        e1.append(float((np.abs(S[0] - Sr[0]) / Sr[0]).max()))
        ej.append(float((np.abs(S[:jmax] - Sr[:jmax]) / Sr[:jmax]).max()))
    return np.asarray(e1), np.asarray(ej)
