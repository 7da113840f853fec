"""Benchmark workloads and their algorithmic byte counts.

3D64: the five-field synthetic LNS-like operator on a 64^3 grid
(N = 5*64^3 = 1,310,720; 1,810,432 dense 5x5 complex128 blocks, about
45.26M nonzeros), k = 10 test vectors, Nw = 32 frequencies, q = 1, diagonal
W_q = W_f from cell volumes in [0.5, 1.5]. Choices the configuration leaves
open and that are fixed here: base frequency w0 = 0.1 (T = 2 pi / w0),
domain x in [0, 10) streamwise and y, z in [-5, 5] (jet radius 1), dt from
the RK4 stability limit 2.5 / rho with rho a Gershgorin bound on |lambda|,
two transient periods, and a spectral shift placing the rightmost
eigenvalue at -0.05, estimated from the growth rate of the unforced RK4
propagator (power iteration with the transient-run kernels on the GPU).

GL1: the 500-node Ginzburg-Landau operator, k = 10, Nw = 64, dt = T/4096,
one transient period.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import synth


@dataclass
class Workload:
    name: str
    N: int
    k: int
    Nw: int
    q: int
    w: float
    dt_in: float
    transient_length: float
    transient_removal: bool
    bcsr: tuple | None = None
    csr: object | None = None
    weights: dict = field(default_factory=dict)
    meta: dict = field(default_factory=dict)

    def params(self, **kw):
        from . import default_params
        return default_params(k=self.k, q=self.q, Nw=self.Nw, w=self.w, dt=self.dt_in,
                              TransientLength=self.transient_length,
                              TransientRemoval=int(self.transient_removal), Display=0, **kw)

    def operator_bytes(self, s_c: int = 16) -> int:
        """S_A: bytes of A (or A^H) read once: values + indices."""
        if self.bcsr is not None:
            br, bc, bl = self.bcsr
            nblk, bs = bl.shape[0], bl.shape[1]
            return nblk * bs * bs * s_c + nblk * 4 + (br.size) * 4
        A = self.csr
        return A.nnz * s_c + A.nnz * 4 + (A.shape[0] + 1) * 4

    def step_bytes(self, R: int, s_c: int = 16, forcing_block: int = 0) -> dict:
        """Algorithmic bytes of one forced RK4 step over all k test vectors:
        B_step = 4 S_A + S_F / G + 19 S_v + S_v / R with S_F = N Nw k s_c
        (the forcing coefficients, read once per step for both forcing
        times, or once per block of G steps when the forcing is synthesised
        ahead in blocks; G = 1 otherwise), S_v = N k s_c (one state-sized
        vector pass), 19 vector passes (stage inputs formed from y and the
        previous stage, forcing written once and read by the stages that add
        it), one ring sample every R steps. Per kernel: stage 1 S_A + S_F +
        5 S_v when it synthesises the forcing, else S_A + 3 S_v and the
        forcing-block kernel S_F / G + 2 S_v per step; stage 2 (or 3) S_A +
        4 S_v; stage 4 S_A + 6 S_v + S_v / R."""
        G = max(1, forcing_block)
        S_A = self.operator_bytes(s_c)
        S_F = self.N * self.Nw * self.k * s_c
        S_v = self.N * self.k * s_c
        out = dict(S_A=S_A, S_F=S_F, S_v=S_v, step=4 * S_A + S_F / G + 19 * S_v + S_v / R,
                   stage234=S_A + 4 * S_v, stage4=S_A + 6 * S_v + S_v / R)
        if forcing_block > 0:
            out.update(forcing=S_F / G + 2 * S_v, stage1=S_A + 3 * S_v)
        else:
            out.update(forcing=0.0, stage1=S_A + S_F + 5 * S_v)
        return out

    def step_flops(self, paired: bool = True) -> dict:
        """Arithmetic of one step as executed: 8 flops per complex
        multiply-add (4 FMA) in the sparse products; the forcing synthesis at
        two times per step, with +-f frequency pairs (complex operator, even
        Nw) costing 2 complex and Nw-2 complex-by-real multiply-adds (4 flops)
        per time, otherwise Nw complex multiply-adds."""
        nnz = self.csr.nnz if self.csr is not None else self.bcsr[2].size
        spmm = 8.0 * nnz * self.k
        if paired and self.Nw % 2 == 0:
            per_time = 2 * 8.0 + (self.Nw - 2) * 4.0
        else:
            per_time = 8.0 * self.Nw
        forcing = 2 * self.N * self.k * per_time
        return dict(step=4 * spmm + forcing, stage1=spmm + forcing)


def gershgorin_bound_bcsr(browptr, bcol, blocks) -> float:
    """max_i sum_j |a_ij| over the rows of a block-CSR matrix."""
    nb = browptr.size - 1
    rowsum = np.abs(blocks).sum(axis=2)  # (nblk, bs)
    rows_of_block = np.repeat(np.arange(nb), np.diff(browptr))
    acc = np.zeros((nb, blocks.shape[1]))
    np.add.at(acc, rows_of_block, rowsum)
    return float(acc.max())


def local_shift(browptr, bcol, blocks, target: float = -0.05) -> float:
    """Shift s such that the rightmost eigenvalue over all centre 5x5 blocks
    of A - s I is `target`."""
    nb = browptr.size - 1
    rows_of_block = np.repeat(np.arange(nb), np.diff(browptr))
    center = blocks[bcol == rows_of_block]
    ev = np.linalg.eigvals(center)
    return float(ev.real.max() - target)


def rk4_growth_rate(bcsr, w: float, Nw: int, dt_in: float, seed: int = 5, max_periods: int = 16,
                    tol: float = 2e-4) -> tuple[float, int]:
    """Rightmost eigenvalue of A estimated by power iteration on the unforced
    RK4 propagator (rsvdt_trans_run, one period at a time, the state
    renormalised between periods): the growth rate of the state norm over
    the second half of a period, ln(|q(t1)| / |q(t0)|) / (t1 - t0), until two
    successive periods agree to `tol`. For the slow modes that dominate it,
    ln|R(lambda dt)| / dt equals Re(lambda) to O(dt^4). Returns (rate,
    periods used)."""
    import rsvdt

    br, bc, bl = bcsr
    ctx = rsvdt.Context(rsvdt.default_params(k=1, q=0, Nw=Nw, w=w, dt=dt_in, TransientLength=0.0, Display=0))
    ctx.set_operator_bcsr(br, bc, bl)
    N = (br.size - 1) * bl.shape[1]
    q = synth.complex_normal(N, 1, seed)[:, 0]
    q /= np.linalg.norm(q)
    info = ctx.trans_grid(periods=1, save_mod=1)
    mod = max(1, info.Nt_period // 8)
    rate, prev, used = 0.0, None, 0
    for used in range(1, max_periods + 1):
        q, norms, info, _, _ = ctx.trans_run(q, periods=1, save_mod=mod, div_val=1e300, con_val=0.0)
        h = norms.size // 2
        rate = math.log(norms[-1] / norms[h]) / ((norms.size - 1 - h) * mod * info.dt)
        q = q / np.linalg.norm(q)
        if prev is not None and abs(rate - prev) < tol:
            break
        prev = rate
    ctx.close()
    return rate, used


# Rightmost eigenvalue of the unshifted operator (grid n, seed) measured by
# rk4_growth_rate on a GB300 (converged within 2e-4 after 3 periods at 64^3,
# 6 at 24^3). Recorded so that every run of these operators, on the GPU or
# on the host cores only (the CPU arm of the benchmark, the exact-resolvent
# fixtures), builds the identical shifted operator.
RECORDED_GROWTH_RATE = {(64, 7): 0.22465966906219464, (24, 7): 0.33317440426416783}


def make_3d(n: int = 64, k: int = 10, Nw: int = 32, q: int = 1, seed: int = 7, w: float = 0.1,
            periods: float = 2.0, with_weights: bool = True, shift: str = "recorded",
            target: float = -0.05) -> Workload:
    """shift = "recorded": the rightmost eigenvalue from RECORDED_GROWTH_RATE
    when (n, seed) is listed there, else as "rk4"; "rk4": the rightmost
    eigenvalue from rk4_growth_rate (needs the GPU); "local": from the local
    5x5 centre blocks only (host-only; an underestimate of the spectral
    abscissa)."""
    br, bc, bl = synth.op3d_blocks(n=n, seed=seed, shift=0.0)
    nb = br.size - 1
    rows_of_block = np.repeat(np.arange(nb), np.diff(br))
    cidx = np.nonzero(bc == rows_of_block)[0]
    eye = np.arange(bl.shape[1])
    if shift == "recorded" and (n, seed) in RECORDED_GROWTH_RATE:
        rate = RECORDED_GROWTH_RATE[(n, seed)]
        s = rate - target
        how = f"rk4 growth rate {rate:.6g} (recorded)"
    elif shift in ("rk4", "recorded"):
        rho0 = gershgorin_bound_bcsr(br, bc, bl)
        rate, used = rk4_growth_rate((br, bc, bl), w, Nw, 2.5 / rho0)
        s = rate - target
        how = f"rk4 growth rate {rate:.6g} over {used} period(s)"
    else:
        s = local_shift(br, bc, bl, target)
        how = "local 5x5 centre blocks"
    bl[cidx[:, None], eye[None, :], eye[None, :]] -= s
    rho = gershgorin_bound_bcsr(br, bc, bl)
    dt_in = 2.5 / rho
    T = 2 * math.pi / w
    N = nb * bl.shape[1]
    wl = Workload(name=f"3D{n}", N=N, k=k, Nw=Nw, q=q, w=w, dt_in=dt_in,
                  transient_length=periods * T, transient_removal=False, bcsr=(br, bc, bl),
                  meta=dict(shift=s, shift_method=how, gershgorin=rho, seed=seed, grid=f"{n}^3",
                            blocks=int(bl.shape[0]), nnz=int(bl.size)))
    if with_weights:
        wl.weights = dict(zip(("W_sqrt", "W_sqrt_inv"), synth.diag_weights(N, seed=seed + 4)))
    return wl


def make_gl1(k: int = 10, q: int = 1, transient_removal: bool = False) -> Workload:
    A = synth.gl_operator(500)
    dt, T = synth.gl_time_grid(0.1, 4096)
    return Workload(name="GL1", N=500, k=k, Nw=64, q=q, w=0.1, dt_in=dt, transient_length=T,
                    transient_removal=transient_removal, csr=A)
