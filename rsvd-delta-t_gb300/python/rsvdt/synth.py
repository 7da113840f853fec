"""Seeded synthetic operators and sketches of the benchmark shapes.

No public dataset is involved: these generators build the linearised
Ginzburg-Landau operator (1D, tridiagonal CSR), the 3D five-field block
operator (7-point stencil of dense 5x5 blocks) and i.i.d. standard complex
normal sketches, deterministically from a seed.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def gl_operator(N: int = 500, L: float = 50.0, nu: complex = 2 + 0.2j, gamma: complex = 1 - 1j,
                mu0: float = 0.38, mu2: float = -0.005) -> sp.csr_matrix:
    """A = -nu d/dx + gamma d^2/dx^2 + mu(x), mu(x) = mu0 + mu2 x^2, on N
    interior nodes of [-L, L] with Dirichlet ends; second-order central
    differences (3N-2 nonzeros)."""
    x = np.linspace(-L, L, N + 2)[1:-1]
    h = x[1] - x[0]
    lower = nu / (2 * h) + gamma / h**2
    upper = -nu / (2 * h) + gamma / h**2
    diag = -2 * gamma / h**2 + (mu0 + mu2 * x**2)
    A = sp.diags([np.full(N - 1, lower), diag.astype(complex), np.full(N - 1, upper)], [-1, 0, 1],
                 shape=(N, N), format="csr", dtype=np.complex128)
    A.sort_indices()
    return A


def gl_stretched(N: int, mu0: float, nu: complex = 2 + 0.2j, gamma: complex = 1 - 1j,
                 mu2: float = -0.005) -> sp.csr_matrix:
    """Ginzburg-Landau operator on N nodes with the grid spacing of the
    500-node case: domain [-L, L] with L = 50 (N+1)/501 and the mu profile
    stretched with it, mu(x) = mu0 + mu2 (50 x / L)^2. The largest |lambda|
    stays near 150 for every N, so one time step (T/4096 at w0 = 0.1) suits
    the whole family."""
    L = 50.0 * (N + 1) / 501
    x = np.linspace(-L, L, N + 2)[1:-1]
    h = x[1] - x[0]
    lower = nu / (2 * h) + gamma / h**2
    upper = -nu / (2 * h) + gamma / h**2
    diag = -2 * gamma / h**2 + (mu0 + mu2 * (50 * x / L) ** 2)
    A = sp.diags([np.full(N - 1, lower), diag.astype(complex), np.full(N - 1, upper)], [-1, 0, 1],
                 shape=(N, N), format="csr", dtype=np.complex128)
    A.sort_indices()
    return A


def gl_rightmost(N: int, mu0: float, nu: complex = 2 + 0.2j, gamma: complex = 1 - 1j,
                 mu2: float = -0.005) -> float:
    """Real part of the leading global eigenvalue of gl_stretched's
    operator, lambda_0 = mu0 - nu^2/(4 gamma) - sqrt(-m gamma) with
    m = mu2 (50/L)^2 the profile's curvature (the harmonic-oscillator
    spectrum of the Ginzburg-Landau operator with a quadratic mu). Iterative
    eigensolvers are unreliable here: the operator is strongly non-normal."""
    L = 50.0 * (N + 1) / 501
    m = mu2 * (50.0 / L) ** 2
    lam0 = mu0 - nu**2 / (4 * gamma) - np.sqrt(-m * gamma + 0j)
    return float(lam0.real)


def gl_family(count: int = 48, seed: int = 2024, n_lo: int = 200, n_hi: int = 20000,
              ks=(6, 10, 16), nws=(16, 32, 64), margin: float = 0.05):
    """The batching family: `count` Ginzburg-Landau problems with N
    log-uniform in [n_lo, n_hi], mu0 uniform in [0.2, 0.45], k and Nw drawn
    from `ks` and `nws`. A problem whose rightmost eigenvalue is above
    -margin gets the reference's discounting A <- A - beta I with beta
    placing it at -margin (SourceCode/LNSStructure.c:53-56)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        N = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        mu0 = float(rng.uniform(0.2, 0.45))
        k = int(rng.choice(ks))
        nw = int(rng.choice(nws))
        A = gl_stretched(N, mu0)
        lr = gl_rightmost(N, mu0)
        beta = max(0.0, lr + margin)
        out.append(dict(N=N, mu0=mu0, k=k, Nw=nw, A=A, beta=beta, rightmost=lr))
    return out


def complex_normal(rows: int, cols: int, seed: int) -> np.ndarray:
    """i.i.d. CN(0,1) = (a + ib)/sqrt(2), a, b ~ N(0,1) from
    numpy.random.default_rng(seed); Fortran order."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((rows, cols))
    b = rng.standard_normal((rows, cols))
    return np.asfortranarray((a + 1j * b) / np.sqrt(2.0))


def gl_sketch(N: int, k: int, Nw: int, seed: int = 14) -> np.ndarray:
    """Sketch F_hat: N x (k*Nw), frequency-major columns (iw*k + ik)."""
    return complex_normal(N, k * Nw, seed)


def gl_time_grid(w: float = 0.1, Ns: int = 4096):
    """dt requested a hair above T/Ns so that SetupTimeFreqGrid's ceil
    reproduces exactly Ns steps per period."""
    T = 2 * np.pi / w
    return T / Ns * (1 + 1e-12), T


# --------------------------------------------------------------------- 3D

def op3d_blocks(n: int = 64, Re: float = 1000.0, Lx: float = 10.0, Lr: float = 5.0, seed: int = 7,
                coupling: float = 0.1, shift: float | None = None, bs: int = 5):
    """Five-field synthetic LNS-like operator on an n^3 grid.

    Grid: x in [0, Lx) streamwise (upwind direction), y, z in [-Lr, Lr];
    jet U(r) = 0.5 (1 - tanh(4 (r - 1))), r = sqrt(y^2 + z^2). Each grid
    point has a 7-point stencil of bs x bs blocks: first-order upwind
    advection -U d/dx, diffusion (1/Re) Laplacian (Dirichlet walls), and a
    dense seeded coupling block with entries coupling*CN(0,1) added to the
    centre block. Every stored block is dense (explicit zeros kept), as the
    benchmark's block-CSR format specifies. The diagonal is shifted by
    -shift (computed by the caller to place the rightmost eigenvalue).

    Returns (browptr, bcol, blocks) with blocks of shape (nblocks, bs, bs).
    """
    rng = np.random.default_rng(seed)
    h = Lx / n
    hr = 2 * Lr / n
    ix = np.arange(n)
    yr = -Lr + (np.arange(n) + 0.5) * hr
    Y, Z = np.meshgrid(yr, yr, indexing="ij")
    r = np.sqrt(Y**2 + Z**2)
    U = 0.5 * (1 - np.tanh(4 * (r - 1)))  # (n, n) over (y, z)
    nb = n**3
    # Index (i, j, l) -> i*n*n + j*n + l, i streamwise.
    I, J, Lz = np.meshgrid(ix, ix, ix, indexing="ij")
    I = I.ravel()
    J = J.ravel()
    Lz = Lz.ravel()
    Ub = U[J, Lz]
    nu = 1.0 / Re
    center = -Ub / h - nu * (2 / h**2 + 4 / hr**2)
    if shift is not None:
        center = center - shift
    # Neighbours: (di, dj, dl, coefficient).
    nbrs = [
        (-1, 0, 0, Ub / h + nu / h**2),  # upwind (U >= 0) + diffusion
        (1, 0, 0, np.full(nb, nu / h**2)),
        (0, -1, 0, np.full(nb, nu / hr**2)),
        (0, 1, 0, np.full(nb, nu / hr**2)),
        (0, 0, -1, np.full(nb, nu / hr**2)),
        (0, 0, 1, np.full(nb, nu / hr**2)),
    ]
    cols = [np.arange(nb)]
    coefs = [center]
    valid = [np.ones(nb, bool)]
    for di, dj, dl, c in nbrs:
        ii, jj, ll = I + di, J + dj, Lz + dl
        ok = (ii >= 0) & (ii < n) & (jj >= 0) & (jj < n) & (ll >= 0) & (ll < n)
        cols.append(np.where(ok, ii * n * n + jj * n + ll, -1))
        coefs.append(c)
        valid.append(ok)
    cols = np.stack(cols, 1)  # (nb, 7)
    coefs = np.stack(coefs, 1)
    valid = np.stack(valid, 1)
    # Sort each block row's stored blocks by column.
    key = np.where(valid, cols, np.iinfo(np.int64).max)
    order = np.argsort(key, axis=1, kind="stable")
    cols = np.take_along_axis(cols, order, 1)
    coefs = np.take_along_axis(coefs, order, 1)
    valid = np.take_along_axis(valid, order, 1)
    counts = valid.sum(1)
    browptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    bcol = cols[valid].astype(np.int64)
    coef = coefs[valid]
    nblocks = bcol.size
    blocks = np.zeros((nblocks, bs, bs), dtype=np.complex128)
    eye = np.arange(bs)
    blocks[:, eye, eye] = coef[:, None]
    # Coupling on the centre (diagonal) blocks.
    rows_of_block = np.repeat(np.arange(nb), counts)
    is_center = bcol == rows_of_block
    cpl = coupling * (rng.standard_normal((nb, bs, bs)) + 1j * rng.standard_normal((nb, bs, bs))) / np.sqrt(2)
    blocks[is_center] += cpl
    return browptr, bcol, blocks


def bcsr_to_csr(browptr, bcol, blocks) -> sp.csr_matrix:
    nb = browptr.size - 1
    bs = blocks.shape[1]
    return sp.bsr_matrix((blocks, bcol, browptr), shape=(nb * bs, nb * bs)).tocsr()


def diag_weights(N: int, seed: int = 11, lo: float = 0.5, hi: float = 1.5):
    """Cell-volume weights vol ~ U[lo, hi]: returns (W^{1/2}, W^{-1/2}) as
    diagonal sparse matrices."""
    vol = np.random.default_rng(seed).uniform(lo, hi, N)
    return (sp.diags(np.sqrt(vol).astype(np.complex128), format="csr"),
            sp.diags((1 / np.sqrt(vol)).astype(np.complex128), format="csr"))
