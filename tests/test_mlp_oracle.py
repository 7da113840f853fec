"""The learned sketch's CPU network oracle against finite differences (its
backward pass is what the GPU gradients are checked against)."""
import numpy as np

from oracle import mlp_ref


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    widths = [3, 7, 6, 5]
    n = sum(widths[i] * widths[i + 1] + widths[i + 1] for i in range(len(widths) - 1))
    p = rng.standard_normal(n) * 0.5
    X = rng.standard_normal((9, 3))
    T = rng.standard_normal((9, 5))
    _, g = mlp_ref.loss_and_grads(p, widths, X, T, bf16=False, dtype=np.float64)
    h = 1e-6
    fd = np.zeros(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = h
        lp, _ = mlp_ref.loss_and_grads(p + e, widths, X, T, bf16=False, dtype=np.float64)
        lm, _ = mlp_ref.loss_and_grads(p - e, widths, X, T, bf16=False, dtype=np.float64)
        fd[i] = (lp - lm) / (2 * h)
    assert np.abs(g - fd).max() < 1e-7 * max(1.0, np.abs(fd).max())


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    r = mlp_ref.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to the even mantissa 1.
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_pod_basis_snapshot_method_matches_correlation():
    """The learned sketch's POD basis: the method of snapshots (tall mode
    matrices, the 3D family) spans the same leading subspace as the N x N
    correlation eigenvectors."""
    from rsvdt import learned

    rng = np.random.default_rng(3)
    N, m, r = 300, 40, 6
    base = rng.standard_normal((N, r)) + 1j * rng.standard_normal((N, r))
    M = base @ (rng.standard_normal((r, m)) * np.logspace(0, -2, r)[:, None]) + 1e-6 * rng.standard_normal((N, m))
    P1, e1 = learned.pod_basis(M, r)  # snapshots (N > m)
    ev, vec = np.linalg.eigh(M @ M.conj().T)
    P2 = vec[:, ::-1][:, :r]
    assert np.allclose(P1.conj().T @ P1, np.eye(r), atol=1e-10)
    # Same subspace: the projector difference is at rounding level.
    assert np.linalg.norm(P1 @ P1.conj().T - P2 @ P2.conj().T) < 1e-8
    assert abs(e1 - ev[::-1][:r].sum() / ev.sum()) < 1e-12
    Ps, es = learned.pod_basis(M[:30].copy(), 5)  # wide (N <= m) branch
    assert np.allclose(Ps.conj().T @ Ps, np.eye(5), atol=1e-10) and 0 < es <= 1
