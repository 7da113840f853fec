"""Capacity mode (rsvdt_set_capacity_mode): actions by chunks of test
vectors written in place, in-place weights and SVDs, U in host memory. It
performs the resident mode's arithmetic element by element (each test
vector's stepping, DFT, transient removal and weight products are the
same operations in the same order; the QR and SVD see the same block), so
results must agree to rounding: 1e-12 relative. With complex64 storage of U
the returned U is the resident U rounded to complex64."""
import numpy as np
import pytest
import scipy.sparse as sp

from rsvdt import synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def gl_problem():
    A = synth.gl_operator(64, mu0=0.2)
    return A, dict(w=0.1, Nw=16, dt=0.15, TransientLength=2 * np.pi / 0.1)


def ctx_for(cfg, k, q, tr, prec=0, capacity=None, A=None, bcsr=None, weights=(), lanes=0):
    import rsvdt
    p = rsvdt.default_params(k=k, q=q, Nw=cfg["Nw"], w=cfg["w"], dt=cfg["dt"], TransientLength=cfg["TransientLength"],
                             TransientRemoval=int(tr), precision=prec, Display=0)
    ctx = rsvdt.Context(p)
    ctx.set_lanes_per_row(lanes)
    if capacity is not None:
        ctx.set_capacity_mode(*capacity)
    if bcsr is not None:
        ctx.set_operator_bcsr(*bcsr)
    else:
        ctx.set_operator(A)
    for which, M in weights:
        ctx.set_weight(which, M)
    return ctx


def solve(cfg, F, k, q, tr, **kw):
    ctx = ctx_for(cfg, k, q, tr, **kw)
    ctx.set_sketch(F)
    ctx.run()
    out = ctx.get_results()
    kc = ctx.capacity_chunk()
    cols = [0, k * ctx.grid().Nw_eff - 1, k + 1]
    sel = ctx.get_result_cols(cols)
    ctx.close()
    return out, kc, sel, cols


@pytest.mark.parametrize("kc,tr", [(2, True), (1, False), (0, True)])
def test_chunked_equals_resident(built_lib, kc, tr):
    A, cfg = gl_problem()
    k = 4
    F = synth.complex_normal(64, k * 16, 21)
    (U0, V0, S0), _, _, _ = solve(cfg, F, k, 1, tr, A=A)
    (U1, V1, S1), used, (Us, Vs), cols = solve(cfg, F, k, 1, tr, A=A, capacity=(kc, False))
    assert used == (kc if kc else k)
    assert np.abs(S1 - S0).max() <= 1e-12 * S0.max()
    assert rel(U1, U0) < 1e-12 and rel(V1, V0) < 1e-12
    assert np.array_equal(Us, U1[:, cols]) and np.array_equal(Vs, V1[:, cols])


def test_chunked_weights_and_complex64_u(built_lib):
    """Rectangular B (N x Nb) and C (Nc x N), diagonal weights; U kept in
    complex64 on the host."""
    import rsvdt
    A, cfg = gl_problem()
    N, Nb, Nc, k = 64, 40, 30, 4
    rng = np.random.default_rng(3)
    Bm = sp.random(N, Nb, density=0.1, random_state=1, dtype=np.float64).astype(np.complex128) + \
        sp.eye(N, Nb, dtype=np.complex128)
    Cm = sp.random(Nc, N, density=0.1, random_state=2, dtype=np.float64).astype(np.complex128) + \
        sp.eye(Nc, N, dtype=np.complex128)
    wf, wq = rng.uniform(0.5, 1.5, Nb), rng.uniform(0.5, 1.5, Nc)
    weights = [(rsvdt.W_F_SQRT_INV, sp.diags(1 / np.sqrt(wf) + 0j, format="csr")), (rsvdt.B, Bm), (rsvdt.C_OUT, Cm),
               (rsvdt.W_Q_SQRT, sp.diags(np.sqrt(wq) + 0j, format="csr")),
               (rsvdt.W_Q_SQRT_INV, sp.diags(1 / np.sqrt(wq) + 0j, format="csr"))]
    F = synth.complex_normal(Nb, k * 16, 8)
    (U0, V0, S0), _, _, _ = solve(cfg, F, k, 1, False, A=A, weights=weights)
    (U1, V1, S1), used, _, _ = solve(cfg, F, k, 1, False, A=A, weights=weights, capacity=(2, True))
    assert used == 2 and U1.shape == (Nc, k * 16) and V1.shape == (Nb, k * 16)
    assert np.abs(S1 - S0).max() <= 1e-12 * S0.max()
    assert rel(V1, V0) < 1e-12
    # complex64 storage: each entry rounded once (relative 2^-24 per part).
    assert np.abs(U1 - U0).max() <= 2 ** -23 * np.abs(U0).max()
    assert rel(U1, U0) > 0


@pytest.mark.parametrize("prec", [0, 1])
def test_chunked_block_operator(built_lib, prec):
    """5x5 block-CSR operator: the k = 2 block-row kernels per chunk against
    the k = 4 kernels of the resident run, both precisions (one lane per
    row: the kernels of large problems)."""
    br, bc, bl = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    cfg = dict(w=0.5, Nw=8, dt=0.05, TransientLength=2 * np.pi / 0.5)
    k = 4
    F = synth.complex_normal(br.size * 5 - 5, k * 8, 9)
    (U0, V0, S0), _, _, _ = solve(cfg, F, k, 1, False, bcsr=(br, bc, bl), prec=prec, lanes=1)
    (U1, V1, S1), used, _, _ = solve(cfg, F, k, 1, False, bcsr=(br, bc, bl), prec=prec, capacity=(2, False), lanes=1)
    tol = 1e-12 if prec == 0 else 1e-5  # complex64 sums in another kernel's order
    assert used == 2
    assert np.abs(S1 - S0).max() <= tol * S0.max()


def test_capacity_mode_state_errors(built_lib):
    import rsvdt
    A, cfg = gl_problem()
    ctx = ctx_for(cfg, 2, 0, False, A=A)
    ctx.set_sketch(synth.complex_normal(64, 2 * 16, 1))
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.set_capacity_mode(1)
    assert e.value.status == rsvdt.ERR_STATE
    ctx.close()
    p = rsvdt.default_params(k=4, q=0, Nw=16, w=0.1, dt=0.15, TransientLength=2 * np.pi / 0.1, Display=0)
    ctx = rsvdt.Context(p)
    ctx.set_capacity_mode(3)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.set_operator(A)
    assert e.value.status == rsvdt.ERR_ARG  # 3 does not divide k = 4
    ctx.close()
