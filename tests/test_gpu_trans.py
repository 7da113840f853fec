"""GPU parity of the transient simulation (rsvdt_trans_run, the replacement
of SourceCode/TransientRunRK4.c) against the oracle (oracle/trans_ref.py)
and against the closed form of RK4 for a diagonal operator.

Tolerances: the state, norms and snapshots are complex128 RK4 in the
reference's update order, differing from the oracle only by FMA contraction
and summation order: 1e-12 relative over hundreds of steps. The updated
transient norm of the removal estimate comes from a different (but exact to
rounding) orthogonalisation than the oracle's Householder QR: 1e-9 relative
where it is well above rounding, 1e-13 absolute where the synthetic
snapshots already span qss.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import trans_ref
from rsvdt import synth

pytestmark = pytest.mark.gpu


def ctx_for(A, w=0.1, Nw=16, dt=0.15, bcsr=None, beta=0.0):
    import rsvdt
    p = rsvdt.default_params(k=1, q=0, Nw=Nw, w=w, dt=dt, TransientLength=2 * np.pi / w, Display=0,
                             DiscFlg=int(beta > 0), beta=beta)
    ctx = rsvdt.Context(p)
    if bcsr is not None:
        ctx.set_operator_bcsr(*bcsr)
    else:
        ctx.set_operator(A)
    return ctx


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_gl_run_snapshots_and_estimates_match_oracle(built_lib):
    A = synth.gl_operator(64, mu0=0.2)
    w, Nw = 0.1, 16
    q0 = synth.complex_normal(64, 1, 3)[:, 0]
    ctx = ctx_for(A, w, Nw)
    q, norms, info, snaps, ests = ctx.trans_run(q0, periods=3, save_mod=50, con_val=0.0, save=True,
                                                removal_est=True)
    ref = trans_ref.trans_run(A, q0, w, Nw, trans_ref.grid_dt(w, Nw, 0.15), periods=3, save_mod=50,
                              con_val=0.0, removal_est_flag=True)
    assert info.dt == ref["dt"] and info.rend == ref["rend"] and info.steps == ref["steps"]
    assert info.stop == 0 and norms.size == ref["norms"].size
    assert rel(q, ref["q"]) < 1e-12
    assert np.abs(norms - ref["norms"]).max() <= 1e-12 * ref["norms"].max()
    assert (np.abs(norms - ref["norms"]) <= 1e-12 * ref["norms"]).all()
    assert sorted(snaps) == sorted(ref["snapshots"])
    for pos, v in snaps.items():
        assert rel(v, ref["snapshots"][pos]) < 1e-12, pos
    assert [e[0] for e in ests] == [1, 2, 3]
    for (p, ini, upd), (pr, inir, updr) in zip(ests, ref["estimates"]):
        assert (np.abs(ini - inir) <= 1e-11 * inir).all(), p
        assert np.abs(upd - updr).max() < 1e-13, p  # both at rounding level here
    ctx.close()


def test_removal_estimate_on_a_many_mode_operator(built_lib):
    """300 decaying modes: the synthetic snapshots do not span qss, so the
    updated transient norm is well above rounding."""
    rng = np.random.default_rng(5)
    N = 300
    lam = -rng.uniform(0.005, 0.05, N) + 1j * rng.uniform(-2, 2, N)
    A = sp.diags(lam).tocsr()
    w, Nw = 0.1, 16
    q0 = synth.complex_normal(N, 1, 3)[:, 0]
    ctx = ctx_for(A, w, Nw)
    q, norms, info, _, ests = ctx.trans_run(q0, periods=3, save_mod=50, con_val=0.0, removal_est=True)
    ref = trans_ref.trans_run(A, q0, w, Nw, trans_ref.grid_dt(w, Nw, 0.15), periods=3, save_mod=50,
                              con_val=0.0, removal_est_flag=True)
    assert rel(q, ref["q"]) < 1e-12
    assert len(ests) == 3
    for (p, ini, upd), (_, inir, updr) in zip(ests, ref["estimates"]):
        assert updr.min() > 1e-3
        assert (np.abs(ini - inir) <= 1e-11 * inir).all(), p
        assert (np.abs(upd - updr) <= 1e-9 * updr).all(), (p, upd, updr)
    ctx.close()


def test_diagonal_operator_closed_form(built_lib):
    rng = np.random.default_rng(0)
    lam = -rng.uniform(0.01, 0.3, 40) + 1j * rng.uniform(-1, 1, 40)
    q0 = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    ctx = ctx_for(sp.diags(lam).tocsr(), 0.1, 8, 0.2)
    q, norms, info, _, _ = ctx.trans_run(q0, periods=2, save_mod=25, con_val=0.0)
    P = trans_ref.rk4_amplification(lam * info.dt)
    ref = P ** info.rend * q0
    assert rel(q, ref) < 1e-12
    for pos in range(norms.size):
        r = np.linalg.norm(P ** (pos * 25) * q0)
        assert abs(norms[pos] - r) <= 1e-12 * r
    ctx.close()


def test_block_csr_single_vector_rows(built_lib):
    """5x5 block-CSR operator: the single-vector row kernel (k = 1) against
    the same operator as CSR in the oracle."""
    br, bc, bl = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    A = synth.bcsr_to_csr(br, bc, bl)
    w, Nw = 0.5, 8
    q0 = synth.complex_normal(A.shape[0], 1, 4)[:, 0]
    ctx = ctx_for(None, w, Nw, 0.05, bcsr=(br, bc, bl))
    q, norms, info, _, _ = ctx.trans_run(q0, periods=2, save_mod=7, con_val=0.0)
    ref = trans_ref.trans_run(A, q0, w, Nw, trans_ref.grid_dt(w, Nw, 0.05), periods=2, save_mod=7, con_val=0.0)
    assert info.stop == 0 and info.steps == ref["rend"]
    assert rel(q, ref["q"]) < 1e-12
    assert (np.abs(norms - ref["norms"]) <= 1e-12 * ref["norms"]).all()
    ctx.close()


def test_real_operator_and_discounting(built_lib):
    """A real operator (DFT over Nw snapshots with Nw/2 frequencies) and
    DiscFlg (A - beta I, SourceCode/LNSStructure.c:52-55)."""
    A = synth.gl_operator(64, nu=2.0, gamma=1.0, mu0=0.2)
    w, Nw, beta = 0.1, 16, 0.05
    q0 = synth.complex_normal(64, 1, 8)[:, 0]
    ctx = ctx_for(A, w, Nw, beta=beta)
    q, norms, info, _, ests = ctx.trans_run(q0, periods=2, save_mod=40, con_val=0.0, removal_est=True)
    Ad = (A - beta * sp.identity(64)).tocsr()
    ref = trans_ref.trans_run(Ad, q0, w, Nw, trans_ref.grid_dt(w, Nw, 0.15), periods=2, save_mod=40,
                              con_val=0.0, removal_est_flag=True, real_op=True)
    assert rel(q, ref["q"]) < 1e-12
    assert (np.abs(norms - ref["norms"]) <= 1e-12 * ref["norms"]).all()
    for (p, ini, upd), (_, inir, updr) in zip(ests, ref["estimates"]):
        assert (np.abs(ini - inir) <= 1e-11 * inir).all(), p
        assert np.abs(upd - updr).max() < 1e-9 * max(1.0, updr.max())
    ctx.close()


@pytest.mark.parametrize("case", ["diverged", "converged", "nan"])
def test_stopping_rules_match_oracle(built_lib, case):
    w, Nw = 0.1, 8
    q0 = np.ones(6, dtype=np.complex128) / 2
    lam, kw = {"diverged": (0.05, dict(div_val=2.0)), "converged": (-0.5, dict(con_val=1e-3)),
               "nan": (-0.1, dict())}[case]
    if case == "nan":
        q0[2] = np.nan
    A = sp.diags(np.full(6, lam, dtype=np.complex128)).tocsr()
    ctx = ctx_for(A, w, Nw, 0.2)
    q, norms, info, _, _ = ctx.trans_run(q0, periods=5, save_mod=10, **kw)
    ref = trans_ref.trans_run(A, q0, w, Nw, trans_ref.grid_dt(w, Nw, 0.2), periods=5, save_mod=10, **kw)
    assert info.stop == ref["stop"] != 0
    assert info.steps == ref["steps"]
    if case != "nan":
        assert rel(q, ref["q"]) < 1e-12
        assert (np.abs(norms - ref["norms"]) <= 1e-12 * np.maximum(ref["norms"], 1e-300)).all()
    else:
        assert np.isnan(q).any() and np.isnan(info.last_norm)
    ctx.close()


def test_bad_save_mod_is_an_argument_error(built_lib):
    import rsvdt
    ctx = ctx_for(sp.identity(8, dtype=np.complex128, format="csr") * -0.1)
    with pytest.raises(rsvdt.RsvdtError) as e:
        ctx.trans_run(np.ones(8, dtype=np.complex128), save_mod=0)
    assert e.value.status == rsvdt.ERR_ARG
    ctx.close()
