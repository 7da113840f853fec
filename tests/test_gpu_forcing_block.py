"""The forcing block of the complex64 block-row stages (rsvdt_set_forcing_block):
the half-step forcings of G steps formed by one kernel ahead of the stages
(SourceCode/CreateForcingOnFly.c:17-19 for every half step of
SourceCode/TSRK4.c:21-27) must give the same bits as stage 1 forming each
step's forcing itself, in both directions, for pair slabs (complex operator,
even Nw) and plain slabs (real operator), for block lengths that divide the
step count and ones that leave a partial block, and through
rsvdt_rk4_steps's host state (the end-of-run F3)."""
import numpy as np
import pytest

from rsvdt import synth

pytestmark = pytest.mark.gpu


def make_ctx(rsvdt, bcsr, k, Nw, fb, tr=0):
    p = rsvdt.default_params(k=k, q=0, Nw=Nw, w=0.5, dt=0.05, TransientLength=2 * np.pi / 0.5,
                             TransientRemoval=tr, precision=rsvdt.PREC_C64, Display=0)
    ctx = rsvdt.Context(p)
    ctx.set_operator_bcsr(*bcsr)
    # The block-row stage kernels (not the small-problem engines).
    ctx.set_step_engine(rsvdt.ENGINE_STAGES)
    ctx.set_lanes_per_row(1)
    ctx.set_forcing_block(fb)
    return ctx


@pytest.mark.parametrize("k,Nw,real", [(2, 8, False), (10, 16, False), (10, 32, False), (4, 16, True)])
def test_forcing_block_actions_are_bit_identical(built_lib, k, Nw, real):
    import rsvdt
    br, bc, bl = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    if real:
        bl = bl.real.astype(np.complex128)
    N = (br.size - 1) * 5
    res = {}
    for fb in (0, -1, 4):
        ctx = make_ctx(rsvdt, (br, bc, bl), k, Nw, fb)
        g = ctx.grid()
        assert g.Nw_eff == (Nw // 2 if real else Nw)
        F = synth.complex_normal(N, k * g.Nw_eff, 11)
        out = []
        for d in (rsvdt.DIRECT, rsvdt.ADJOINT):
            ctx.set_sketch(F)
            ctx.action(d)
            out.append(ctx.get_block())
        res[fb] = (out, ctx.forcing_block())
        ctx.close()
    # Automatic length: what fits in the spare half of the slab buffer.
    nwe = Nw // 2 if real else Nw
    assert res[0][1] == 0 and res[-1][1] == min(16, nwe // 2) and res[4][1] == 4
    for fb in (-1, 4):
        for a, b in zip(res[fb][0], res[0][0]):
            assert np.array_equal(a, b), fb


def test_forcing_block_rk4_steps_partial_blocks(built_lib):
    """21 steps = one graph of 16 (one block of 16, or four of 4) and a rest
    of 5 (a block of 5, or 4 + 1): y and the end-of-run F3 downloaded by
    rsvdt_rk4_steps are identical to the per-step synthesis."""
    import rsvdt
    bcsr = synth.op3d_blocks(n=4, shift=0.5, seed=5)
    N, k, Nw = 320, 10, 16
    F = synth.complex_normal(N, k * Nw, 21)
    y0 = synth.complex_normal(N, k, 22)
    f0 = synth.complex_normal(N, k, 23)
    out = {}
    for fb in (0, 16, 4):
        ctx = make_ctx(rsvdt, bcsr, k, Nw, fb)
        ctx.set_sketch(F)
        for d in (rsvdt.DIRECT, rsvdt.ADJOINT):
            out[(fb, d)] = ctx.rk4_steps(d, 7, 21, y0.copy(), f0.copy())
        ctx.close()
    for fb in (16, 4):
        for d in (rsvdt.DIRECT, rsvdt.ADJOINT):
            assert np.array_equal(out[(fb, d)][0], out[(0, d)][0]), (fb, d)
            assert np.array_equal(out[(fb, d)][1], out[(0, d)][1]), (fb, d)


def test_forcing_block_with_transient_removal(built_lib):
    import rsvdt
    bcsr = synth.op3d_blocks(n=4, shift=0.5, seed=3)
    Y = []
    for fb in (0, -1):
        ctx = make_ctx(rsvdt, bcsr, 2, 8, fb, tr=1)
        ctx.set_sketch(synth.complex_normal(320, 16, 9))
        ctx.action(rsvdt.DIRECT)
        Y.append(ctx.get_block())
        ctx.close()
    assert np.array_equal(Y[0], Y[1])


def test_forcing_block_rejects_other_lengths_and_skips_other_shapes(built_lib):
    import rsvdt
    bcsr = synth.op3d_blocks(n=3, shift=0.5, seed=3)
    ctx = make_ctx(rsvdt, bcsr, 2, 15, -1)  # odd Nw: not a compiled slab count
    with pytest.raises(rsvdt.RsvdtError):
        ctx.set_forcing_block(3)
    ctx.set_sketch(synth.complex_normal(135, 30, 1))
    ctx.action(rsvdt.DIRECT)
    assert ctx.forcing_block() == 0
    ctx.close()
