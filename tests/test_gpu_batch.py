"""Batching form: problems of uneven N, k, Nw and q solved together
(rsvdt_batch_*) give the same results as solving each on its own context
(the reference's main.c sequence, SourceCode/main.c:134-144, per problem)."""
import numpy as np
import pytest

from rsvdt import synth

pytestmark = pytest.mark.gpu

W0 = 0.1


def family():
    # (N, mu0, k, Nw, q): uneven sizes, test-vector counts, frequencies, q.
    specs = [(64, 0.2, 2, 8, 0), (150, 0.3, 3, 16, 1), (97, 0.25, 4, 8, 1), (233, 0.4, 2, 16, 0),
             (400, 0.35, 3, 8, 0)]
    T = 2 * np.pi / W0
    dt = T / 4096 * (1 + 1e-12)
    out = []
    for i, (N, mu0, k, nw, q) in enumerate(specs):
        A = synth.gl_stretched(N, mu0)
        F = synth.complex_normal(N, k * nw, 100 + i)
        out.append(dict(A=A, k=k, Nw=nw, q=q, F=F, dt=dt, T=T))
    return out


def params_of(rsvdt, pr, prec=0):
    return rsvdt.default_params(k=pr["k"], q=pr["q"], Nw=pr["Nw"], w=W0, dt=pr["dt"], TransientLength=pr["T"],
                                precision=prec, Display=0)


def solve_alone(rsvdt, pr, prec=0):
    ctx = rsvdt.Context(params_of(rsvdt, pr, prec))
    ctx.set_operator(pr["A"])
    ctx.set_sketch(pr["F"])
    ctx.run()
    out = ctx.get_results()
    ctx.close()
    return out


def mode_angle(U, Uref, k, nw):
    ang = 0.0
    for iw in range(nw):
        u = U[:, iw * k] / np.linalg.norm(U[:, iw * k])
        v = Uref[:, iw * k] / np.linalg.norm(Uref[:, iw * k])
        c = np.vdot(v, u)
        ang = max(ang, 2 * np.arcsin(min(1.0, np.linalg.norm(u - c / abs(c) * v) / 2)))
    return ang


def test_batch_matches_one_context_per_problem(built_lib):
    import rsvdt
    fam = family()
    b = rsvdt.Batch(rsvdt.PREC_C128)
    for pr in fam:
        i = b.add(params_of(rsvdt, pr), pr["A"])
        b.set_sketch(i, pr["F"])
    b.run()
    threads, lanes, ms = b.tuning()
    assert threads in (128, 256) and lanes in (1, 2, 4, 8) and ms > 0
    for i, pr in enumerate(fam):
        U, V, S = b.get_results(i)
        Ur, Vr, Sr = solve_alone(rsvdt, pr)
        # Batched stages sum nonzeros and forcing slabs over several lanes:
        # same operations, different summation order.
        assert (np.abs(S - Sr) / Sr).max() < 1e-9, i
        assert mode_angle(U, Ur, pr["k"], pr["Nw"]) < 1e-7
        assert mode_angle(V, Vr, pr["k"], pr["Nw"]) < 1e-7
    b.close()


def test_batch_precision_form_close_to_plain(built_lib):
    import rsvdt
    fam = family()
    b = rsvdt.Batch(rsvdt.PREC_C64)
    for pr in fam:
        i = b.add(params_of(rsvdt, pr), pr["A"])
        b.set_sketch(i, pr["F"])
    b.run()
    for i, pr in enumerate(fam):
        _, _, S = b.get_results(i)
        _, _, Sr = solve_alone(rsvdt, pr)
        assert (np.abs(S[0] - Sr[0]) / Sr[0]).max() < 1e-3, i
    b.close()


def test_batch_refinement_form(built_lib):
    """Refinement form in a batch: complex64 actions, the last adjoint
    action of every problem in complex128 (lockstep, its own graph): the
    gains come closer to the plain form's than the all-complex64 batch's,
    and equal the single-context refinement form's."""
    import rsvdt
    fam = family()
    res = {}
    for prec in (rsvdt.PREC_C64, rsvdt.PREC_C64_REFINE):
        b = rsvdt.Batch(prec)
        for pr in fam:
            i = b.add(params_of(rsvdt, pr), pr["A"])
            b.set_sketch(i, pr["F"])
        b.run()
        res[prec] = [b.get_results(i)[2] for i in range(len(fam))]
        b.close()
    e64, eref = [], []
    for i, pr in enumerate(fam):
        _, _, Sr = solve_alone(rsvdt, pr)
        _, _, Sa = solve_alone(rsvdt, pr, rsvdt.PREC_C64_REFINE)
        e64.append((np.abs(res[rsvdt.PREC_C64][i][0] - Sr[0]) / Sr[0]).max())
        eref.append((np.abs(res[rsvdt.PREC_C64_REFINE][i][0] - Sr[0]) / Sr[0]).max())
        # Same arithmetic as the single context up to the batched stages'
        # summation order (complex64 sums: 1e-6).
        assert (np.abs(res[rsvdt.PREC_C64_REFINE][i] - Sa) / Sa).max() < 1e-5, i
    print("leading-gain errors, complex64 batch:", max(e64), "refinement batch:", max(eref))
    assert max(eref) < max(e64)


@pytest.mark.parametrize("prec", [1, 2])
def test_launch_shapes_give_identical_results(built_lib, prec):
    """Every launch shape of the batched stages computes each value with the
    same operations in the same order: the gains of a complex64 batch (and
    of the refinement form, whose last action runs in complex128 from its
    own work list) are bit-identical for 128/256 threads, one lane per row
    and two test vectors per lane (all problems with an even k); the
    autotuner's choice agrees to the complex64 rounding."""
    import rsvdt
    fam = [pr for pr in family() if pr["k"] % 2 == 0]
    assert len(fam) >= 3
    out = {}
    for shape in ((128, 1, 1), (256, 1, 1), (128, 1, 2), (256, 1, 2), (0, 0, 0)):
        b = rsvdt.Batch(prec)
        for pr in fam:
            i = b.add(params_of(rsvdt, pr), pr["A"])
            b.set_sketch(i, pr["F"])
        if shape[0]:
            b.set_launch_shape(*shape)
        b.run()
        out[shape] = [b.get_results(i)[2] for i in range(len(fam))]
        if shape[0]:
            assert b.values_per_lane() == shape[2]
        b.close()
    base = out[(128, 1, 1)]
    for shape, S in out.items():
        for a, c in zip(S, base):
            if shape[0]:
                assert np.array_equal(a, c), shape
            else:  # the tuner may split rows over lanes: another summation order
                assert (np.abs(a - c) / c).max() < 1e-5
    b = rsvdt.Batch(rsvdt.PREC_C128)
    b.add(params_of(rsvdt, fam[0]), fam[0]["A"])
    with pytest.raises(rsvdt.RsvdtError):
        b.set_launch_shape(128, 1, 2)  # two values per lane need complex64 stages
    b.close()


def test_batch_errors(built_lib):
    import rsvdt
    b = rsvdt.Batch()
    with pytest.raises(rsvdt.RsvdtError) as e:
        b.run()
    assert e.value.status == rsvdt.ERR_STATE
    b.close()
