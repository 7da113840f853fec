"""Tiny problems through every stage-kernel family, in the release build and
in the bounds-checked debug build (RSVDT_DEBUG: every gathered column and
ring slot is checked on the device; a failed check skips the access and
makes the action return RSVDT_ERR_ARG). Random CSR operators with N in
{7, 33} and k in {1, 3, 10} (one lane per row: k_stage; automatic: the
lane-split batched kernel), the 3^3 five-field block operator with k in {2,
10} (k_rstage, and k_bstage in complex64); both directions, with and
without transient removal (N > Nw + 1 only), against the C restatement."""
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
pytestmark = pytest.mark.gpu


def random_operator(N, seed):
    """-2 I + a random complex sparse part with entries 0.3 CN(0,1)
    (|lambda| < 4: RK4-stable and accurate at dt = 0.05)."""
    rng = np.random.default_rng(seed)
    M = sp.random(N, N, density=0.3, random_state=seed, dtype=np.float64).tocsr()
    M.data = 0.3 * (rng.standard_normal(M.nnz) + 1j * rng.standard_normal(M.nnz)) / np.sqrt(2)
    return (M - 2.0 * sp.eye(N)).astype(np.complex128).tocsr()


def run_cases(expect_debug):
    import oracle
    import rsvdt
    from rsvdt import synth

    assert rsvdt.load_library().rsvdt_debug_build() == (1 if expect_debug else 0)
    cfg = dict(w=0.5, Nw=8, dt=0.05, TransientLength=2 * np.pi / 0.5)
    cases = []
    for N in (7, 33):
        for k in (1, 3, 10):
            for lanes in (1, 0):
                cases.append(("csr", N, k, lanes, rsvdt.PREC_C128))
    for k in (2, 10):
        for prec in (rsvdt.PREC_C128, rsvdt.PREC_C64):
            cases.append(("bcsr", 3, k, 1, prec))
    n = 0
    for kind, size, k, lanes, prec in cases:
        if kind == "csr":
            A = random_operator(size, seed=size + k)
            bcsr = None
        else:
            bcsr = synth.op3d_blocks(n=size, shift=0.5, seed=3)
            A = synth.bcsr_to_csr(*bcsr)
        # Transient removal projects on Nw + 1 snapshots: it needs N > Nw + 1.
        for tr in (False, True) if A.shape[0] > cfg["Nw"] + 1 else (False,):
            p = rsvdt.default_params(k=k, q=0, Nw=cfg["Nw"], w=cfg["w"], dt=cfg["dt"],
                                     TransientLength=cfg["TransientLength"], TransientRemoval=int(tr),
                                     precision=prec, Display=0)
            ctx = rsvdt.Context(p)
            if bcsr is not None:
                ctx.set_operator_bcsr(*bcsr)
            else:
                ctx.set_operator(A)
            ctx.set_lanes_per_row(lanes)
            F = synth.complex_normal(A.shape[0], k * ctx.grid().Nw_eff, 7)
            orc = oracle.Oracle(A, cfg["Nw"], cfg["w"], cfg["dt"], cfg["TransientLength"], transient_removal=tr)
            for d in (1, 0):
                ctx.set_sketch(F)
                ctx.action(d)
                Y = ctx.get_block()
                Yo = orc.ts_action(d, F)
                err = np.linalg.norm(Y - Yo) / np.linalg.norm(Yo)
                tol = 1e-4 if prec == rsvdt.PREC_C64 else (1e-9 if tr else 1e-10)
                assert err < tol, (kind, size, k, lanes, prec, tr, d, err)
                n += 1
            ctx.synchronize()
            ctx.close()
            orc.close()
    return n


def test_tiny_cases_release_build(built_lib):
    assert run_cases(expect_debug=False) == 52


def test_tiny_cases_debug_build(built_lib):
    from rsvdt import build

    path = build.build_library(debug=True)
    env = dict(os.environ, RSVDT_LIBRARY=path)
    root = os.path.dirname(HERE)
    code = ("import sys; sys.path[:0] = [%r, %r, %r]; import test_gpu_debug_build as t; "
            "print('cases', t.run_cases(expect_debug=True))" %
            (HERE, root, os.path.join(root, "rsvd-delta-t_gb300", "python")))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cases 52" in r.stdout
