"""The reference's own known-answer case on the GPU: the Ginzburg-Landau
tutorial (Tutorial/Ginzburg-Landau/A_GL with the parameters of
variables.yaml:16-39: k = 10, q = 1, Nw = 42, w = 0.05, dt = 0.003,
TransientLength = 10, transient removal), on the seeded sketch of the golden
fixture (tests/golden/gl_tutorial.json, made by make_golden.py with the CPU
oracle). The plain form must reproduce the oracle's gains (tolerance 1e-9,
the plain form's parity target), hence the published peak sigma_1 ~ 1.6e3 at
omega = -0.65 (README.md:419-424, gains.png); the drop-in driver, fed the
same files and keys, writes the same S_hat."""
import json
import os
import subprocess

import numpy as np
import pytest

from rsvdt import petsc_io, synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture():
    g = json.load(open(os.path.join(GOLDEN, "gl_tutorial.json")))
    A = petsc_io.read_mat(os.path.join(GOLDEN, "A_GL"))
    p = g["tutorial"]
    F = synth.gl_sketch(A.shape[0], p["k"], p["Nw"], seed=p["RandSeed"])
    return g, A, p, F


def check_gains(S, g):
    So = np.array(g["oracle_gains"])
    Sd = np.array(g["dense_gains"])
    assert S.shape == So.shape
    err = np.abs(S - So) / So
    print("tutorial: max gain error against the oracle", err.max(), "(j <= 3:", err[:3].max(), ")")
    assert err.max() < 1e-9
    iw = int(np.argmax(S[0]))
    ka = g["known_answer"]
    assert abs(g["omega"][iw] - ka["omega_peak"]) < 1e-12
    assert abs(S[0, iw] - ka["sigma1_peak"]) / ka["sigma1_peak"] < 0.06
    assert abs(S[0, iw] - Sd[0, iw]) / Sd[0, iw] < 1e-6


def test_tutorial_gains_through_the_library(built_lib):
    import rsvdt
    g, A, p, F = fixture()
    ctx = rsvdt.Context(rsvdt.default_params(k=p["k"], q=p["q"], Nw=p["Nw"], w=p["w"], dt=p["dt"],
                                             TransientLength=p["TransientLength"],
                                             TransientRemoval=int(p["TransientRemoval"]), Display=0))
    ctx.set_operator(A)
    gr = ctx.grid()
    assert (gr.Ns, gr.Nt, gr.ResRatio) == (g["grid"]["Ns"], g["grid"]["Nt"], g["grid"]["ResRatio"])
    ctx.set_sketch(F)
    ctx.run()
    S = ctx.get_results(U=False, V=False)[2]
    ctx.close()
    check_gains(S, g)


def test_tutorial_gains_through_the_driver(built_lib, tmp_path):
    from rsvdt import build
    g, A, p, F = fixture()
    driver = build.build_host()
    petsc_io.write_mat(str(tmp_path / "F"), F)
    keys = dict(RootDir=str(tmp_path) + "/", ResultsDir="", OperatorDir="A_GL", InputForcingFlg="true",
                InputForcingDir="F", k=p["k"], q=p["q"], Nw=p["Nw"], w=p["w"], TwoPI="false",
                TransientLength=p["TransientLength"], dt=p["dt"], TransientRemoval="true", Display=0,
                TransICDir="ic", RandSeed=p["RandSeed"])
    os.symlink(os.path.join(GOLDEN, "A_GL"), tmp_path / "A_GL")
    with open(tmp_path / "variables.yaml", "w") as f:
        for key, v in keys.items():
            f.write(f"{key}: {v}\n")
    r = subprocess.run([driver, "-inputs", str(tmp_path / "variables.yaml")], cwd=tmp_path, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr + r.stdout
    S = petsc_io.read_mat(str(tmp_path / "ResolventModes_0" / "S_hat")).toarray()
    assert np.abs(S.imag).max() == 0
    check_gains(S.real, g)
