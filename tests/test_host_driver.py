"""The C drop-in driver for the reference's main.c (bin/rsvdt_main):
variables.yaml keys, defaults and errors of SourceCode/ReadUserInput.c,
PETSc-binary inputs and the results folder of SourceCode/SaveResults.c."""
import os
import subprocess

import numpy as np
import pytest

from rsvdt import petsc_io, synth


@pytest.fixture(scope="module")
def driver(built_lib):
    from rsvdt import build
    path = build.build_host()
    assert path and os.path.exists(path)
    return path


def write_yaml(path, **keys):
    with open(path, "w") as f:
        f.write("# generated for a test\n")
        for k, v in keys.items():
            f.write(f"{k}: {v}   # comment\n")


BASE = dict(RootDir="ROOT/", ResultsDir="", OperatorDir="A", k=2, q=0, Nw=8, w=0.1, TwoPI="false",
            TransientLength=62.83185307179586, dt=0.15, TransientRemoval="false", Display=0,
            TransICDir="ic", RandSeed=5)


def run(driver, tmp_path, **keys):
    cfg = dict(BASE)
    cfg.update(keys)
    cfg = {k: v for k, v in cfg.items() if v is not None}
    if cfg.get("RootDir") == "ROOT/":
        cfg["RootDir"] = str(tmp_path) + "/"
    y = tmp_path / "variables.yaml"
    write_yaml(y, **cfg)
    return subprocess.run([driver, "-inputs", str(y)], cwd=tmp_path, capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("missing,message", [
    ("TransientLength", "Must specify 'TransientLength'"),
    ("dt", "Must specify 'dt'"),
    ("w", "Must specify 'dt'"),  # the reference's message for a missing w (SourceCode/ReadUserInput.c:28)
    ("RootDir", "Must specify 'RootDir'"),
    ("OperatorDir", "Must specify 'OperatorDir'"),
    ("Nw", "Must specify 'Nw'"),
    ("TransICDir", "Must specify 'TransICDir'"),
])
def test_required_keys(driver, tmp_path, missing, message):
    r = run(driver, tmp_path, **{missing: None})
    assert r.returncode != 0
    assert message in r.stderr


def test_flag_requires_directory_and_bad_values(driver, tmp_path):
    r = run(driver, tmp_path, InputForcingFlg="true")
    assert r.returncode != 0 and "Must specify 'InputForcingDir'" in r.stderr
    r = run(driver, tmp_path, k="1.5")
    assert r.returncode != 0 and "no integer value" in r.stderr
    r = run(driver, tmp_path, TwoPI="maybe")
    assert r.returncode != 0 and "Unknown logical value" in r.stderr
    r = run(driver, tmp_path, DiscFlg="true")
    assert r.returncode != 0 and "specify 'beta'" in r.stderr
    # TransICFlg given (true or false) needs TransICDir, also in a transient run.
    r = run(driver, tmp_path, TransRun="true", TransICFlg="false", TransICDir=None)
    assert r.returncode != 0 and "Must specify 'TransICDir'" in r.stderr
    r = run(driver, tmp_path, TransSaveMod="2.5")
    assert r.returncode != 0 and "no integer value" in r.stderr
    # The drop-in driver's own key (resume points) follows the same logical syntax.
    r = run(driver, tmp_path, SaveResumeQ="maybe")
    assert r.returncode != 0 and "Unknown logical value" in r.stderr


def test_defaults_are_announced(driver, tmp_path):
    r = run(driver, tmp_path, k=None, q=None)
    out = r.stdout
    assert "Setting 'k' to default value: 3" in out
    assert "Setting 'q' to default value: 0" in out
    # The transient-run keys default only in a transient run
    # (SourceCode/ReadUserInput.c:142-171).
    assert "TransSaveMod" not in out
    r = run(driver, tmp_path, TransRun="true", TransICDir=None)
    out = r.stdout
    for key, val in [("TransICFlg", "0"), ("TransDivVal", "1000"), ("TransConVal", "1e-08"), ("TransSave", "0"),
                     ("TransRemovalEst", "0"), ("TransSaveMod", "100"), ("TransPeriods", "1")]:
        assert f"Setting '{key}' to default value: {val}" in out, key
    assert "Must specify 'TransICDir'" not in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("opt", [1, 2])
def test_end_to_end_matches_the_library(driver, tmp_path, opt):
    import rsvdt
    A = synth.gl_operator(64, mu0=0.2)
    petsc_io.write_mat(str(tmp_path / "A"), A)
    k, nw = 2, 8
    F = synth.complex_normal(64, k * nw, 9)
    petsc_io.write_mat(str(tmp_path / "F"), F)
    r = run(driver, tmp_path, InputForcingFlg="true", InputForcingDir="F", q=1, SaveResultsOpt=opt)
    assert r.returncode == 0, r.stderr + r.stdout
    folder = tmp_path / "ResolventModes_0"
    S = petsc_io.read_mat(str(folder / "S_hat")).toarray()
    assert S.shape == (k, nw)
    ctx = rsvdt.Context(rsvdt.default_params(k=k, q=1, Nw=nw, w=0.1, dt=0.15, TransientLength=BASE["TransientLength"],
                                             Display=0))
    ctx.set_operator(A)
    ctx.set_sketch(F)
    ctx.run()
    U, V, Sr = ctx.get_results()
    ctx.close()
    assert np.abs(S.real - Sr).max() <= 1e-12 * Sr.max() and np.abs(S.imag).max() == 0
    if opt == 1:
        for ik in range(k):
            Uk = petsc_io.read_mat(str(folder / f"U_hat_k{ik + 1}_allFreqs")).toarray()
            Vk = petsc_io.read_mat(str(folder / f"V_hat_k{ik + 1}_allFreqs")).toarray()
            assert Uk.shape == (64, nw) and Vk.shape == (64, nw)
            assert np.allclose(Uk, U[:, [iw * k + ik for iw in range(nw)]], atol=1e-14)
            assert np.allclose(Vk, V[:, [iw * k + ik for iw in range(nw)]], atol=1e-14)
    else:
        for iw in range(nw):
            Uw = petsc_io.read_mat(str(folder / f"U_hat_Freq{iw}_allK")).toarray()
            assert Uw.shape == (64, k)
            assert np.allclose(Uw, U[:, iw * k:(iw + 1) * k], atol=1e-14)
    assert (folder / "variables.yaml").exists()
    # A second run goes to the next folder (SourceCode/CreateResultsDir.c:21-27).
    r = run(driver, tmp_path, InputForcingFlg="true", InputForcingDir="F", q=0, SaveResultsOpt=opt)
    assert r.returncode == 0
    assert (tmp_path / "ResolventModes_1" / "S_hat").exists()


@pytest.mark.gpu
def test_transient_run_writes_the_reference_files(driver, tmp_path):
    """TransRun: true from a given initial vector (TransICFlg, path RootDir +
    ResultsDir + TransICDir): TransientSnapshots_0/ holds q_transient_<pos>
    every TransSaveMod steps, q_transient_norms, q_transient_last_snapshot,
    the per-period estimate vectors and the inputs copy
    (SourceCode/TransientRunRK4.c:116-222), matching the oracle."""
    from oracle import trans_ref
    A = synth.gl_operator(64, mu0=0.2)
    petsc_io.write_mat(str(tmp_path / "A"), A)
    q0 = synth.complex_normal(64, 1, 21)[:, 0]
    petsc_io.write_vec(str(tmp_path / "ic"), q0)
    r = run(driver, tmp_path, TransRun="true", TransICFlg="true", TransICDir="ic", TransSave="true",
            TransSaveMod=60, TransPeriods=2, TransRemovalEst="true", TransConVal=0)
    assert r.returncode == 0, r.stderr + r.stdout
    folder = tmp_path / "TransientSnapshots_0"
    ref = trans_ref.trans_run(A, q0, 0.1, 8, trans_ref.grid_dt(0.1, 8, 0.15), periods=2, save_mod=60, con_val=0.0,
                              removal_est_flag=True)
    norms = petsc_io.read_vec(str(folder / "q_transient_norms"))
    assert norms.size == ref["norms"].size and np.abs(norms.imag).max() == 0
    assert (np.abs(norms.real - ref["norms"]) <= 1e-12 * ref["norms"]).all()
    last = petsc_io.read_vec(str(folder / "q_transient_last_snapshot"))
    assert np.linalg.norm(last - ref["q"]) <= 1e-12 * np.linalg.norm(ref["q"])
    for pos, v in ref["snapshots"].items():
        got = petsc_io.read_vec(str(folder / f"q_transient_{pos}"))
        assert np.linalg.norm(got - v) <= 1e-12 * np.linalg.norm(v), pos
    assert not (folder / f"q_transient_{len(ref['snapshots'])}").exists()
    for p, ini, upd in ref["estimates"]:
        gi = petsc_io.read_vec(str(folder / f"Initial_transient_norm_period_{p}")).real
        gu = petsc_io.read_vec(str(folder / f"Updated_transient_norm_period_{p}")).real
        assert gi.size == 4 and (np.abs(gi - ini) <= 1e-11 * ini).all()
        assert np.abs(gu - upd).max() < 1e-12
    assert (folder / "variables.yaml").exists()
    assert "Transient run" in r.stdout and "Total snapshots to be saved" in r.stdout


@pytest.mark.gpu
def test_resume_point_continues_the_run(driver, tmp_path):
    """SaveResumeQ writes the forcing of every power sweep's direct action;
    fed back through InputForcingDir with q reduced by the sweep, it gives
    the same gains as the uninterrupted run."""
    A = synth.gl_operator(64, mu0=0.2)
    petsc_io.write_mat(str(tmp_path / "A"), A)
    F = synth.complex_normal(64, 2 * 8, 19)
    petsc_io.write_mat(str(tmp_path / "F"), F)
    r = run(driver, tmp_path, InputForcingFlg="true", InputForcingDir="F", q=2, SaveResumeQ="true",
            TransientRemoval="true")
    assert r.returncode == 0, r.stderr + r.stdout
    first = tmp_path / "ResolventModes_0"
    assert "Resume point (InputForcingDir with q = 1)" in r.stdout
    S_full = petsc_io.read_mat(str(first / "S_hat")).toarray()
    for sweep in (1, 2):
        Q = petsc_io.read_mat(str(first / f"Q_resume_sweep{sweep}"))
        assert Q.shape == (64, 16)
        r = run(driver, tmp_path, InputForcingFlg="true", InputForcingDir=f"ResolventModes_0/Q_resume_sweep{sweep}",
                q=2 - sweep, TransientRemoval="true")
        assert r.returncode == 0, r.stderr + r.stdout
        S = petsc_io.read_mat(str(tmp_path / f"ResolventModes_{sweep}" / "S_hat")).toarray()
        assert np.array_equal(S, S_full), sweep
