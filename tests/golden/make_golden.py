"""Generates the golden fixtures of the Ginzburg-Landau tutorial, the
reference's own known-answer case (Tutorial/Ginzburg-Landau/README.md:371-457
with the parameters of variables.yaml:16-39).

Writes, next to this script:
  A_GL                     the tutorial operator (PETSc binary, copied as data)
  gl_tutorial.json         the tutorial parameters; the dense FP64 resolvent
                           gains sigma_1..3 at its 42 frequencies (the known
                           answer that gains.png plots: sigma_1 peaks near
                           1.6e3 at omega = -0.65); the CPU oracle's RSVD-dt
                           gains for the full tutorial run (k=10, q=1,
                           transient removal) on a seeded sketch.

Run from the repository root:
    python tests/golden/make_golden.py <reference checkout>
(or set RSVDT_REFERENCE to the checkout); the fixtures it writes are what
the tests read.
"""
import json
import os
import shutil
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "rsvd-delta-t_gb300", "python"))

import oracle  # noqa: E402
from rsvdt import petsc_io, synth  # noqa: E402


# variables.yaml:16-39 (k, q, Nw, w, TwoPI, TransientLength, dt,
# TransientRemoval, RandSeed).
TUTORIAL = dict(k=10, q=1, Nw=42, w=0.05, TwoPI=False, TransientLength=10.0, dt=0.003,
                TransientRemoval=True, RandSeed=14)


def reference_root():
    """The reference checkout: the first argument, else RSVDT_REFERENCE."""
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RSVDT_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set RSVDT_REFERENCE)")
    return ref


def main():
    src = os.path.join(reference_root(), "Tutorial", "Ginzburg-Landau", "A_GL")
    dst = os.path.join(HERE, "A_GL")
    shutil.copyfile(src, dst)
    A = petsc_io.read_mat(dst)
    p = TUTORIAL
    om = [oracle.freq_of(i, p["Nw"], p["w"]) for i in range(p["Nw"])]
    Sd, _, _ = oracle.dense_resolvent_svd(A, om, 3)
    dt, Ns, Nt, R = oracle.setup_grid(p["w"], p["Nw"], p["dt"], p["TransientLength"])
    F = synth.gl_sketch(A.shape[0], p["k"], p["Nw"], seed=p["RandSeed"])
    t0 = time.time()
    orc = oracle.Oracle(A, p["Nw"], p["w"], p["dt"], p["TransientLength"], transient_removal=True)
    _, _, So = orc.run(F, p["q"])
    t_orc = time.time() - t0
    out = {
        "tutorial": p,
        "grid": {"dt": dt, "Ns": Ns, "Nt": Nt, "ResRatio": R},
        "omega": om,
        "dense_gains": Sd.tolist(),
        "oracle_gains": So.tolist(),
        "oracle_seconds": t_orc,
        "sketch": "synth.gl_sketch(500, 10, 42, seed=14): CN(0,1) from numpy default_rng(14)",
        "known_answer": {"sigma1_peak": 1.6e3, "omega_peak": -0.65,
                         "source": "Tutorial/Ginzburg-Landau/README.md:419-424, gains.png"},
    }
    with open(os.path.join(HERE, "gl_tutorial.json"), "w") as f:
        json.dump(out, f, indent=1)
    iw = int(np.argmax(Sd[0]))
    print(f"dense sigma1 peak {Sd[0, iw]:.2f} at omega {om[iw]:+.2f}; oracle {So[0, iw]:.2f} "
          f"({t_orc:.1f} s)")


if __name__ == "__main__":
    main()
