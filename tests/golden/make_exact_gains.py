"""Generates the exact-resolvent gains that the time-to-gains measurement and
its tests compare against (tests/golden/exact_gains_*.npz).

The oracle for a gain is the singular value of the continuous resolvent
W_q^{1/2} (i w I - A)^{-1} W_f^{-1/2} (the quantity RSVD-Delta-t
approximates, README.md:13-33 of the reference), computed in FP64 by a
sparse LU of (i w I - A) (SuperLU) and Lanczos (ARPACK through
scipy.sparse.linalg.svds) on the operator applied through the LU factors:
oracle.sparse_resolvent_svd. The operators are rebuilt from their seeds, so
the fixtures hold gains only.

  op3d24   the five-field 3D operator on a 24^3 grid (N = 69,120) with the
           benchmark's choices (k = 10, 32 frequencies j*0.1 for j = -16..15,
           diagonal W_q = W_f from cell volumes, recorded spectral shift):
           the 10 leading gains at every frequency. About an hour of CPU on
           8 cores.
  glfam48  the 48-problem Ginzburg-Landau batching family
           (synth.gl_family(48, seed=2024), discounted where unstable): the
           k leading gains of every problem at its Nw frequencies. A few
           minutes.

Run from the repository root:
    python tests/golden/make_exact_gains.py [op3d24] [glfam48] [--procs P]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "rsvd-delta-t_gb300", "python"))

import oracle  # noqa: E402
from rsvdt import synth, workloads  # noqa: E402


def op3d24(procs: int):
    wl = workloads.make_3d(n=24, k=10, Nw=32, shift="recorded")
    assert "recorded" in wl.meta["shift_method"], wl.meta
    A = synth.bcsr_to_csr(*wl.bcsr)
    om = [oracle.freq_of(iw, wl.Nw, wl.w) for iw in range(wl.Nw)]
    t0 = time.time()
    S, _, _ = oracle.sparse_resolvent_svd(A, om, wl.k, wq=wl.weights["W_sqrt"].diagonal(),
                                          wf_inv=wl.weights["W_sqrt_inv"].diagonal(), tol=1e-10,
                                          procs=procs)
    np.savez_compressed(os.path.join(HERE, "exact_gains_op3d24.npz"), S=S, omega=np.array(om),
                        shift=wl.meta["shift"], dt_in=wl.dt_in, N=wl.N, k=wl.k, Nw=wl.Nw)
    print(f"op3d24: {time.time() - t0:.0f} s, sigma_1 in [{S[0].min():.4g}, {S[0].max():.4g}]")


def glfam48(procs: int):
    import scipy.sparse as sp

    fam = synth.gl_family(48, seed=2024)
    out = {}
    t0 = time.time()
    for i, pr in enumerate(fam):
        A = pr["A"]
        if pr["beta"] > 0:
            A = (A - pr["beta"] * sp.eye(A.shape[0], format="csr")).tocsr()
        om = [oracle.freq_of(iw, pr["Nw"], 0.1) for iw in range(pr["Nw"])]
        S, _, _ = oracle.sparse_resolvent_svd(A, om, pr["k"], tol=1e-12, procs=procs)
        out[f"S{i}"] = S
        print(f"glfam48 problem {i}: N={pr['N']} k={pr['k']} Nw={pr['Nw']} sigma_1 max {S[0].max():.4g} "
              f"({time.time() - t0:.0f} s)", flush=True)
    np.savez_compressed(os.path.join(HERE, "exact_gains_glfam48.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="*", default=["glfam48", "op3d24"])
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    for w in a.which:
        {"op3d24": op3d24, "glfam48": glfam48}[w](a.procs)


if __name__ == "__main__":
    main()
