"""Benchmark of the RSVD-Delta-t RK4 hot path on one GB300.

A "step" is one forced RK4 step (SourceCode/TSRK4.c: four sparse products
with the forcing synthesis, stage updates and sampling fused into four
kernels) over all k = 10 test vectors of the 3D64 five-field operator
(N = 1,310,720, 45.26M complex128 nonzeros in 5x5 blocks, 32 frequencies),
the plain complex128 form. The metric is the step's algorithmic HBM
traffic over its device time:
    B_step = 4 S_A + S_F + 19 S_v + S_v / R
(S_A operator bytes, S_F = N Nw k 16 forcing coefficients, S_v = N k 16).
Inputs (14 GB working set) are far larger than L2, so no flush is needed.

Extra keys: roofline of the dominant kernel (stage 1, timed live with CUDA
events on the library's stream; DRAM traffic from a one-pass ncu capture),
the FP64 rate it achieves against a measured FP64 peak (the plain form is
FP64-bound on this part), the complex64 precision form's step, e2e through
the C ABI with host buffers, the CPU baseline (the C restatement timed on
the host cores), and the side experiments: time to gains of the whole q = 1
solve in the plain, complex64 and refinement forms with phase times; the
48-problem batching form with the autotuned launch shapes; the 500-node
Ginzburg-Landau configuration with its step engine and CPU baseline; with
flags, the learned sketch (GL and 3D families) and the 128^3 capacity
case.

--impl reference times the reference's CPU algorithm (the C restatement
in oracle/, since the reference itself needs PETSc/SLEPc/MPI) on all host
threads for the same step and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "rsvd-delta-t_gb300", "python")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "time-to-gains at ≤1e-3 rel err: chosen vs plain GPU; RK4 SpMM HBM GB/s vs peak"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch):
    """FP64 peak of this GPU, measured: best of 5 cuBLAS DGEMMs 4096^3."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    del a, b
    return 2 * 4096**3 / (best * 1e-3) / 1e12


def cpu_baseline(wl, g, Fk, steps: int, threads: int, warmup: int = 0):
    """C restatement (oracle/) timing one step of all k test vectors: the
    test vectors one after another, the row loops of each RK4 step on
    `threads` host threads (all cores; faster than one thread per test
    vector, which leaves cores idle when k is below the core count).
    `warmup` untimed steps first; returns the mean seconds per timed step."""
    import oracle
    from rsvdt import synth

    A = synth.bcsr_to_csr(*wl.bcsr) if wl.bcsr is not None else wl.csr
    orc = oracle.Oracle(A, wl.Nw, wl.w, wl.dt_in, wl.transient_length)
    orc.set_row_threads(threads)
    N = wl.N
    y = [np.zeros(N, complex) for _ in range(wl.k)]
    F3 = [np.zeros(N, complex) for _ in range(wl.k)]
    times = []
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        for ik in range(wl.k):
            y[ik], F3[ik] = orc.rk4_steps(1, Fk, 1 + s, 1, y[ik], F3[ik])
        if s >= warmup:
            times.append(time.perf_counter() - t0)
    orc.close()
    return float(np.mean(times))


def parity_steps(wl, ctx, ctx64, threads: int, seed: int = 77):
    """Parity at the benchmark's own size: two forced RK4 steps of all k test
    vectors on the full operator through rsvdt_rk4_steps (host state, the
    stage kernels the benchmark times: complex128 and the complex64
    precision form) from a seeded state y0, F3_0 and the contexts' seeded
    sketch, against the C restatement (SourceCode/TSRK4.c:18-47) on the same
    inputs. The steps start at i0 = Ns, so the second one crosses the wrap
    of the forcing index (jt = 2 Ns -> 0). Complex128 is checked in both
    directions; the complex64 form (rounded state, FP32 arithmetic) against
    the same complex128 oracle, where its error is the FP32 rounding."""
    import oracle
    import rsvdt
    from rsvdt import synth

    t0 = time.perf_counter()
    g = ctx.grid()
    F = ctx.get_block()
    F64 = ctx64.get_block()
    same_sketch = bool(np.array_equal(F, F64))
    del F64
    N, k = wl.N, wl.k
    y0 = synth.complex_normal(N, k, seed)
    F30 = synth.complex_normal(N, k, seed + 1)
    A = synth.bcsr_to_csr(*wl.bcsr)
    orc = oracle.Oracle(A, wl.Nw, wl.w, wl.dt_in, wl.transient_length)
    orc.set_row_threads(threads)
    i0, nsteps = g.Ns, 2
    out = {"workload": f"{wl.name}: {nsteps} forced RK4 steps (i0 = Ns = {g.Ns}, across the forcing-index wrap) "
                       f"of all k = {k} test vectors through rsvdt_rk4_steps, against the C restatement",
           "same_sketch_in_both_contexts": same_sketch}
    for name, c, d in (("c128_direct", ctx, rsvdt.DIRECT), ("c128_adjoint", ctx, rsvdt.ADJOINT),
                       ("c64_direct", ctx64, rsvdt.DIRECT)):
        y, F3 = c.rk4_steps(d, i0, nsteps, y0.copy(), F30.copy())
        ey, ef = [], []
        for ik in range(k):
            Fk = np.asfortranarray(F[:, [iw * k + ik for iw in range(g.Nw_eff)]])
            yo, F3o = orc.rk4_steps(d, Fk, i0, nsteps, y0[:, ik], F30[:, ik])
            ey.append(float(np.linalg.norm(y[:, ik] - yo) / np.linalg.norm(yo)))
            ef.append(float(np.linalg.norm(F3[:, ik] - F3o) / np.linalg.norm(F3o)))
        out[name] = {"y_rel_err_max": max(ey), "F3_rel_err_max": max(ef)}
    orc.close()
    # Tolerances: complex128 1e-11 (the GPU's negative-frequency phasor is the
    # exact conjugate of the positive one, the reference's is evaluated from
    # a larger argument); complex64 1e-5 (FP32 rounding of the state, the
    # operator, the forcing slabs and the sums, u = 6e-8, times the stage
    # count and the cancellation in the products).
    out["tolerance"] = {"c128": 1e-11, "c64": 1e-5}
    out["pass"] = bool(same_sketch and all(out[n]["y_rel_err_max"] < 1e-11 and out[n]["F3_rel_err_max"] < 1e-11
                                           for n in ("c128_direct", "c128_adjoint")) and
                       out["c64_direct"]["y_rel_err_max"] < 1e-5 and out["c64_direct"]["F3_rel_err_max"] < 1e-5)
    out["s"] = round(time.perf_counter() - t0, 1)
    return out


def parity_batch(fam, sketches, params, S_batched: dict, threads: int, q: int, count: int = 6):
    """Parity of the batching form against the C restatement: `count` of
    the batch's problems (the one where the complex64 batch is furthest
    from the complex128 one, then the smallest ones, up to a row budget)
    solved by the oracle's whole sequence (SourceCode/main.c:134-144) with
    the batch's sketches, compared per gain with every batched form."""
    import oracle

    t0 = time.perf_counter()
    worst = S_batched.get("worst_c64")
    order = sorted(range(len(fam)), key=lambda i: fam[i]["N"] * fam[i]["k"] * fam[i]["Nw"])
    pick = ([worst] if worst is not None else []) + [i for i in order if i != worst]
    pick = pick[:count]
    out = {"problems": [{"index": i, "N": fam[i]["N"], "k": fam[i]["k"], "Nw": fam[i]["Nw"]} for i in pick]}
    errs = {name: [] for name in S_batched if name != "worst_c64"}
    for i in pick:
        pr = fam[i]
        p = params(pr)
        A = pr["A"]
        if pr["beta"] > 0:
            import scipy.sparse as sp
            A = (A - pr["beta"] * sp.eye(A.shape[0], format="csr")).tocsr()
        orc = oracle.Oracle(A, pr["Nw"], p.w, p.dt, p.TransientLength, threads=threads)
        _, _, So = orc.run(sketches[i], q)
        orc.close()
        for name in errs:
            Sb = S_batched[name][i]
            errs[name].append((float((np.abs(Sb[:3] - So[:3]) / So[:3]).max()),
                               float((np.abs(Sb - So) / So).max())))
    for name, e in errs.items():
        out[name] = {"gain_rel_err_max_j<=3": max(x[0] for x in e), "gain_rel_err_max": max(x[1] for x in e),
                     "per_problem_j<=3": [x[0] for x in e]}
    out["tolerance"] = {"batched_c128": 1e-9}
    out["pass_c128"] = bool(out["batched_c128"]["gain_rel_err_max"] < 1e-9) if "batched_c128" in out else None
    out["s"] = round(time.perf_counter() - t0, 1)
    return out


TTG_TOL = 1e-3  # relative gain error that time-to-gains is measured at


def gain_rel_err(S, S_exact, jmax: int = 3) -> float:
    """max over frequencies and j <= jmax of |s_j - sigma_j| / sigma_j,
    sigma_j the exact resolvent gains (k x Nw, as the results' S)."""
    j = min(jmax, S.shape[0], S_exact.shape[0])
    return float((np.abs(S[:j] - S_exact[:j]) / S_exact[:j]).max())


def ttg_search(run, err, plans, q_max: int, log=None, deadline: float = float("inf")):
    """Time to gains of one solver form: for each plan (transient periods,
    transient removal, dt factor), q = 0, 1, ... until the gains are within
    TTG_TOL of the exact ones (max over j <= 3 and all frequencies); a run
    already slower than the best time found ends its plan (a larger q costs
    more). run(q, periods, tr, dtf) -> (seconds, S); err(S, jmax) -> the
    gain error of S against the exact gains. Returns (best, trace): best =
    the fastest run that met the tolerance (None if none did)."""
    best, trace = None, []
    for periods, tr, dtf in plans:
        for q in range(q_max + 1):
            if time.perf_counter() > deadline:
                break
            t, S = run(q, periods, tr, dtf)
            e = err(S, 3)
            e1 = err(S, 1)
            rec = {"q": q, "periods": periods, "tr": int(tr), "dt_factor": dtf, "s": round(t, 4),
                   "err_j<=3": float(f"{e:.3e}"), "err_j1": float(f"{e1:.3e}")}
            trace.append(rec)
            if log:
                log(rec)
            if e <= TTG_TOL:
                if best is None or t < best["s"]:
                    best = rec
                break
            if best is not None and t >= best["s"]:
                break
    return best, trace


def ttg_gl1(q_max: int = 8):
    """Time to gains on the 500-node Ginzburg-Landau configuration (k = 10,
    64 frequencies j*0.1, j = -32..31, dt = T/4096) against the dense FP64
    resolvent: plain complex128 against the precision forms."""
    import oracle
    import rsvdt
    from rsvdt import synth, workloads

    wl = workloads.make_gl1(k=10)
    F = synth.gl_sketch(500, 10, 64)
    om = [oracle.freq_of(i, 64, 0.1) for i in range(64)]
    Sx = oracle.dense_resolvent_svd(wl.csr, om, 3)[0]
    T = 2 * np.pi / 0.1

    def runner(prec):
        def run(q, periods, tr, dtf):
            p = rsvdt.default_params(k=10, q=q, Nw=64, w=0.1, dt=wl.dt_in * dtf, TransientLength=periods * T,
                                     TransientRemoval=int(tr), precision=prec, Display=0)
            ctx = rsvdt.Context(p)
            ctx.set_operator(wl.csr)
            ctx.set_sketch(F)
            ctx.synchronize()
            t0 = time.perf_counter()
            ctx.run()
            S = ctx.get_results(U=False, V=False)[2]
            t = time.perf_counter() - t0
            ctx.close()
            return t, S
        return run

    plans = [(1, 0, 1.0), (2, 0, 1.0), (3, 0, 1.0), (1, 1, 1.0)]
    return ttg_forms(runner, lambda S, j: gain_rel_err(S, Sx, j), [float(Sx[0].min()), float(Sx[0].max())],
                     plans, q_max,
                     "GL1: N=500 Ginzburg-Landau, k=10, Nw=64, dt=T/4096; exact gains: dense FP64 SVD of "
                     "(i w I - A)^-1")


def ttg_3d24(q_max: int = 24, seed: int = 99, k: int = 16):
    """Time to gains on the five-field 3D operator at 24^3 (N = 69,120, the
    3D64 configuration's 32 frequencies, diagonal W, recorded spectral
    shift, dt at 0.7 of the RK4 stability limit) against the exact resolvent gains
    of tests/golden/exact_gains_op3d24.npz (sparse LU + Lanczos, FP64), with
    k = 16 test vectors: the leading singular values of this operator's
    resolvent are close together at every frequency, and with the
    configuration's k = 10 the sketch needs about q = 40 power iterations
    (measured: 3.4e-3 at q = 24, falling by 7% per iteration)."""
    import rsvdt
    from rsvdt import workloads

    fx = np.load(os.path.join(ROOT, "tests", "golden", "exact_gains_op3d24.npz"))
    wl = workloads.make_3d(n=24, k=k, Nw=32)
    assert "recorded" in wl.meta["shift_method"] and abs(float(fx["shift"]) - wl.meta["shift"]) < 1e-15
    Sx = fx["S"]
    T = 2 * np.pi / wl.w

    def runner(prec):
        def run(q, periods, tr, dtf):
            p = rsvdt.default_params(k=wl.k, q=q, Nw=wl.Nw, w=wl.w, dt=wl.dt_in * dtf, TransientLength=periods * T,
                                     TransientRemoval=int(tr), precision=prec, Display=0)
            ctx = rsvdt.Context(p)
            ctx.set_operator_bcsr(*wl.bcsr)
            ctx.set_weight(rsvdt.W_Q_SQRT, wl.weights["W_sqrt"])
            ctx.set_weight(rsvdt.W_F_SQRT_INV, wl.weights["W_sqrt_inv"])
            ctx.set_weight(rsvdt.W_Q_SQRT_INV, wl.weights["W_sqrt_inv"])
            ctx.random_sketch(seed)
            ctx.synchronize()
            t0 = time.perf_counter()
            ctx.run()
            S = ctx.get_results(U=False, V=False)[2]
            t = time.perf_counter() - t0
            ctx.close()
            return t, S
        return run

    # The transient decays as exp(-0.05 t) (rightmost eigenvalue -0.05): two
    # periods leave 2e-3 of it, three 8e-5. Transient removal is not in the
    # plans: its FP64 Galerkin step costs more per action here than a third
    # period does. At the stability-limit dt the RK4 response itself is off
    # by about 1e-3 at the highest frequencies (w dt = 0.68; RK4's error
    # grows as (w dt)^4): measured, the complex64 run levels off near 1.4e-3
    # by q = 20 and never meets the tolerance. With dt at 0.7 of the limit
    # (w dt = 0.48) it meets it at q = 22 (9.7e-4; 1.3e-3 at q = 21), with
    # 0.5 at q = 24; the error falls about 20% per power iteration near
    # there. The plan starts at q = 22 and searches up or down from there,
    # since a search from q = 0 would cost minutes of complex128 runs.
    plans = [(3, 0, 0.7)]
    return ttg_forms(runner, lambda S, j: gain_rel_err(S, Sx, j), [float(Sx[0].min()), float(Sx[0].max())],
                     plans, q_max, budget_s=300.0, q_start={(3, 0, 0.7): 22}, workload=
                     f"3D24: N={wl.N} five-field operator (5x5 blocks), k={k}, Nw=32, diagonal W, shift "
                     f"{wl.meta['shift']:.6g} ({wl.meta['shift_method']}), dt={wl.dt_in:.4g} (RK4 limit) x 0.7; "
                     "exact gains: sparse LU + Lanczos (tests/golden/exact_gains_op3d24.npz)")


def ttg_followup(run, err, plans, q_start: dict, q_max: int, log=None, deadline: float = float("inf")):
    """ttg_search from a given q per plan: the run starts at q_start[plan],
    goes up until the tolerance is met, and down while it still is, so that
    every reported q is the form's own smallest one; plans without a start
    are skipped. Used for the further forms, starting one q below the q at
    which the first form met the tolerance (the sketch sets the error, not
    the arithmetic: the forms' errors agree to far below the tolerance), and
    for a first form whose plan comes with a starting q."""
    best, trace = None, []
    for periods, tr, dtf in plans:
        q = q_start.get((periods, tr, dtf))
        if q is None:
            continue
        q = max(0, q)
        met = {}
        while 0 <= q <= q_max and q not in met and time.perf_counter() <= deadline:
            t, S = run(q, periods, tr, dtf)
            e = err(S, 3)
            rec = {"q": q, "periods": periods, "tr": int(tr), "dt_factor": dtf, "s": round(t, 4),
                   "err_j<=3": float(f"{e:.3e}"), "err_j1": float(f"{err(S, 1):.3e}")}
            trace.append(rec)
            if log:
                log(rec)
            met[q] = rec if e <= TTG_TOL else None
            if met[q] is None:
                if q - 1 in met and met[q - 1]:
                    break
                q += 1
            else:
                if q == 0 or (q - 1 in met):
                    break
                q -= 1
        ok = [r for r in met.values() if r]
        if ok:
            r = min(ok, key=lambda r: r["q"])
            if best is None or r["s"] < best["s"]:
                best = r
    return best, trace


def ttg_forms(runner, err, sigma1_range, plans, q_max, workload, forms=None, budget_s: float = 180.0,
              q_start: dict | None = None):
    """Time to gains of every form: the first form (the fastest per run,
    complex64) is searched over all plans and q (ttg_search), or from
    q_start[plan] up or down when given (ttg_followup), the others around
    the q it needed (ttg_followup). Each form is run once untimed first
    (kernel loading). `forms`: (name, precision) pairs, the plain form named
    plain_c128. The first form's search stops after half of budget_s
    seconds, every further form's after its share of the rest."""
    import rsvdt

    forms = forms or (("precision_c64", rsvdt.PREC_C64), ("plain_c128", rsvdt.PREC_C128),
                      ("precision_c64_refine", rsvdt.PREC_C64_REFINE))
    out = {"workload": workload, "tolerance": TTG_TOL,
           "search": "per plan (transient periods, transient removal, dt factor): the smallest q with "
                     "max_{w, j<=3} |s_j - sigma_j| / sigma_j <= 1e-3; the fastest such run per form (first "
                     "form: q = 0, 1, ..., or from the plan's starting q up or down; the others from one q "
                     "below the first form's q, up or down)",
           "plans": [list(pl) for pl in plans], "sigma1_range": sigma1_range}
    if q_start:
        out["q_start"] = {",".join(str(x) for x in pl): q for pl, q in q_start.items()}
    q_found = None
    t_start = time.perf_counter()
    for fi, (name, prec) in enumerate(forms):
        if fi == 0:
            deadline = t_start + budget_s / 2
        else:
            deadline = time.perf_counter() + (t_start + budget_s - time.perf_counter()) / (len(forms) - fi)
        run = runner(prec)
        run(0, plans[0][0], plans[0][1], plans[0][2])  # warm-up

        def log(r, n=name):
            print(f"ttg {n} {r}", file=sys.stderr, flush=True)

        if q_found is None:
            if q_start:
                best, trace = ttg_followup(run, err, plans, q_start, q_max, log=log, deadline=deadline)
            else:
                best, trace = ttg_search(run, err, plans, q_max, log=log, deadline=deadline)
            q_found = {}  # per plan, the smallest q that met the tolerance
            for r in trace:
                key = (r["periods"], r["tr"], r["dt_factor"])
                if r["err_j<=3"] <= TTG_TOL:
                    q_found[key] = min(q_found.get(key, r["q"]), r["q"])
        else:
            best, trace = ttg_followup(run, err, plans, {pl: q - 1 for pl, q in q_found.items()}, q_max, log=log,
                                       deadline=deadline)
        out[name] = {"best": best, "trace": trace}
        if trace:
            lo = min(trace, key=lambda r: r["err_j<=3"])
            out[name]["lowest_err_j<=3"] = {k: lo[k] for k in ("q", "periods", "err_j<=3", "err_j1", "s")}
    base = out["plain_c128"]["best"]
    chosen = [(out[n]["best"]["s"], n) for n, _ in forms if n != "plain_c128" and out[n]["best"]]
    if base and chosen:
        t, n = min(chosen)
        out["chosen"] = n
        out["ratio_plain_over_chosen"] = round(base["s"] / t, 3)
    else:
        out["chosen"] = None
        out["ratio_plain_over_chosen"] = None
    out["wall_s"] = round(time.perf_counter() - t_start, 1)
    return out


def ttg_batch(q_max: int = 12, sigma_max: float = 1e3, seed: int = 2024, budget_s: float = 120.0):
    """Time to gains on the batching family (48 Ginzburg-Landau problems, N
    log-uniform in [200, 20000], k in {6, 10, 16}, Nw in {16, 32, 64}, one
    transient period) against the exact resolvent gains of
    tests/golden/exact_gains_glfam48.npz, on the problems whose exact leading
    gain is at most sigma_max. (Above it the transient growth of these
    non-normal operators, up to 1e43, exceeds what a run of the configured
    transient length removes: no form reaches the exact gains there.)

    Each problem gets its own q, as the batch allows: the smallest q with
    max_{w, j<=3} error <= 1e-3 in the complex128 batch (q = 0 .. q_max, all
    problems at each q; a problem that never meets it leaves the set). Then
    every form solves the set with those q: the plain method one context
    after another in complex128, and the batch in complex64, complex64 with
    the FP64 sweep, and complex128; each form's time, worst error and the
    problems it leaves above the tolerance are reported, and the chosen form
    is the fastest with none above."""
    import rsvdt
    from rsvdt import synth

    t_start = time.perf_counter()
    fam = synth.gl_family(48, seed=seed)
    fx = np.load(os.path.join(ROOT, "tests", "golden", "exact_gains_glfam48.npz"))
    idx = [i for i in range(len(fam)) if fx[f"S{i}"][0].max() <= sigma_max]
    Sx = {i: fx[f"S{i}"] for i in idx}
    T = 2 * np.pi / 0.1
    dt = T / 4096 * (1 + 1e-12)
    sk = {i: synth.complex_normal(fam[i]["N"], fam[i]["k"] * fam[i]["Nw"], seed + 1 + i) for i in idx}

    def params(i, prec, q):
        pr = fam[i]
        return rsvdt.default_params(k=pr["k"], q=q, Nw=pr["Nw"], w=0.1, dt=dt, TransientLength=T,
                                    DiscFlg=int(pr["beta"] > 0), beta=pr["beta"], precision=prec, Display=0)

    def run(prec, qs: dict, batched: bool):
        """qs: problem -> q. Returns (seconds, problem -> S)."""
        S = {}
        if batched:
            b = rsvdt.Batch(prec)
            order = list(qs)
            for i in order:
                b.add(params(i, prec, qs[i]), fam[i]["A"])
            for j, i in enumerate(order):
                b.set_sketch(j, sk[i])
            t0 = time.perf_counter()
            b.run()
            for j, i in enumerate(order):
                S[i] = b.get_results(j)[2]
            t = time.perf_counter() - t0
            b.close()
            return t, S
        t = 0.0
        for i, q in qs.items():
            ctx = rsvdt.Context(params(i, prec, q))
            ctx.set_operator(fam[i]["A"])
            ctx.set_sketch(sk[i])
            ctx.synchronize()
            t0 = time.perf_counter()
            ctx.run()
            S[i] = ctx.get_results(U=False, V=False)[2]
            t += time.perf_counter() - t0
            ctx.close()
        return t, S

    # Per-problem q (complex128 batch).
    run(rsvdt.PREC_C128, {i: 0 for i in idx}, True)  # warm-up (autotuning, kernel loading)
    qstar, scan = {}, []
    for q in range(q_max + 1):
        todo = {i: q for i in idx if i not in qstar}
        if not todo or time.perf_counter() - t_start > budget_s:
            break
        t, S = run(rsvdt.PREC_C128, todo, True)
        met = [i for i in todo if gain_rel_err(S[i], Sx[i]) <= TTG_TOL]
        for i in met:
            qstar[i] = q
        scan.append({"q": q, "problems": len(todo), "met": len(met), "s": round(t, 3)})
        print(f"ttg batch scan {scan[-1]}", file=sys.stderr, flush=True)
    out = {"workload": f"{len(idx)} of the 48 batching-family problems with exact sigma_1 <= {sigma_max:g} "
                       f"(N {min(fam[i]['N'] for i in idx)}..{max(fam[i]['N'] for i in idx)}), dt = T/4096, one "
                       "transient period; exact gains: sparse LU + Lanczos (tests/golden/exact_gains_glfam48.npz)",
           "tolerance": TTG_TOL, "problems_in_range": len(idx),
           "problems_excluded_sigma1": sorted(float(f"{fx[f'S{i}'][0].max():.3g}") for i in range(len(fam))
                                              if i not in idx),
           "q_scan": scan, "problems_met": len(qstar),
           "problems_not_met_within_q_max": [i for i in idx if i not in qstar],
           "q_per_problem": {str(i): q for i, q in sorted(qstar.items())}}
    if not qstar:
        out["chosen"] = None
        out["ratio_plain_over_chosen"] = None
        return out
    for name, prec, batched in (("batched_c64", rsvdt.PREC_C64, True),
                                ("batched_c64_refine", rsvdt.PREC_C64_REFINE, True),
                                ("batched_c128", rsvdt.PREC_C128, True),
                                ("plain_c128", rsvdt.PREC_C128, False)):
        if not batched:
            run(prec, {i: 0 for i in list(qstar)[:2]}, False)  # warm-up
        t, S = run(prec, qstar, batched)
        errs = {i: gain_rel_err(S[i], Sx[i]) for i in qstar}
        out[name] = {"s": round(t, 3), "err_max_j<=3": float(f"{max(errs.values()):.3e}"),
                     "problems_over_tolerance": sorted(i for i, e in errs.items() if e > TTG_TOL)}
        print(f"ttg batch {name} {out[name]}", file=sys.stderr, flush=True)
    ok = [(out[n]["s"], n) for n in ("batched_c64", "batched_c64_refine", "batched_c128")
          if not out[n]["problems_over_tolerance"]]
    base = out["plain_c128"]
    if ok and not base["problems_over_tolerance"]:
        t, n = min(ok)
        out["chosen"] = n
        out["ratio_plain_over_chosen"] = round(base["s"] / t, 3)
    else:
        out["chosen"] = None
        out["ratio_plain_over_chosen"] = None
    out["wall_s"] = round(time.perf_counter() - t_start, 1)
    return out


def equal_q_speedup(n: int, seed: int = 4321):
    """Speed-up at equal work (not time to gains: no exact gains exist at
    this size). Full RSVD-Delta-t solve (SourceCode/main.c:134-144: direct action,
    q = 1 power iteration, SVDs, adjoint action) on the 3D operator of an
    n^3 grid, k = 10, Nw = 32, two transient periods: wall time from the
    first device action to the gains on the host, inputs resident. Plain
    complex128 against the precision form (complex64 stages, FP64 DFT / QR /
    SVD) and the refinement form (the same with the last adjoint action in
    complex128); their gain and first-mode errors are measured against the
    plain result. Before the timed run each form steps 32 untimed steps in
    both directions (kernel loading, graph capture)."""
    import rsvdt
    from rsvdt import workloads

    wl = workloads.make_3d(n=n)
    out = {}
    res = {}
    for name, prec in (("plain_c128", rsvdt.PREC_C128), ("precision_c64", rsvdt.PREC_C64),
                       ("precision_c64_refine", rsvdt.PREC_C64_REFINE)):
        ctx = rsvdt.Context(wl.params(precision=prec))
        ctx.set_operator_bcsr(*wl.bcsr)
        ctx.set_weight(rsvdt.W_Q_SQRT, wl.weights["W_sqrt"])
        ctx.set_weight(rsvdt.W_F_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.set_weight(rsvdt.W_Q_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.random_sketch(seed)
        for d in (rsvdt.DIRECT, rsvdt.ADJOINT):
            ctx.rk4_reset(d)
            ctx.rk4_advance(d, 1, 32)
        ctx.random_sketch(seed)
        ctx.synchronize()
        ctx.reset_timings()
        t0 = time.perf_counter()
        ctx.run()
        S = ctx.get_results(U=False, V=False)[2]
        t = time.perf_counter() - t0
        U = ctx.get_result_cols([iw * wl.k for iw in range(wl.Nw)], U=True, V=False)[0]
        res[name] = (U, None, S)
        out[name + "_s"] = round(t, 4)
        out[name + "_phase_s"] = {key: round(v, 4) for key, v in ctx.timings()["seconds"].items()}
        ctx.close()
    S0, U0 = res["plain_c128"][2], res["plain_c128"][0]
    k = wl.k
    out["workload"] = (f"3D{n}: N={wl.N}, k={k}, Nw={wl.Nw}, q=1, two transient periods, "
                       f"diagonal W_q = W_f from cell volumes; shift {wl.meta['shift']:.5g} "
                       f"({wl.meta['shift_method']})")
    out["sigma1_range_plain"] = [float(S0[0].min()), float(S0[0].max())]
    for name in ("precision_c64", "precision_c64_refine"):
        S1, U1 = res[name][2], res[name][0]
        rel = np.abs(S1 - S0) / S0
        ang = []
        for iw in range(S0.shape[1]):
            u, v = U0[:, iw], U1[:, iw]
            # Chord-based angle (accurate below 1e-8, where arccos is not).
            ph = np.vdot(u, v)
            ph = ph / abs(ph) if abs(ph) > 0 else 1.0
            d = np.linalg.norm(u / np.linalg.norm(u) * ph - v / np.linalg.norm(v))
            ang.append(float(2 * np.arcsin(min(1.0, d / 2))))
        out[name] = {"speedup": round(out["plain_c128_s"] / out[name + "_s"], 3),
                     "gain_rel_err_max_j<=3": float(rel[:3].max()), "gain_rel_err_max": float(rel.max()),
                     "mode1_angle_max_rad": max(ang)}
    return out


def batch_form(count: int = 48, q: int = 0, seed: int = 2024, parity_threads: int = 0):
    """Batching form: `count` Ginzburg-Landau problems (N log-uniform in
    [200, 20000], mu0 in [0.2, 0.45], k in {6, 10, 16}, Nw in {16, 32, 64};
    grid spacing of the 500-node case, dt = T/4096, one transient period,
    q = 0, discounting where a problem is unstable) solved one context after
    another in complex128 (the plain method, 48 sequential solves) and as
    one batch in complex128 and complex64. Wall time from the first action
    to every problem's gains on the host; each batch is run once untimed
    first (autotuning, graph capture), then re-run on the same sketches.
    parity_threads > 0: also compares 6 of the problems with the C
    restatement (parity_batch), returned under "parity"."""
    import rsvdt
    from rsvdt import synth

    fam = synth.gl_family(count, seed=seed)
    T = 2 * np.pi / 0.1
    dt = T / 4096 * (1 + 1e-12)

    def params(pr, prec):
        return rsvdt.default_params(k=pr["k"], q=q, Nw=pr["Nw"], w=0.1, dt=dt, TransientLength=T,
                                    DiscFlg=int(pr["beta"] > 0), beta=pr["beta"], precision=prec, Display=0)

    sketches = [synth.complex_normal(pr["N"], pr["k"] * pr["Nw"], seed + 1 + i) for i, pr in enumerate(fam)]
    S_seq = []
    t0 = time.perf_counter()
    for pr, F in zip(fam, sketches):
        ctx = rsvdt.Context(params(pr, rsvdt.PREC_C128))
        ctx.set_operator(pr["A"])
        ctx.set_sketch(F)
        ctx.run()
        S_seq.append(ctx.get_results()[2])
        ctx.close()
    t_seq = time.perf_counter() - t0
    out = {"workload": f"{count} Ginzburg-Landau problems, N {min(p['N'] for p in fam)}..{max(p['N'] for p in fam)} "
                       f"(log-uniform), k in {{6,10,16}}, Nw in {{16,32,64}}, dt = T/4096, q = {q}, seed {seed}",
           "sum_N_k": int(sum(p["N"] * p["k"] for p in fam)), "sequential_plain_c128_s": round(t_seq, 3)}
    S_batched = {}
    for name, prec in (("batched_c128", rsvdt.PREC_C128), ("batched_c64", rsvdt.PREC_C64),
                       ("batched_c64_refine", rsvdt.PREC_C64_REFINE)):
        b = rsvdt.Batch(prec)
        for pr in fam:
            b.add(params(pr, prec), pr["A"])
        for i, F in enumerate(sketches):
            b.set_sketch(i, F)
        b.run()
        for i, F in enumerate(sketches):
            b.set_sketch(i, F)
        t0 = time.perf_counter()
        b.run()
        S_b = [b.get_results(i)[2] for i in range(len(fam))]
        t_b = time.perf_counter() - t0
        errs = [float((np.abs(Sb[:3] - Ss[:3]) / Ss[:3]).max()) for Sb, Ss in zip(S_b, S_seq)]
        err1 = [float((np.abs(Sb[0] - Ss[0]) / Ss[0]).max()) for Sb, Ss in zip(S_b, S_seq)]
        worst = int(np.argmax(errs))
        err = errs[worst]
        S_batched[name] = S_b
        if name == "batched_c64":
            S_batched["worst_c64"] = worst
        th, lanes, ms = b.tuning()
        out[name + "_s"] = round(t_b, 3)
        out[name + "_speedup_vs_sequential"] = round(t_seq / t_b, 3)
        out[name + "_gain_rel_err_max_j<=3"] = err
        out[name + "_gain1_rel_err_max"] = max(err1)
        out[name + "_worst_problem"] = {"N": fam[worst]["N"], "mu0": round(fam[worst]["mu0"], 4),
                                        "k": fam[worst]["k"], "Nw": fam[worst]["Nw"],
                                        "beta": round(fam[worst]["beta"], 4),
                                        "sigma1_max": float(S_seq[worst][0].max()),
                                        "problems_over_1e-3": int(sum(e > 1e-3 for e in errs))}
        out[name + "_tuned"] = {"threads": th, "lanes_per_row": lanes, "values_per_lane": b.values_per_lane(),
                                "ms_per_batched_step": round(ms, 4)}
        b.close()
    if parity_threads:
        out["parity"] = parity_batch(fam, sketches, lambda pr: params(pr, rsvdt.PREC_C128), S_batched,
                                     parity_threads, q)
    return out


def gl1_form(threads: int):
    """The 500-node Ginzburg-Landau configuration (k = 10, 64 frequencies
    j*0.1 for j = -32..31, dt = T/4096, one transient period): wall time of
    the whole sequence on the GPU (plain complex128) for q = 0 and q = 1,
    the leading gains' deviation from the dense resolvent (numpy, FP64), and
    the CPU baseline: the C restatement of the same run on `threads` host
    threads (q = 0)."""
    import rsvdt
    from rsvdt import synth, workloads

    out = {"workload": "GL1: N=500 Ginzburg-Landau, k=10, Nw=64, dt=T/4096, one transient period"}
    wl = workloads.make_gl1(k=10)
    F = synth.gl_sketch(500, 10, 64)
    A = wl.csr.toarray()
    om = np.array([(i if i <= 31 else i - 64) * 0.1 for i in range(64)])
    sd = np.array([np.linalg.svd(np.linalg.inv(1j * w * np.eye(500) - A), compute_uv=False)[:3] for w in om]).T
    for q, engine in ((0, rsvdt.ENGINE_AUTO), (1, rsvdt.ENGINE_AUTO), (0, rsvdt.ENGINE_STAGES)):
        ctx = rsvdt.Context(rsvdt.default_params(k=10, q=q, Nw=64, w=0.1, dt=wl.dt_in,
                                                 TransientLength=wl.transient_length, Display=0))
        ctx.set_step_engine(engine)
        ctx.set_operator(wl.csr)
        ctx.set_sketch(F)
        ctx.run()
        ctx.set_sketch(F)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.run()
        S = ctx.get_results(U=False, V=False)[2]
        t = time.perf_counter() - t0
        used = "cluster" if ctx.step_engine() == rsvdt.ENGINE_CLUSTER else "stages"
        ctx.close()
        if engine == rsvdt.ENGINE_STAGES:
            out["gpu_q0_stage_launches_s"] = round(t, 4)
            continue
        out[f"gpu_q{q}_s"] = round(t, 4)
        out["step_engine"] = used
        out[f"q{q}_gain1_vs_dense_max"] = float((np.abs(S[0] - sd[0]) / sd[0]).max())
    import oracle

    o = oracle.Oracle(wl.csr, 64, 0.1, wl.dt_in, wl.transient_length, threads=threads)
    t0 = time.perf_counter()
    o.run(F, 0)
    out["cpu_baseline_q0"] = {"s": round(time.perf_counter() - t0, 3), "cores": threads, "kind": "port",
                              "sample": "the whole q = 0 run of the C restatement, OpenMP over test vectors"}
    out["speedup_q0_vs_cpu"] = round(out["cpu_baseline_q0"]["s"] / out["gpu_q0_s"], 2)
    o.close()
    return out


def large_precision_form(n: int = 128, k: int = 16, Nw: int = 64, periods: float = 1.0, seed: int = 99,
                         full_c128: bool = False):
    """Precision form on the 3D operator at n^3 (n = 128: N = 10.5M, 14.6M
    5x5 blocks, k = 16, 64 frequencies, q = 1): variant 1 = complex64 stages
    with FP32 accumulation, FP64 DFT/QR/SVD and the FP64 sweep (the last
    adjoint action in complex128); variant 2 = plain complex128. One
    spectral block is 172 GB, so both run in capacity mode (test vectors in
    chunks, U in host memory in complex64). Wall time of the whole sequence,
    per-stage times of one chunk step, and variant 1's gain and first-mode
    (V) errors against variant 2. `periods` transient periods. Unless
    full_c128, variant 2 is timed by its chunk stage times only (its whole
    sequence takes about 24 minutes)."""
    import rsvdt
    from rsvdt import workloads

    t0 = time.perf_counter()
    wl = workloads.make_3d(n=n, k=k, Nw=Nw, periods=periods)
    build_s = time.perf_counter() - t0
    out = {"workload": f"3D{n}: N={wl.N}, {wl.meta['blocks']} 5x5 blocks, k={k}, Nw={Nw}, q=1, "
                       f"{periods:g} transient period(s), diagonal W_q = W_f; shift {wl.meta['shift']:.5g} "
                       f"({wl.meta['shift_method']})", "build_s": round(build_s, 1)}
    res = {}
    for name, prec in (("variant1_c64_fp64_sweep", rsvdt.PREC_C64_REFINE), ("variant2_plain_c128", rsvdt.PREC_C128)):
        ctx = rsvdt.Context(wl.params(precision=prec))
        ctx.set_capacity_mode(0, True)
        ctx.set_operator_bcsr(*wl.bcsr)
        ctx.set_weight(rsvdt.W_Q_SQRT, wl.weights["W_sqrt"])
        ctx.set_weight(rsvdt.W_F_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.set_weight(rsvdt.W_Q_SQRT_INV, wl.weights["W_sqrt_inv"])
        ctx.random_sketch(seed)
        g = ctx.grid()
        kc = ctx.capacity_chunk()
        # One chunk's stage times (the first kc test vectors), complex64 and
        # complex128 stage kernels as the variant uses them.
        ctx.rk4_reset(rsvdt.DIRECT)
        st = [x / 2 for x in ctx.rk4_profile(rsvdt.DIRECT, 1, 2)]
        if prec == rsvdt.PREC_C128 and not full_c128:
            out[name] = {"chunk_k": kc, "Ns": g.Ns, "Nt": g.Nt, "steps_per_action": g.Ns + g.Nt,
                         "chunk_stage_ms": [round(x, 3) for x in st],
                         "run_s_estimate": round(4 * (k // kc) * (g.Ns + g.Nt) * sum(st) / 1e3, 1)}
            ctx.close()
            continue
        fb_note = None
        if prec != rsvdt.PREC_C128:
            ctx.rk4_reset(rsvdt.DIRECT)
            t5 = [x / 2 for x in ctx.rk4_profile_ex(rsvdt.DIRECT, 1, 2)]
            fb_note = {"forcing_block_steps": ctx.forcing_block(), "forcing_block_ms_per_step": round(t5[4], 3),
                       "stage_ms_without_forcing": [round(x, 3) for x in t5[:4]]}
        ctx.random_sketch(seed)
        ctx.synchronize()
        ctx.reset_timings()
        t1 = time.perf_counter()
        ctx.run()
        ctx.synchronize()
        run_s = time.perf_counter() - t1
        S = ctx.get_results(U=False, V=False)[2]
        _, V1 = ctx.get_result_cols([iw * k for iw in range(g.Nw_eff)], U=False, V=True)
        res[name] = (np.asfortranarray(S), V1)
        out[name] = {"run_s": round(run_s, 1), "chunk_k": kc, "Ns": g.Ns, "Nt": g.Nt,
                     "steps_per_action": g.Ns + g.Nt, "chunk_stage_ms": [round(x, 3) for x in st],
                     "phase_s": {key: round(v, 2) for key, v in ctx.timings()["seconds"].items()}}
        if fb_note:
            out[name].update(fb_note)
        ctx.close()
    out["sigma1_range_variant1"] = [float(res["variant1_c64_fp64_sweep"][0][0].min()),
                                    float(res["variant1_c64_fp64_sweep"][0][0].max())]
    if "variant2_plain_c128" not in res:
        return out
    S1, V1 = res["variant1_c64_fp64_sweep"]
    S2, V2 = res["variant2_plain_c128"]
    rel = np.abs(S1 - S2) / S2
    ang = []
    for j in range(V1.shape[1]):
        u, v = V1[:, j], V2[:, j]
        ph = np.vdot(u, v)
        ph = ph / abs(ph) if abs(ph) > 0 else 1.0
        d = np.linalg.norm(u / np.linalg.norm(u) * ph - v / np.linalg.norm(v))
        ang.append(float(2 * np.arcsin(min(1.0, d / 2))))
    out["variant1_vs_variant2"] = {"gain_rel_err_max_j<=3": float(rel[:3].max()), "gain_rel_err_max": float(rel.max()),
                                   "mode1_angle_max_rad": max(ang),
                                   "speedup": round(out["variant2_plain_c128"]["run_s"] /
                                                    out["variant1_c64_fp64_sweep"]["run_s"], 3)}
    out["sigma1_range"] = [float(S2[0].min()), float(S2[0].max())]
    return out


def learned_form(n_train: int = 200, n_held: int = 12, N: int = 2000, seed: int = 77, q_max: int = 4):
    """Learned-sketch form on the Ginzburg-Landau family (N = 2000, k = 10,
    Nw = 16; mu0 in [0.2, 0.45], U in [1.5, 2.5]): the method's own forcing
    modes at n_train seeded points (complex64 batch, q = 2), r = 64 POD
    basis, network 3 -> 4 x 256 GELU -> 2 r k trained on the GPU by the
    library's kernels. At n_held held-out points, against their exact
    resolvent gains (sparse LU + Lanczos, FP64, on the host cores):

    - per point, the smallest q whose gains are within 1e-3 (max over the
      frequencies and j <= 3) from the learned sketch and from the random
      sketch (complex128 batch, q = 0 .. q_max);
    - time to gains: every point at its own q, the batch in complex64 and in
      complex128, from the learned sketch (inference time included) and
      from the random sketch;
    - the FP64 gain check of the learned q = 0 run (| |R v_j| - s_j | / s_j,
      j <= 3, one complex128 direct action on the computed forcing modes),
      the fallback test: how many points pass it, and their true errors."""
    import oracle
    import rsvdt
    import scipy.sparse as sp
    from rsvdt import learned

    t_start = time.perf_counter()
    fam = learned.Family(N=N, k=10, Nw=16)
    train = fam.points(n_train, seed=seed)
    held = fam.points(n_held, seed=seed + 1)
    # Exact gains of the held-out points (host, one core: tridiagonal LU).
    t0 = time.perf_counter()
    Sx = []
    for pt in held:
        A, beta = fam.operator(pt)
        if beta > 0:
            A = (A - beta * sp.eye(A.shape[0], format="csr")).tocsr()
        Sx.append(oracle.sparse_resolvent_svd(A, list(fam.omegas()), 3, tol=1e-12)[0])
    t_exact = time.perf_counter() - t0
    res, t_data = learned.solve_batch(fam, train, q=2, precision=rsvdt.PREC_C64, seed=seed * 10)
    ls = learned.LearnedSketch(fam, r=64, hidden=256, depth=4, seed=1)
    t0 = time.perf_counter()
    ls.fit(train, [V for (_, V, _) in res], steps=4000, batch=256, lr=1e-3)
    t_fit = time.perf_counter() - t0
    res = None
    t0 = time.perf_counter()
    sk_l = [ls.sketch(p) for p in held]
    t_inf = time.perf_counter() - t0
    sk_r = [synth_normal(fam.N, fam.k * fam.Nw, seed * 30 + i) for i in range(len(held))]
    out = {"workload": f"Ginzburg-Landau family N={N}, k=10, Nw=16, mu0 in [0.2, 0.45], U in [1.5, 2.5]; "
                       f"{n_train} training / {n_held} held-out points; exact gains: sparse LU + Lanczos",
           "tolerance": TTG_TOL, "exact_gains_s": round(t_exact, 1), "training_data_s": round(t_data, 2),
           "fit_s": round(t_fit, 2), "train_s_on_gpu": round(ls.train_seconds, 2),
           "pod_energy_r64": round(ls.pod_energy, 6), "final_loss": ls.final_loss,
           "inference_s": round(t_inf, 3), "sigma1_max": float(max(S[0].max() for S in Sx))}

    def solve(pts, sketches, qs, prec):
        """Batch of the points, point i at q = qs[i]; (seconds, results)."""
        b = rsvdt.Batch(prec)
        for pt, q in zip(pts, qs):
            A, beta = fam.operator(pt)
            b.add(fam.params(rsvdt, q, beta, prec), A)
        for i, F in enumerate(sketches):
            b.set_sketch(i, F)
        t0 = time.perf_counter()
        b.run()
        r = [b.get_results(i) for i in range(len(pts))]
        t = time.perf_counter() - t0
        b.close()
        return t, r

    solve(held, sk_r, [0] * len(held), rsvdt.PREC_C128)  # warm-up
    qstar = {}
    for name, sks in (("learned", sk_l), ("random", sk_r)):
        qs, scan = [None] * len(held), []
        for q in range(q_max + 1):
            _, r = solve(held, sks, [q] * len(held), rsvdt.PREC_C128)
            errs = [gain_rel_err(S, x) for (_, _, S), x in zip(r, Sx)]
            for i, e in enumerate(errs):
                if qs[i] is None and e <= TTG_TOL:
                    qs[i] = q
            e1 = [gain_rel_err(S, x, 1) for (_, _, S), x in zip(r, Sx)]
            scan.append({"q": q, "err_median": float(f"{np.median(errs):.3e}"),
                         "err_max": float(f"{max(errs):.3e}"), "met": int(sum(e <= TTG_TOL for e in errs)),
                         "err_j1_median": float(f"{np.median(e1):.3e}"),
                         "met_j1": int(sum(e <= TTG_TOL for e in e1))})
            if name == "learned":
                # The fallback gate on the learned run at this q: points whose
                # FP64 gain check passes keep the result, the others fall back.
                checks = [learned.gain_check(fam, p, rr, jmax=3) for p, rr in zip(held, r)]
                passed = [i for i, c in enumerate(checks) if c <= TTG_TOL]
                gates = out.setdefault("gate_learned", [])
                gates.append({
                    "q": q, "check_median": float(f"{np.median(checks):.3e}"), "passed": len(passed),
                    "fell_back": len(held) - len(passed),
                    "passed_within_tolerance": int(sum(errs[i] <= TTG_TOL for i in passed)),
                    "within_tolerance_but_failed": int(sum(errs[i] <= TTG_TOL for i in range(len(held))
                                                           if i not in passed))})
            print(f"learned {name} {scan[-1]}", file=sys.stderr, flush=True)
            if all(v is not None for v in qs):
                break
        qstar[name] = qs
        out[f"{name}_q_scan"] = scan
        out[f"{name}_q_per_point"] = qs
    both = [i for i in range(len(held)) if qstar["learned"][i] is not None and qstar["random"][i] is not None]
    out["points_timed"] = len(both)
    if both:
        def sub(lst):
            return [lst[i] for i in both]

        for name, sks in (("learned", sk_l), ("random", sk_r)):
            for pname, prec in (("c64", rsvdt.PREC_C64), ("c128", rsvdt.PREC_C128)):
                t, r = solve(sub(held), sub(sks), sub(qstar[name]), prec)
                errs = [gain_rel_err(S, Sx[i]) for (_, _, S), i in zip(r, both)]
                if name == "learned":
                    t += t_inf * len(both) / len(held)
                out[f"{name}_{pname}"] = {"s": round(t, 3), "q_sum": int(sum(sub(qstar[name]))),
                                          "err_max_j<=3": float(f"{max(errs):.3e}"),
                                          "over_tolerance": int(sum(e > TTG_TOL for e in errs))}
        out["ratio_random_over_learned_c64"] = round(out["random_c64"]["s"] / out["learned_c64"]["s"], 3)
        out["ratio_random_c128_over_learned_c64"] = round(out["random_c128"]["s"] / out["learned_c64"]["s"], 3)
    out["wall_s"] = round(time.perf_counter() - t_start, 1)
    return out


def synth_normal(rows, cols, seed):
    from rsvdt import synth
    return synth.complex_normal(rows, cols, seed)


def learned3d_form(n: int = 48, n_train: int = 24, n_held: int = 8, seed: int = 91):
    """Learned-sketch form on the 3D half of the family: the five-field
    operator at n^3 (n = 48: N = 552,960) over Re in [500, 2000] and a
    uniform reaction term mu0 in [0.2, 0.45], k = 4, Nw = 16. Training data:
    the method's own forcing modes (complex64, q = 1) at n_train seeded
    points; POD basis r = 64 by the method of snapshots; network 3 -> 4 x 256
    GELU -> 2 r k trained on the GPU. At n_held held-out points: q = 0 from
    the learned sketch against q = 0, 1, 2 from random sketches, all in the
    refinement form, gains against a q = 3 solve."""
    import rsvdt
    from rsvdt import learned

    fam = learned.Family3D(n=n, k=4, Nw=16)
    t0 = time.perf_counter()
    _ = fam.shift  # the family's spectral shift (RK4 growth rate at the least stable corner)
    t_shift = time.perf_counter() - t0
    train = fam.points(n_train, seed=seed)
    held = fam.points(n_held, seed=seed + 1)
    res, t_data = learned.solve_batch(fam, train, q=1, precision=rsvdt.PREC_C64, seed=seed * 10)
    ls = learned.LearnedSketch(fam, r=64, hidden=256, depth=4, seed=1)
    t0 = time.perf_counter()
    ls.fit(train, [V for (_, V, _) in res], steps=3000, batch=128, lr=1e-3)
    t_fit = time.perf_counter() - t0
    res = None
    prec = rsvdt.PREC_C64_REFINE
    ref, t_ref = learned.solve_batch(fam, held, q=3, precision=prec, seed=seed * 20)
    out = {"workload": f"3D family {n}^3 (N={fam.N}), Re in [500, 2000], mu0 in [0.2, 0.45], k=4, Nw=16; "
                       f"{n_train} training / {n_held} held-out points", "family_shift": round(fam.shift, 6),
           "shift_s": round(t_shift, 2), "training_data_s": round(t_data, 2), "fit_s": round(t_fit, 2),
           "train_s_on_gpu": round(ls.train_seconds, 2), "pod_energy_r64": round(ls.pod_energy, 6),
           "final_loss": ls.final_loss, "reference_q3_s": round(t_ref, 2)}
    sk = [ls.sketch(p) for p in held]
    runs = {"learned_q0": (0, sk)}
    for q in (0, 1, 2):
        runs[f"random_q{q}"] = (q, None)
    for name, (q, s_) in runs.items():
        r, t = learned.solve_batch(fam, held, q=q, precision=prec, sketches=s_, seed=seed * 30)
        e1, e3 = learned.gain_errors(r, ref)
        out[name] = {"solve_s": round(t, 2), "gain1_err_median": float(np.median(e1)), "gain1_err_max": float(e1.max()),
                     "gain_j<=3_err_median": float(np.median(e3)), "within_1e-3": int((e3 <= 1e-3).sum())}
    return out


def summarize(out):
    """The headline figures of the side experiments in a few scalars (kept
    last on the JSON line)."""
    sm = {}
    ttg = out.get("time_to_gains_1e-3") or {}
    for key, d in ttg.items():
        if not d:
            continue
        sm[f"ttg_{key}_ratio"] = d.get("ratio_plain_over_chosen")
        sm[f"ttg_{key}_chosen"] = d.get("chosen")
        for form in ("plain_c128", d.get("chosen")):
            b = (d.get(form) or {}).get("best") if form else None
            if b:
                sm[f"ttg_{key}_{form}_s"] = b["s"]
                sm[f"ttg_{key}_{form}_q"] = b["q"]
    ratios = [(d.get("ratio_plain_over_chosen"), key) for key, d in ttg.items() if d and d.get("ratio_plain_over_chosen")]
    if ratios:
        sm["ttg_best_ratio"], sm["ttg_best_workload"] = max(ratios)
    lrn = out.get("learned_sketch") or {}
    for name in ("learned", "random"):
        scan = lrn.get(f"{name}_q_scan") or []
        if scan:
            sm[f"learned_{name}_q0_err_j1_median"] = scan[0].get("err_j1_median")
    if lrn.get("ratio_random_over_learned_c64") is not None:
        sm["learned_ttg_ratio_random_over_learned_c64"] = lrn["ratio_random_over_learned_c64"]
    c64 = out.get("precision_form_c64") or {}
    sm["c64_ms_per_step"] = c64.get("ms_per_step")
    sm["c64_step_frac"] = c64.get("frac")
    par = out.get("parity") or {}
    for key, d in par.items():
        sm[f"parity_{key}_pass"] = d.get("pass", d.get("pass_c128"))
    eqq = out.get("equal_q_speedup") or {}
    if eqq.get("precision_c64"):
        sm["equal_q_3d64_c64_speedup"] = eqq["precision_c64"]["speedup"]
    return sm


def step_config(wl, dt, Ns, R, step_bytes, world):
    """The benchmark step's `config` (both arms)."""
    return {"workload": f"{wl.name}: one forced RK4 step over k={wl.k} test vectors of the five-field "
                        f"{wl.meta['grid']} block operator (5x5 blocks), Nw={wl.Nw}, "
                        "complex128",
            "N": wl.N, "nnz": wl.meta["nnz"], "k": wl.k, "Nw": wl.Nw, "dt": dt, "Ns": Ns, "ResRatio": R,
            "step_bytes": step_bytes,
            "l2": (f"{step_bytes / 1e9:.1f} GB moved per step >> L2 (129 MB), no flush" if step_bytes > 1e9 else
                   f"{step_bytes / 1e6:.0f} MB per step: small case, partly L2-resident"),
            "parallelism": f"replicas x{world}",
            "spectral_shift": round(wl.meta["shift"], 6), "shift_method": wl.meta["shift_method"]}


def run_reference(args):
    """CPU arm: the reference algorithm on the host cores (oracle port)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from rsvdt import workloads
    # The recorded shift builds the same operator as the GPU arm without a
    # GPU; for a grid with no recorded shift the host-only estimate stands
    # in (the per-step work does not depend on the diagonal shift).
    known = (args.n, 7) in workloads.RECORDED_GROWTH_RATE
    wl = workloads.make_3d(n=args.n, shift="recorded" if known else "local")
    import oracle
    dt, Ns, Nt, R = oracle.setup_grid(wl.w, wl.Nw, wl.dt_in, wl.transient_length)
    Fk = np.asfortranarray(np.random.default_rng(1).standard_normal((wl.N, wl.Nw)) + 0j)
    threads = os.cpu_count() or 1
    # W untimed steps, then K timed steps of all k test vectors (0.45 s per
    # 3D64 step on 16 Grace cores: the default run takes about half a minute).
    t = cpu_baseline(wl, None, Fk, args.steps, threads, warmup=args.warmup)
    b = wl.step_bytes(R)
    val = b["step"] / t / 1e9
    out = {"impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "GB/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
           "config": step_config(wl, dt, Ns, R, b["step"], args.gpus),
           "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} steps x {wl.k} test vectors, row loops on "
                                      f"{threads} threads; C restatement of SourceCode/TSRK4.c (PETSc/SLEPc/MPI "
                                      "absent)"},
           "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def profile_case(n: int):
    """The complex64 forcing-block step of the five-field operator on an n^3
    grid, launch for launch the same every run, so that a profiler can pick
    kernels by position: 3 warm-up steps (the forcing block of the first 16
    steps, then 4 stage launches per step), then rsvdt_rk4_profile_ex over 2
    steps (one forcing block for both, then 8 stage launches). Prints the
    event times of the profiled steps."""
    import rsvdt
    from rsvdt import workloads

    wl = workloads.make_3d(n=n)
    ctx = rsvdt.Context(wl.params(precision=rsvdt.PREC_C64))
    ctx.set_operator_bcsr(*wl.bcsr)
    ctx.random_sketch(1234)
    ctx.rk4_reset(rsvdt.DIRECT)
    ctx.rk4_advance(rsvdt.DIRECT, 1, 3)
    ctx.synchronize()
    t = ctx.rk4_profile_ex(rsvdt.DIRECT, 4, 2)
    print(json.dumps({"profile_case": f"3D{n} complex64 forcing-block step", "N": wl.N, "k": wl.k, "Nw": wl.Nw,
                      "forcing_block": ctx.forcing_block(), "stage_ms_2_steps": [round(x, 4) for x in t[:4]],
                      "forcing_block_ms": round(t[4], 4)}))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=64, help="3D grid size (64 for the benchmark)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-ttg", action="store_true", help="skip the time-to-gains and equal-q solves")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching-form comparison")
    ap.add_argument("--no-gl1", action="store_true", help="skip the 500-node Ginzburg-Landau runs")
    ap.add_argument("--no-parity", action="store_true", help="skip the at-size parity checks against the oracle")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-sketch experiment")
    ap.add_argument("--equal-q", action="store_true",
                    help="also time the whole 3D64 solve at q = 1 in the three forms (equal work, no exact gains)")
    ap.add_argument("--learned3d", action="store_true", help="run the 3D learned-sketch experiment (a few minutes)")
    ap.add_argument("--ttg-n", type=int, default=64, help="grid of the time-to-gains solves")
    ap.add_argument("--large-n", type=int, default=0,
                    help="run the precision form on the n^3 operator in capacity mode (128: the 10.5M-row case)")
    ap.add_argument("--large-periods", type=float, default=1.0, help="transient periods of the --large-n runs")
    ap.add_argument("--large-full", action="store_true", help="run the whole complex128 sequence in --large-n too")
    ap.add_argument("--profile-case", action="store_true",
                    help="only the complex64 forcing-block step on the --n grid, for a profiler: 3 warm-up steps "
                         "(13 launches: one forcing block, 12 stages), then one forcing block for 2 steps and "
                         "their 8 stages")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_case:
        profile_case(args.n)
        return

    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import rsvdt
    from rsvdt import replicas, workloads

    wl = workloads.make_3d(n=args.n)
    ctx = rsvdt.Context(wl.params(precision=rsvdt.PREC_C128))
    ctx.set_operator_bcsr(*wl.bcsr)
    g = ctx.grid()
    ctx.random_sketch(replicas.rank_seed(1234, rank))
    b = wl.step_bytes(g.ResRatio)
    fl = wl.step_flops()
    def timed(c, i0, n):
        """CUDA events on the context's own stream around n device steps."""
        stream = torch.cuda.ExternalStream(c.stream())
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        c.rk4_advance(rsvdt.DIRECT, i0, n)
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e)

    # Everything from here to the end of the complex64 step is inside one NVTX
    # range, so that a profiler can keep to it (ncu --nvtx --nvtx-include
    # "rsvdt bench step/").
    torch.cuda.nvtx.range_push("rsvdt bench step")
    ctx.rk4_reset(rsvdt.DIRECT)
    ctx.rk4_advance(rsvdt.DIRECT, 1, args.warmup)
    ctx.synchronize()
    launches0 = ctx.launch_count()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(1.5)  # let nvidia-smi start sampling before the timed region
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms = timed(ctx, 1 + args.warmup, args.steps)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    ms = replicas.max_over_ranks(ms, dist, device="cuda")
    ms_step = ms / args.steps
    value = replicas.whole_job_rate(b["step"], ms_step, world) / 1e9

    # Dominant kernel: stage 1 timed launch by launch.
    nprof = 5
    st_ms = ctx.rk4_profile(rsvdt.DIRECT, 1 + args.warmup + args.steps, nprof)
    st_ms = [x / nprof for x in st_ms]
    hbm, peak_kind = peaks()
    ach = b["stage1"] / (st_ms[0] * 1e-3) / 1e9
    fp64_peak = fp64_peak_tflops(torch)
    ach_fp64 = fl["stage1"] / (st_ms[0] * 1e-3) / 1e12
    step_fp64 = fl["step"] / (ms_step * 1e-3) / 1e12

    # e2e through the C ABI with host (pinned) state buffers: every call
    # copies y and F3 in and out and restages the forcing block.
    e2e_steps = 3
    yh = torch.zeros((wl.k, wl.N), dtype=torch.complex128, pin_memory=True)
    fh = torch.zeros((wl.k, wl.N), dtype=torch.complex128, pin_memory=True)
    ynp, fnp = yh.numpy().T, fh.numpy().T  # N x k, Fortran order views
    ctx.rk4_steps(rsvdt.DIRECT, 1, 1, ynp, fnp)
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        ctx.rk4_steps(rsvdt.DIRECT, 2 + s, 1, ynp, fnp)
    e2e_t = (time.perf_counter() - t0) / e2e_steps
    io_bytes = 2 * wl.N * wl.k * 16

    # Precision form (complex64 stages, FP32 accumulation) on the same shape.
    ctx64 = rsvdt.Context(wl.params(precision=rsvdt.PREC_C64))
    ctx64.set_operator_bcsr(*wl.bcsr)
    ctx64.random_sketch(replicas.rank_seed(1234, rank))
    ctx64.rk4_reset(rsvdt.DIRECT)
    ctx64.rk4_advance(rsvdt.DIRECT, 1, 3)
    ms64 = timed(ctx64, 4, args.steps) / args.steps
    fb64 = ctx64.forcing_block()
    b64 = wl.step_bytes(g.ResRatio, s_c=8, forcing_block=fb64)
    # Per-kernel times over 2 forcing blocks (32 steps), per step.
    nprof64 = 2 * max(fb64, 1) if fb64 else nprof
    st64 = [x / nprof64 for x in ctx64.rk4_profile_ex(rsvdt.DIRECT, 4 + args.steps, nprof64)]
    # The same step with stage 1 synthesising every step's forcing (the
    # form before the forcing block), for comparison.
    ctx64.set_forcing_block(0)
    ctx64.rk4_advance(rsvdt.DIRECT, 4 + args.steps + nprof64, 3)
    ms64_nofb = timed(ctx64, 7 + args.steps + nprof64, args.steps) / args.steps
    ctx64.set_forcing_block(-1)
    torch.cuda.nvtx.range_pop()

    threads = os.cpu_count() or 1
    parity = {}
    if rank == 0 and not args.no_parity:
        parity["steps_" + wl.name] = parity_steps(wl, ctx, ctx64, threads)
    # Both step contexts are done: their device memory (about 25 GB) goes
    # back before the side experiments (the 128^3 case needs all of it).
    ctx64.close()
    ctx.close()
    eqq = None
    if rank == 0 and args.equal_q:
        eqq = equal_q_speedup(args.ttg_n)
    ttg = {}
    if rank == 0 and not args.no_ttg:
        ttg["gl1"] = ttg_gl1()
        if os.path.exists(os.path.join(ROOT, "tests", "golden", "exact_gains_op3d24.npz")):
            ttg["3d24"] = ttg_3d24()
        if not args.no_batch:
            ttg["batch"] = ttg_batch()
    batching = None
    if rank == 0 and not args.no_batch:
        batching = batch_form(parity_threads=0 if args.no_parity else threads)
        if "parity" in batching:
            parity["batch"] = batching.pop("parity")
    learned_res = None
    if rank == 0 and not args.no_learned:
        learned_res = learned_form()
    learned3d = None
    if rank == 0 and args.learned3d:
        learned3d = learned3d_form()
    gl1 = None
    if rank == 0 and not args.no_gl1:
        gl1 = gl1_form(min(os.cpu_count() or 1, 10))
    large = None
    if rank == 0 and args.large_n:
        torch.cuda.empty_cache()  # the DGEMM probe's cached blocks
        large = large_precision_form(n=args.large_n, periods=args.large_periods, full_c128=args.large_full)

    cpu = None
    if rank == 0 and not args.no_cpu:
        Fk = np.asfortranarray(np.random.default_rng(1).standard_normal((wl.N, wl.Nw)) + 0j)
        t_cpu = cpu_baseline(wl, g, Fk, 2, threads)
        cpu = {"value": round(b["step"] / t_cpu / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"2 steps x {wl.k} test vectors of the same 3D64 step, row loops on {threads} threads "
                         f"({t_cpu:.2f} s/step); C restatement of SourceCode/TSRK4.c"}

    def gbs(nbytes, ms):
        return nbytes / (ms * 1e-3) / 1e9 if ms > 0 else 0.0

    c64 = {"ms_per_step": round(ms64, 4), "forcing_block_steps": fb64,
           "value": round(gbs(b64["step"], ms64), 3), "unit": "GB/s", "frac": round(gbs(b64["step"], ms64) / hbm, 4),
           "step_bytes": b64["step"],
           "stage_ms": [round(x, 4) for x in st64[:4]], "forcing_block_ms": round(st64[4], 4),
           "kernels": "k_forcing_block<32,pair> + k_bstage<z64,10,2,1..4,FB> (lane groups per 5x5 block row)",
           "forcing_gbs": round(gbs(b64["forcing"], st64[4]), 2),
           "forcing_frac": round(gbs(b64["forcing"], st64[4]) / hbm, 4),
           "stage1_gbs": round(gbs(b64["stage1"], st64[0]), 2),
           "stage1_frac": round(gbs(b64["stage1"], st64[0]) / hbm, 4),
           "stage2_gbs": round(gbs(b64["stage234"], st64[1]), 2),
           "stage2_frac": round(gbs(b64["stage234"], st64[1]) / hbm, 4),
           "stage4_gbs": round(gbs(b64["stage4"], st64[3]), 2),
           "ms_per_step_without_forcing_block": round(ms64_nofb, 4),
           "speedup_vs_c128": round(ms_step / ms64, 3)}

    if rank == 0:
        out = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded operator and sketch)",
            "config": step_config(wl, g.dt, g.Ns, g.ResRatio, b["step"], world),
            "roofline": {"bound": "hbm", "kernel": "k_rstage<z128,10,1> (block-row SpMM + forcing synthesis)",
                         "achieved": round(ach, 2), "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
                         "peak_kind": peak_kind,
                         # DRAM bytes of one launch: a one-pass ncu capture of this kernel on
                         # the 64^3 operator (7.990 GB read + 0.832 GB written), scaled by N
                         # for other grids.
                         "traffic": round(8.8219e9 * wl.N / 1310720),
                         "traffic_source": "ncu dram__bytes_read+write of k_rstage<z128,10,1> at 3D64, one launch",
                         "bytes_per_launch": b["stage1"], "ms_per_launch": round(st_ms[0], 4),
                         "fp64_frac": round(ach_fp64 / fp64_peak, 4),
                         # The precision form's step (complex64 stages, forcing block) on the
                         # same operator, against the same HBM peak.
                         "c64_ms_per_step": c64["ms_per_step"], "c64_step_frac": c64["frac"],
                         "c64_forcing_frac": c64["forcing_frac"], "c64_stage1_frac": c64["stage1_frac"],
                         "c64_stage2_frac": c64["stage2_frac"],
                         "fp64": {"achieved_tflops": round(ach_fp64, 4), "peak_tflops": round(fp64_peak, 4),
                                  "frac": round(ach_fp64 / fp64_peak, 4),
                                  "note": "plain complex128 form is FP64-bound on GB300; peak = cuBLAS DGEMM"}},
            "stage_ms": [round(x, 4) for x in st_ms],
            "step_fp64_tflops": round(step_fp64, 4),
            "precision_form_c64": c64,
            "clocks": clk,
            "gpu_launches": int(launches),
            "e2e": {"value": round(b["step"] / e2e_t / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": io_bytes,
                    "d2h_bytes_per_step": io_bytes, "ms_per_step": round(e2e_t * 1e3, 3),
                    "api": "rsvdt_rk4_steps (host y, F3 in pinned memory)"},
            "cpu_baseline": cpu,
            "equal_q_speedup": eqq,
            "time_to_gains_1e-3": ttg or None,
            "batching": batching,
            "learned_sketch": learned_res,
            "learned_sketch_3d": learned3d,
            "gl1": gl1,
            "precision_form_large": large,
            "parity": parity or None,
        }
        out["summary"] = summarize(out)
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
