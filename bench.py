#!/usr/bin/env python
"""Benchmark of the GB300 electrostatic PIC step (push + deposit + CG solve).

One "step" = PIC::time_step (PIC.cpp:245-267) over the whole particle list:
fixed-point charge -> field solve -> E per tet -> fused push/walk/deposit.

Default workload (N=1, the mixed-precision target configuration): 128^3
Kuhn-split unit cube (12,582,912 tets, 2,146,689 nodes), 128M electrons
(q/m = -1) in two counter-streaming Maxwellian beams (drift +-0.2 along x,
v_th = 0.02, equal halves) over a fixed uniform neutralising background,
absorbing walls, dt = 0.005, cell sort every 10 steps, mixed precision
(FP32 push/gather, int64 fixed-point deposit, FP32 multigrid-preconditioned
CG inside FP64 refinement to 1e-10).  Particle state (128M x 28 B = 3.8 GB)
is far larger than L2, so no L2 flush is needed between steps.

Printed JSON line (rank 0): metric/value in particle-steps/s of the mixed
form with its state resident in HBM; the mixed form with the plain inner CG
(the same solver family as the FP64 form) and the plain FP64 form on the
same fill, each with its ratio; per-phase device times; the roofline of the
dominant kernel and of the FP64 form's solver; the error of the mixed form
against the FP64 form over the configuration's 100 steps (phi per step, E,
particle positions and velocities matched by particle id, survivor counts,
exact charge); the CPU baseline (the CPU restatement of the reference's
algorithm, timed on this host's cores); the end-to-end number through the C
ABI with host buffers; clocks sampled during the timed region; the 256-run
ensemble (p50/p99 step latency) and the 48^3 two-species configuration as
extra keys.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload large|standard|two-stream|small|ensemble|serving]

Ensemble: 256 independent runs (n^3 Kuhn meshes, n uniform in [8,32];
particle counts log-uniform in [1e4, 2e6]; v_th uniform in [0.02, 0.1]; seeds
1000+i; 100 steps each) advanced together by the batch engine, with the
solver block size and sort interval picked by a short autotuning pass.
Serving: Poisson arrivals (20 runs/s for --serve-seconds, default 60) of the
same run mix, 5% of them 64^3 meshes with 16M particles, 50-500 steps each,
admitted against a 150 GB device budget (see run_serving).
"""
import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "particle-steps/s (push+deposit+CG) mixed vs FP64 plain; ensemble p50/p99 ms"
UNIT = "particle-steps/s"

WORKLOADS = {
    # 48^3 jittered Kuhn, two species (electrons + ions), mixed precision
    "standard": dict(name="kuhn48-jitter0.2-e8M-ion8M-mixed", n_side=48, jitter=0.2, dt=0.01, sort_interval=10,
                     steps=200,
                     species=[dict(q=-1.0, m=1.0, n=8 << 20, vth=0.05, drift=(0, 0, 0), seed=1),
                              dict(q=1.0, m=100.0, n=8 << 20, vth=0.005, drift=(0, 0, 0), seed=2)],
                     rho_background=0.0),
    # 128^3 Kuhn, 128M electrons in two counter-streaming beams over a fixed background
    "large": dict(name="kuhn128-2beam-e128M-mixed", n_side=128, jitter=0.0, dt=0.005, sort_interval=10, steps=100,
                  species=[dict(q=-1.0, m=1.0, n=64 << 20, vth=0.02, drift=(0.2, 0, 0), seed=1),
                           dict(q=-1.0, m=1.0, n=64 << 20, vth=0.02, drift=(-0.2, 0, 0), seed=2, same=0)],
                  rho_background=1.0),
    # the reference's two-stream problem (main.cpp:89-106) at GPU scale: 48^3
    # Kuhn mesh of [-1,1]^3 periodic in x, its ParticleFill set-up per tet
    # (two electron beams v_x = +-0.5 (1 - 0.05 sin(pi x)), H+ at rest),
    # density 2/3 pi^2, absorbing y/z walls, mixed precision
    "two-stream": dict(name="kuhn48-periodic-twostream-e8M-H8M-mixed", n_side=48, jitter=0.0, dt=0.01,
                       sort_interval=10, steps=100, periodic=1, lo=-1.0, hi=1.0, rho_background=0.0,
                       ref_fills=[dict(nppe=6, type=0, density=np.pi ** 2 / 3.0, vel=(0.5, 0.0, 0.0), temp=-0.05),
                                  dict(nppe=6, type=0, density=np.pi ** 2 / 3.0, vel=(-0.5, 0.0, 0.0), temp=-0.05),
                                  dict(nppe=12, type=2, density=2.0 * np.pi ** 2 / 3.0, vel=(0.0, 0.0, 0.0),
                                       temp=0.0)],
                       species=[dict(q=-1.0, m=1.0, n=12 * 6 * 48 ** 3), dict(q=1.0, m=1837.0, n=12 * 6 * 48 ** 3)]),
    # 10^3 Kuhn, 1e5 electrons over a uniform background, plain FP64
    "small": dict(name="kuhn10-e100k-plain", n_side=10, jitter=0.0, dt=0.01, sort_interval=0, steps=100,
                  species=[dict(q=-1.0, m=1.0, n=100000, vth=0.05, drift=(0, 0, 0), seed=1)],
                  rho_background=1.0),
}


def _pkg():
    name = "minipic_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "minipic-crossroads_gb300", "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def total_particles(w):
    return sum(s["n"] for s in w["species"])


# CG initial guess of the single-run workloads (both forms): 2 = linear
# extrapolation from the last two solutions, 1 = the previous solution
WARM_START = 2
# inner solver of the mixed form: "cg" plain FP32 CG, "mg" CG preconditioned
# by the geometric multigrid V-cycle (falls back to "cg" on grids too small to coarsen)
MIXED_SOLVER = "mg"


def make_ctx(mpg, w, precision, device=0, seed_offset=0, solver=None, track_ids=0):
    """One run of workload w in the given form; solver "mg" or "cg" picks the
    mixed form's inner solver (default MIXED_SOLVER)."""
    ctx = mpg.Ctx(device)
    ctx.mesh(w["n_side"], split=mpg.SPLIT_KUHN6, lo=w.get("lo", 0.0), hi=w.get("hi", 1.0),
             mapping=mpg.MAP_JITTER if w["jitter"] else mpg.MAP_NONE, jitter=w["jitter"], seed=7,
             periodic=w.get("periodic", 0))
    solver = solver or MIXED_SOLVER
    kind = mpg.SOLVER_CG_MG if precision == mpg.MIXED and solver == "mg" else mpg.SOLVER_CG
    ctx.configure(precision=precision, deposit=mpg.DEPOSIT_LINEAR, solver=kind, tol=1e-10, max_iter=5000,
                  warm_start=WARM_START, kill_on_wall=1, max_crossings=1000,
                  sort_interval=w["sort_interval"] if precision == mpg.MIXED else 0,
                  rho_background=w["rho_background"], track_ids=track_ids)
    if "ref_fills" in w:
        # the reference's per-tet fill (particle_fill.hpp:129-164); species
        # 0 = e- (-1, 1) and 2 = H+ (1, 1837) as in particle_type.hpp
        ctx.reserve(total_particles(w))
        ctx.species(0, -1.0, 1.0)
        ctx.species(2, 1.0, 1837.0)
        for f in w["ref_fills"]:
            ctx.fill_ref(f["nppe"], f["type"], f["density"], vel=f["vel"], temp=f["temp"])
        return ctx
    # weights: each species carries a total charge of magnitude 1 in the unit cube
    by_charge = {}
    for s in w["species"]:
        by_charge[s["q"]] = by_charge.get(s["q"], 0) + s["n"]
    ctx.reserve(total_particles(w))
    for i, s in enumerate(w["species"]):
        sp = s.get("same", i)
        ctx.species(sp, s["q"], s["m"])
        ctx.fill_uniform(s["n"], s["seed"] + 1000 * seed_offset, sp, 1.0 / by_charge[s["q"]], drift=s["drift"],
                         vth=s["vth"])
    return ctx


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def uses_mg(w):
    return MIXED_SOLVER == "mg" and bool(mg_levels(w["n_side"], w.get("periodic", 0)))


def mg_levels(n_side, periodic=0, dense_max=1500):
    """(x, y/z) node extents of the multigrid levels: halve (g -> g // 2 + 1)
    while the interior has more than dense_max unknowns (the host hierarchy's
    rule; a periodic x axis holds n planes and halves while even and the
    result stays >= 4)."""
    def interior(x, g):
        return (x if periodic else x - 2) * (g - 2) ** 2
    lev = [(n_side if periodic else n_side + 1, n_side + 1)]
    while len(lev) < 8 and interior(*lev[-1]) > dense_max:
        x, g = lev[-1]
        okx = (x % 2 == 0 and x // 2 >= 4) if periodic else x >= 5
        if not okx or g < 5:
            break
        lev.append((x // 2 if periodic else x // 2 + 1, g // 2 + 1))
    if len(lev) < 2 or interior(*lev[-1]) > dense_max:
        return []
    return [(x, g, interior(x, g)) for x, g in lev]


def mg_iter_bytes(n_side, N, coef, periodic=0):
    """Algorithmic bytes of one multigrid-preconditioned inner iteration.

    Fine level (two Jacobi sweeps on each side), per row: fused update +
    first pre-smoothing reads p, u, s, w, z, r, D^-1 and writes p, s, z, r, t1
    (44 B); the second reads t1, D^-1 and writes t (12 B); restriction reads t
    (4 B); the three ascending passes read D^-1, r, t1 / e / e2 and write e /
    e2 / u (48 B); w = A u and the four dots read u, r, s, p and write w (20 B);
    five stencil passes read the FP32 coefficients (5 coef).
    Coarse levels, per row: 27 FP32 coefficients in two passes plus about 80 B
    of vectors.  Coarsest level: its dense inverse (m^2 FP32)."""
    lev = mg_levels(n_side, periodic)
    b = (44 + 12 + 4 + 48 + 20 + 5 * coef) * N
    for x, g, _ in lev[1:-1]:
        b += (2 * 27 * 4 + 80) * x * g * g
    x, g, m = lev[-1]
    return b + 4 * m * m + 40 * x * g * g


def kuhn_structured(w):
    """The library walks an unjittered, non-periodic Kuhn cube through its
    6-type table (mpg_kernels.h KuhnTable)."""
    return w["jitter"] == 0 and not w.get("periodic", 0) and "ref_fills" not in w and w["n_side"] >= 3


def phase_bytes(w, ctx, stats, steps, mpg):
    """Algorithmic bytes per launch of each phase of the mixed step.

    Solver (structured diagonal operator, nd = 15 diagonals on the Kuhn grid),
    plain inner CG: per inner iteration 4*nd bytes of FP32 coefficients per row (none with the
    constant stencil of an unjittered mesh) + 16 B of vector reads (r, q, p, z)
    + 16 B of vector writes; per refinement sweep (about 3 per solve) the FP64
    residual reads 8*nd + 16 B and writes 8 B per row, the restart 20 B.
    Multigrid-preconditioned inner CG: mg_iter_bytes per inner iteration.
    """
    T, N = ctx.T, ctx.N
    P = total_particles(w)
    nd = 15
    iters = stats.solver_iters / max(steps, 1)
    coef = 0 if w["jitter"] == 0 else 4 * nd
    cg_iter = (coef + 32) * N
    sweep = (8 * nd + 24 + 20) * N
    if uses_mg(w):
        cg_iter = mg_iter_bytes(w["n_side"], N, coef, w.get("periodic", 0))
    if kuhn_structured(w):
        # uniform Kuhn mesh: the walk tables are a 6-type table: per tet E
        # (16 B) and the charge-slot indices (16 B) are read and its four
        # 8-byte charge slots written; the E pass reads the node ids (16 B) and
        # writes E (16 B) per tet
        move_tet, efield_tet = 16 + 16 + 32, 16 + 16
        dep = N * (4 + 8 + 1 + 8) + T * 32
    else:
        # per tet the walk record (48 B), the neighbour table (16 B) and the
        # charge-slot indices (16 B) read once and its four 8-byte charge
        # slots written once; the E pass reads node ids and the record and
        # writes E; the conversion reads slot offsets, background, flag, rhs
        # per node and the 4T slots
        move_tet, efield_tet, dep = 48 + 16 + 16 + 32, 16 + 48 + 12, N * (4 + 8 + 1 + 8) + T * 32
    return {
        # 28 B read + 28 B write per particle
        "move": P * 56 + T * move_tet,
        "solve": iters * cg_iter + 3 * sweep,
        "efield": T * efield_tet + N * 8,
        "deposit": dep,
        "cg_iter_bytes": cg_iter, "iters_per_step": iters,
    }


def read_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from a committed ncu
    summary (profiles/<kernel>*.txt with a matching "workload:" line), if any."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if not fn.startswith(kernel) or not fn.endswith(".txt"):
            continue
        wl, val = None, None
        with open(os.path.join(pdir, fn)) as f:
            for line in f:
                if line.startswith("workload:"):
                    wl = line.split(":", 1)[1].split()[0]
                elif line.startswith("dram_bytes_per_launch_full_workload:"):
                    try:
                        val = float(line.split(":", 1)[1].split()[0])
                    except ValueError:
                        val = None
        if wl == workload and val is not None:
            return val
    return None


# ---------------------------------------------------------------------------
# ensemble and serving
def ensemble_trace(count=256, seed=2026):
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    runs = []
    for i in range(count):
        n = int(rng.integers(8, 33))
        P = int(round(math.exp(rng.uniform(math.log(1e4), math.log(2e6)))))
        runs.append(dict(n_side=n, n_particles=P, seed=1000 + i, vth=float(rng.uniform(0.02, 0.1)), steps=100))
    return runs


def serving_trace(seconds=60.0, rate=20.0, seed=2027):
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    t, runs, i = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        if rng.uniform() < 0.05:
            n, P = 64, 16 << 20
        else:
            n = int(rng.integers(8, 33))
            P = int(round(math.exp(rng.uniform(math.log(1e4), math.log(2e6)))))
        runs.append(dict(arrival=t, n_side=n, n_particles=P, seed=5000 + i, vth=float(rng.uniform(0.02, 0.1)),
                         steps=int(rng.integers(50, 501))))
        i += 1
    return runs


def batch_admit(bt, r, steps=None):
    return bt.admit(r["n_side"], r["n_particles"], r["seed"], vth=r["vth"], dt=0.01, tol=1e-10, max_iter=5000,
                    steps=r["steps"] if steps is None else steps, allow=(-3,))


def autotune(mpg, runs, device=0):
    """Pick the batch engine's block size, step form (one persistent launch
    per step or one launch per phase) and sort interval on a sample of runs:
    first block size x step form at sort interval 10, then the best of those
    at sort intervals 5 and 20.  The one-launch form is kept unless one launch
    per phase is more than 1 % faster at the same block size."""
    sample = runs[: min(24, len(runs))]
    cap = sum(r["n_particles"] for r in sample)
    results = []

    def trial(th, fused, si):
        bt = mpg.Batch(device, budget_bytes=64 << 30, particle_capacity=cap)
        bt.tuning(th, si, fused=fused)
        for r in sample:
            batch_admit(bt, r, steps=1000)
        bt.step(2)
        st = bt.step(8)
        bt.close()
        results.append((st.particle_steps / max(st.ms, 1e-9), th, fused, si))

    for th in (256, 512, 1024):
        for fused in (True, False):
            trial(th, fused, 10)
    _, th, fused, _ = max(results)
    rate = {(t, f): v for v, t, f, _ in results}
    if not fused and rate[(th, True)] * 1.01 >= rate[(th, False)]:
        fused = True
    for si in (5, 20):
        trial(th, fused, si)
    best = max((r for r in results if r[1] == th and r[2] == fused), key=lambda r: r[0])
    return {"cg_threads": best[1], "fused": best[2], "sort_interval": best[3],
            "tried": [{"cg_threads": th, "fused": fu, "sort_interval": si, "particle_steps_per_ms": round(v, 1)}
                      for v, th, fu, si in results]}


def _by_id(d, n_ids):
    """Particle arrays of a download placed at their ids (NaN / -1 where dead)."""
    live = d["cell"] >= 0
    ids = d["id"][live]
    cell = np.full(n_ids, -1, np.int64)
    x = np.full((n_ids, 3), np.nan)
    v = np.full((n_ids, 3), np.nan)
    cell[ids] = d["cell"][live]
    x[ids] = d["x"][live]
    v[ids] = d["v"][live]
    return cell, x, v


def accuracy_vs_plain(mpg, w, steps, device=0):
    """Error of the mixed form against the FP64 plain form over `steps` steps
    of the same fills (both forms stepped side by side):
      * phi: max |phi_mixed - phi_plain| / max |phi_plain| after every step;
      * E per tet after the last step: max |E_mixed - E_plain| / max |E_plain|;
      * particles after the last step, matched by id: survivors in both forms,
        in one form only, cell-id disagreements, max and rms |x_mixed -
        x_plain| (box length 1), max |v_mixed - v_plain| / max |v_plain|;
      * the kinetic energy per step and the survivor counts per step;
      * charge_exact: the mixed form's fixed-point charge sums exactly to its
        particles' quanta.
    Also returns the plain form's per-phase device times over these steps."""
    m = make_ctx(mpg, w, mpg.MIXED, device=device, track_ids=1)
    p = make_ctx(mpg, w, mpg.PLAIN, device=device, track_ids=1)
    n_ids = total_particles(w) if "ref_fills" not in w else p.count()
    p.set_timing(True)
    errs, ke, alive = [], 0.0, []
    tp = {k: 0.0 for k in ("deposit", "solve", "efield", "move", "sort")}
    iters_p, iters_m = 0, 0
    for _ in range(steps):
        sm = m.step(w["dt"], 1)
        sp = p.step(w["dt"], 1)
        for k in tp:
            tp[k] += getattr(sp, "ms_" + k)
        iters_p += sp.solver_iters
        iters_m += sm.solver_iters
        pm = m.get_field(mpg.FIELD_PHI)
        pp = p.get_field(mpg.FIELD_PHI)
        errs.append(float(np.abs(pm - pp).max() / max(np.abs(pp).max(), 1e-300)))
        ke = max(ke, abs(sm.ke - sp.ke) / max(abs(sp.ke), 1e-300))
        alive.append((int(sm.n_alive), int(sp.n_alive)))
    p.set_timing(False)
    Em = m.get_field(mpg.FIELD_E_TET)
    Ep = p.get_field(mpg.FIELD_E_TET)
    e_err = float(np.abs(Em - Ep).max() / max(np.abs(Ep).max(), 1e-300))
    acc, _, qfix = m.charge()
    cs, _, _ = m.mixed_download()
    live = cs != mpg.DEAD
    species = (cs[live] >> 24).astype(np.int64)
    expect = int(np.bincount(species, minlength=len(qfix)).astype(object).dot(qfix.astype(object)))
    exact = int(acc.astype(object).sum()) == expect
    del cs, live, species
    cm, xm, vm = _by_id(m.download(), n_ids)
    m.close()
    cp, xp, vp = _by_id(p.download(), n_ids)
    p.close()
    both = (cm >= 0) & (cp >= 0)
    dx = np.abs(xm[both] - xp[both])
    dv = np.abs(vm[both] - vp[both])
    vscale = max(float(np.abs(vp[both]).max()) if both.any() else 0.0, 1e-300)
    parts = {"alive_both": int(both.sum()), "alive_mixed_only": int(((cm >= 0) & (cp < 0)).sum()),
             "alive_plain_only": int(((cp >= 0) & (cm < 0)).sum()),
             "cell_mismatch": int((cm[both] != cp[both]).sum()),
             "x_abs_err_max": float(dx.max()) if dx.size else 0.0,
             "x_abs_err_rms": float(np.sqrt((dx ** 2).mean())) if dx.size else 0.0,
             "v_rel_err_max": float(dv.max() / vscale) if dv.size else 0.0,
             "v_rel_err_rms": float(np.sqrt((dv ** 2).mean()) / vscale) if dv.size else 0.0}
    plain_phases = {k: round(v / steps, 4) for k, v in tp.items()}
    out = {"steps": steps, "phi_rel_err_max": max(errs), "phi_rel_err_last": errs[-1],
           "phi_rel_err_every_10": [errs[i] for i in range(9, steps, 10)],
           "e_rel_err_last": e_err, "ke_rel_diff_max": ke, "charge_exact": bool(exact),
           "particles_last_step": parts,
           "alive_mixed_vs_plain_every_10": [alive[i] for i in range(9, steps, 10)],
           "alive_max_abs_diff": max(abs(a - b) for a, b in alive),
           "solver_iters_per_step": {"mixed": iters_m / steps, "plain": iters_p / steps},
           "how": "same fills, both forms stepped side by side; phi and E: max|mixed-plain|/max|plain|; "
                  "particles matched by id after the last step (x in units of the box length)"}
    return out, plain_phases


def run_ensemble(mpg, args, device=0):
    import numpy as np
    runs = ensemble_trace()
    if args.batch_form:
        # fixed tuning instead of the autotuner (profiler captures)
        tune = {"cg_threads": 1024, "fused": args.batch_form == "fused", "sort_interval": 10, "tried": []}
    else:
        tune = autotune(mpg, runs, device)
    cap = sum(r["n_particles"] for r in runs)
    bt = mpg.Batch(device, budget_bytes=150 << 30, max_runs=256, particle_capacity=cap)
    bt.tuning(tune["cg_threads"], tune["sort_interval"], fused=tune["fused"])
    t0 = time.perf_counter()
    for r in runs:
        assert batch_admit(bt, r) is not None
    t_admit = time.perf_counter() - t0
    lat, ps, ms, graph = [], 0, 0.0, 0
    clocks = ClockSampler(device)
    clocks.start()
    while True:
        st = bt.step(1)
        if st.active_runs == 0:
            break
        lat.append(st.ms)
        ps += st.particle_steps
        ms += st.ms
        graph = max(graph, st.graph)
    clk = clocks.stop()
    bt.close()
    if args.no_plain:
        seq_s, seq_detail = float("nan"), {"skipped": "--no-plain"}
    else:
        seq_s, seq_detail = plain_sequential_time(mpg, runs, device)
    seq = sum(r["n_particles"] * r["steps"] for r in runs) / seq_s
    value = ps / (ms * 1e-3)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": len(lat), "warmup": 0,
            "ms_per_step": ms / max(len(lat), 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "ensemble256-kuhn8to32-1e4to2e6-mixed", "runs": len(runs),
                       "particles": cap, "steps_per_run": 100},
            "ensemble": {"p50_step_ms": float(np.percentile(lat, 50)), "p99_step_ms": float(np.percentile(lat, 99)),
                         "batch_steps": len(lat), "admission_s": round(t_admit, 2), "graph": graph,
                         "autotune": tune, "plain_sequential_particle_steps_per_s": seq,
                         "plain_sequential_sample": seq_detail, "speedup_vs_plain_sequential": value / seq},
            "clocks": clk}


def plain_sequential_time(mpg, runs, device=0, sample_small=None, sample_big=8, steps=2):
    """Seconds the plain FP64 form needs to run `runs` one after another.
    Each timed run is set up (mesh, fill), stepped once untimed, then `steps`
    steps are timed with device events; its time is steps_i x the mean step
    time.  All runs are timed when the sample covers them (the ensemble);
    otherwise (the serving stream) per stratum -- the 64^3 runs and the
    others -- a random sample is timed and the step time of the others is
    predicted by a least-squares fit t = c0 + c1 nodes + c2 particles on it."""
    rng = np.random.default_rng(7)
    strata = {"big": [r for r in runs if r["n_side"] >= 64], "small": [r for r in runs if r["n_side"] < 64]}
    total_s, detail = 0.0, {}

    def step_ms(r):
        ctx = mpg.Ctx(device)
        ctx.mesh(r["n_side"], split=mpg.SPLIT_KUHN6)
        ctx.configure(precision=mpg.PLAIN, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10,
                      max_iter=5000, warm_start=1, kill_on_wall=1, rho_background=1.0)
        ctx.reserve(r["n_particles"])
        ctx.fill_uniform(r["n_particles"], r["seed"], 0, 1.0 / r["n_particles"], vth=r["vth"])
        ctx.step(0.01, 1)
        ctx.timer_start()
        ctx.step(0.01, steps)
        ms = ctx.timer_stop() / steps
        ctx.close()
        return ms

    for name, rs in strata.items():
        if not rs:
            continue
        k = sample_big if name == "big" else (sample_small or len(rs))
        idx = np.arange(len(rs)) if k >= len(rs) else rng.choice(len(rs), size=k, replace=False)
        times = {int(i): step_ms(rs[int(i)]) for i in idx}
        if len(times) == len(rs):
            ms_all = [times[i] for i in range(len(rs))]
            how = "all runs timed"
        else:
            X = np.array([[1.0, (rs[i]["n_side"] + 1) ** 3, rs[i]["n_particles"]] for i in times])
            y = np.array([times[i] for i in times])
            coef, *_ = np.linalg.lstsq(X, y, rcond=None)
            ms_all = [times[i] if i in times else
                      max(float(coef @ [1.0, (r["n_side"] + 1) ** 3, r["n_particles"]]), min(y))
                      for i, r in enumerate(rs)]
            how = "sampled, step time fitted on nodes and particles"
        t = sum(m * r["steps"] for m, r in zip(ms_all, rs)) * 1e-3
        total_s += t
        detail[name] = {"runs": len(rs), "timed": len(times), "seconds": t, "how": how}
    return total_s, detail


def run_serving(mpg, args, device=0):
    """Continuous batching on the host wall clock.  Runs arrive at their trace
    times; a pool of host threads builds each arrived run's mesh and tables
    (mpg_batch_prepare, overlapping the batch's steps on the GPU); between
    steps the stepping thread admits prepared runs in arrival order while they
    fit the budget and slots (mpg_batch_admit_prepared), advances every
    resident run by one batch step, and retires finished runs.  A run's
    latency is its completion time minus its arrival time on the wall clock,
    admission included."""
    from collections import deque
    from concurrent.futures import ThreadPoolExecutor
    runs = serving_trace(seconds=args.serve_seconds)
    tune = autotune(mpg, [r for r in runs if r["n_side"] < 64], device)
    cap = 200 << 20
    bt = mpg.Batch(device, budget_bytes=150 << 30, max_runs=256, particle_capacity=cap)
    bt.tuning(tune["cg_threads"], tune["sort_interval"], fused=tune["fused"])
    pool = ThreadPoolExecutor(max_workers=max(2, min(8, (os.cpu_count() or 2) // 2)))

    def prepare(r):
        return mpg.RunPrep(r["n_side"], r["n_particles"], r["seed"], vth=r["vth"], dt=0.01, tol=1e-10,
                           max_iter=5000, steps=r["steps"])

    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0  # noqa: E731
    nxt, prepared, resident = 0, deque(), {}
    step_ms, step_wall_ms, done, adm_wait, ps, busy = [], [], [], [], 0, 0.0
    max_resident = 0
    while nxt < len(runs) or prepared or resident:
        t = now()
        while nxt < len(runs) and runs[nxt]["arrival"] <= t:
            prepared.append((runs[nxt], pool.submit(prepare, runs[nxt])))
            nxt += 1
        while prepared and prepared[0][1].done():
            r, fut = prepared[0]
            prep = fut.result()
            slot = bt.admit_prepared(prep, allow=(mpg.ERR_CAPACITY,))
            if slot is None:
                break
            prep.close()
            prepared.popleft()
            resident[slot] = r
            adm_wait.append(now() - r["arrival"])
        max_resident = max(max_resident, len(resident))
        if not resident:
            time.sleep(0.0005)
            continue
        w0 = time.perf_counter()
        st = bt.step(1)
        step_wall_ms.append((time.perf_counter() - w0) * 1e3)
        step_ms.append(st.ms)
        busy += st.ms * 1e-3
        ps += st.particle_steps
        for slot in list(resident):
            if bt.info(slot).finished:
                r = resident.pop(slot)
                done.append(now() - r["arrival"])
                bt.retire(slot)
    completion = now()
    pool.shutdown()
    bt.close()
    seq_s, seq_detail = plain_sequential_time(mpg, runs, device, sample_small=64)
    value = ps / completion
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": len(step_ms), "warmup": 0,
            "ms_per_step": busy * 1e3 / max(len(step_ms), 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serving-poisson20-%ds-mixed" % int(args.serve_seconds), "runs": len(runs),
                       "budget_bytes": 150 << 30, "clock": "host wall clock, admission included"},
            "serving": {"p50_step_ms": float(np.percentile(step_ms, 50)),
                        "p99_step_ms": float(np.percentile(step_ms, 99)),
                        "p50_step_wall_ms": float(np.percentile(step_wall_ms, 50)),
                        "p99_step_wall_ms": float(np.percentile(step_wall_ms, 99)),
                        "completion_s": completion, "arrival_window_s": args.serve_seconds,
                        "gpu_busy_s": busy, "particle_steps": ps, "max_resident_runs": max_resident,
                        "throughput_while_busy": ps / busy,
                        "run_latency_p50_s": float(np.percentile(done, 50)),
                        "run_latency_p99_s": float(np.percentile(done, 99)),
                        "admission_wait_p50_s": float(np.percentile(adm_wait, 50)),
                        "admission_wait_p99_s": float(np.percentile(adm_wait, 99)),
                        "autotune": tune,
                        "plain_sequential_s": seq_s, "plain_sequential_sample": seq_detail,
                        "speedup_vs_plain_sequential": seq_s / completion,
                        "how": "speedup = time the plain FP64 form needs for the same runs one after another "
                               "(stratified sample, see plain_sequential_sample) / serving completion time"}}


class CpuRun:
    """The CPU restatement of the reference step (plain FP64, OpenMP on all
    host cores) set up on workload w: mesh, assembled system, fill."""

    def __init__(self, w):
        sys.path.insert(0, ROOT)
        from oracle import oracle as O
        O.build()
        self.O, self.w = O, w
        self.cores = os.cpu_count() or 1
        m = O.Mesh(w["n_side"], split=6, lo=w.get("lo", 0.0), hi=w.get("hi", 1.0), mapping=4 if w["jitter"] else 0,
                   jitter=w["jitter"], seed=7, periodic=w.get("periodic", 0))
        m.assemble(1)
        P = total_particles(w)
        parts = O.Particles(P)
        qs, ms = [0.0] * 16, [1.0] * 16
        if "ref_fills" in w:
            qs[0], ms[0], qs[2], ms[2] = -1.0, 1.0, 1.0, 1837.0
            for f in w["ref_fills"]:
                parts.fill_ref(m, f["nppe"], f["type"], f["density"], vel=f["vel"], temp=f["temp"],
                               mass=ms[f["type"]])
        else:
            by_charge = {}
            for sp in w["species"]:
                by_charge[sp["q"]] = by_charge.get(sp["q"], 0) + sp["n"]
            for i, sp in enumerate(w["species"]):
                k = sp.get("same", i)
                qs[k], ms[k] = sp["q"], sp["m"]
                parts.fill_uniform(m, sp["n"], sp["seed"], k, 1.0 / by_charge[sp["q"]], drift=sp["drift"],
                                   vth=sp["vth"], nthreads=self.cores)
        self.m, self.parts, self.qs, self.ms = m, parts, qs, ms
        self.bg = m.background(w["rho_background"]) if w["rho_background"] else None
        self.phi = np.zeros(m.N)
        self.cfg = O.StepCfg(1, 1, 1e-10, 5000, 1, 1, 1, 1000, 1, self.cores)
        self.scratch = np.zeros((P, 3))

    def step(self):
        """One full step; returns (particles at its start, seconds)."""
        n0 = self.parts.n
        t0 = time.perf_counter()
        self.O.step(self.m, self.parts, self.cfg, self.w["dt"], self.qs, self.ms, self.bg, self.phi, self.scratch)
        return n0, time.perf_counter() - t0


def cpu_baseline(w, budget_s=15.0, max_steps=3):
    """A bounded sample of the workload on the CPU restatement: full steps of
    the whole workload until budget_s seconds of stepping or max_steps."""
    run = CpuRun(w)
    done, ps, t_used = 0, 0, 0.0
    while done < max_steps and t_used < budget_s:
        n0, dt = run.step()
        t_used += dt
        ps += n0
        done += 1
    return {"value": ps / t_used, "unit": UNIT, "cores": run.cores, "kind": "port", "steps_timed": done,
            "sample": f"{done} full steps of the same workload ({total_particles(w)} particles, plain FP64, "
                      f"OpenMP {run.cores} threads)",
            "seconds": round(t_used, 3)}


def run_reference(args, w, budget_s=60.0):
    """The reference arm: the CPU restatement of the reference's step (the
    reference itself cannot be built here) on all host cores, rank 0 only.
    Full steps of the whole workload: min(W, 3) untimed ones and up to K
    timed ones, stopping once budget_s seconds of timed steps are spent, so
    that the run ends within a few minutes on the large workloads; the line
    reports the steps actually timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    run = CpuRun(w)
    warm = min(args.warmup, 3)
    for _ in range(warm):
        run.step()
    ps, t_used, k = 0, 0.0, 0
    while k < max(args.steps, 1) and (k == 0 or t_used < budget_s):
        n0, dt = run.step()
        ps += n0
        t_used += dt
        k += 1
    value = ps / t_used
    cb = {"value": value, "unit": UNIT, "cores": run.cores, "kind": "port", "steps_timed": k,
          "steps_requested": args.steps, "warmup_steps": warm,
          "sample": f"{k} timed full steps after {warm} untimed of the whole workload "
                    f"({total_particles(w)} particles, plain FP64, OpenMP {run.cores} threads; at most "
                    f"{budget_s:.0f} s of timed steps)",
          "seconds": round(t_used, 3)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": k, "warmup": warm, "ms_per_step": t_used / k * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"]}, "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def plain_bytes(w, ctx, phases_ms, iters_per_step):
    """Algorithmic bytes (and FP64 operations) per step of the plain FP64
    form's phases, for its roofline.
    move (k_plain_move): per particle 88 B read (cell, x, x_ref, v, weight,
      species) + 76 B written (cell, x, x_ref, v); per tet the walk tables
      (neighbours 16 B, J^-1 72 B, E 24 B, first node 16 B) once.
    solve (k_cg64_dia): per CG iteration and row the FP64 diagonals (8 nd B)
      and eight 8-byte vector touches (p read and written, p gathered, q
      written and read, x and r read and written); nd = 15 on the Kuhn split.
      FP64 operations per row and iteration: nd + 5 fused multiply-adds
      (the product; p, p.q, x, r, r.r), each counted as two.
    compaction (the plain form's 'sort' phase): per particle 4 B (live count)
      + 88 B read + 88 B written."""
    T, N = ctx.T, ctx.N
    P = total_particles(w)
    nd = 15
    return {"move": P * 164 + T * 128, "solve": iters_per_step * (8 * nd + 64) * N,
            "solve_fp64_ops": iters_per_step * 2 * (nd + 5) * N, "sort": P * 180}


def time_steps(ctx, w, steps, warmup):
    """(particle-steps, device ms, stats) of `steps` steps after `warmup`."""
    for _ in range(warmup):
        ctx.step(w["dt"], 1)
    n0 = ctx.count()
    ctx.timer_start()
    st = ctx.step(w["dt"], steps)
    ms = ctx.timer_stop()
    return 0.5 * (n0 + st.n_alive) * steps, ms, st


def phase_times(ctx, w, k):
    ctx.set_timing(True)
    ph = ctx.step(w["dt"], k)
    ctx.set_timing(False)
    return {n: getattr(ph, "ms_" + n) / k for n in ("deposit", "solve", "efield", "move", "sort")}, ph


def e2e_mixed(mpg, ctx, w, steps, barrier_sum, barrier_max):
    """End to end through the C ABI with host buffers: state upload, K steps
    with the step statistics read back each step, state download; host wall
    clock, median of three passes."""
    for _ in range(2):
        ctx.step(w["dt"], 1)
    cs, b, v = ctx.mixed_download()
    pinned = False
    try:
        import torch

        def pin(a):
            t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(a.dtype).reshape(a.shape)
            np.copyto(t, a)
            return t
        cs, b, v = pin(cs), pin(b), pin(v)
        out = tuple(pin(np.empty_like(a)) for a in (cs, b, v))
        pinned = True
    except Exception:
        out = None
    reps = []
    for _ in range(3):
        t0 = time.perf_counter()
        ctx.mixed_upload(cs, b, v)
        n_e = ctx.count()
        for _ in range(steps):
            ctx.step(w["dt"], 1)
        cs2, b2, v2 = ctx.mixed_download(out=out)
        t1 = time.perf_counter()
        reps.append(barrier_sum(n_e * steps) / barrier_max(t1 - t0))
    nbytes = cs.nbytes + b.nbytes + v.nbytes
    return {"value": sorted(reps)[1], "unit": UNIT, "h2d_bytes_per_step": int(nbytes / steps),
            "d2h_bytes_per_step": int((cs2.nbytes + b2.nbytes + v2.nbytes) / steps + 136),
            "pinned_host_buffers": pinned, "passes": [round(x, 1) for x in reps],
            "how": "mpg_mixed_upload from host buffers, mpg_step x K with stats read back each "
                   "step, mpg_mixed_download into host buffers; host wall clock, median of 3 passes"}


def standard_summary(mpg, args, device):
    """The 48^3 two-species configuration, mixed and plain, as an extra key."""
    w = WORKLOADS["standard"]
    ctx = make_ctx(mpg, w, mpg.MIXED, device=device)
    ps, ms, st = time_steps(ctx, w, args.steps, max(args.warmup, 3))
    ctx.close()
    pc = make_ctx(mpg, w, mpg.PLAIN, device=device)
    kp = max(1, min(args.steps, 5))
    pps, pms, _ = time_steps(pc, w, kp, 2)
    pc.close()
    v, pv = ps / (ms * 1e-3), pps / (pms * 1e-3)
    return {"workload": w["name"], "value": v, "unit": UNIT, "steps": args.steps, "ms_per_step": ms / args.steps,
            "plain_fp64": {"value": pv, "steps": kp, "ms_per_step": pms / kp}, "mixed_over_plain": v / pv}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS) + ["ensemble", "serving"])
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the 48^3 configuration key")
    ap.add_argument("--batch-form", default=None, choices=["fused", "phases"],
                    help="ensemble: fixed batch tuning (1024-thread solver blocks, sort interval 10) with this "
                         "step form instead of the autotuner")
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="steps of the mixed-vs-FP64 comparison (default: the configuration's step count)")
    ap.add_argument("--warm-start", type=int, default=2, choices=[0, 1, 2, 3],
                    help="CG initial guess: 0 zero, 1 previous phi, 2/3 linear/quadratic extrapolation")
    ap.add_argument("--sort-interval", type=int, default=None,
                    help="cell sort every K steps in the mixed form (default: the workload's, 10)")
    ap.add_argument("--mixed-solver", default="mg", choices=["cg", "mg"],
                    help="inner solver of the mixed form: plain CG or multigrid-preconditioned CG")
    ap.add_argument("--form", default=None, choices=["mixed", "plain"],
                    help="form of the timed run (default: plain for the small workload, mixed otherwise)")
    ap.add_argument("--particle-scale", type=float, default=1.0,
                    help="scale the workload's particle counts (small cases for profiler captures; the "
                         "workload name then carries the scale)")
    args = ap.parse_args()
    global WARM_START, MIXED_SOLVER
    WARM_START = args.warm_start
    MIXED_SOLVER = args.mixed_solver
    if args.sort_interval is not None:
        for wl in WORKLOADS.values():
            if wl["sort_interval"]:
                wl["sort_interval"] = args.sort_interval
    if args.workload in ("ensemble", "serving"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or serving mode; "
                              "its CPU step is timed by the single-run workloads"}))
            return 0
        mpg = _pkg()
        mpg.build()
        mpg.load()
        line = run_ensemble(mpg, args) if args.workload == "ensemble" else run_serving(mpg, args)
        print(json.dumps(line), flush=True)
        return 0
    w = WORKLOADS[args.workload]
    if args.particle_scale != 1.0:
        w = dict(w, name=w["name"] + "-pscale%g" % args.particle_scale,
                 species=[dict(sp, n=max(1, int(sp["n"] * args.particle_scale))) for sp in w["species"]])
    if args.impl == "reference":
        return run_reference(args, w)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(local)

    def barrier_max(x):
        if dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def barrier_sum(x):
        if dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())

    mpg = _pkg()
    mpg.build()
    mpg.load()
    form = args.form or ("plain" if args.workload == "small" else "mixed")
    precision = mpg.PLAIN if form == "plain" else mpg.MIXED
    mixed = precision == mpg.MIXED
    ctx = make_ctx(mpg, w, precision, device=local, seed_offset=rank)
    for _ in range(args.warmup):
        ctx.step(w["dt"], 1)
    n0 = ctx.count()
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ctx.timer_start()
    st = ctx.step(w["dt"], args.steps)
    ms = ctx.timer_stop()
    clk = clocks.stop()
    launches = st.n_launches
    particle_steps = 0.5 * (n0 + st.n_alive) * args.steps
    t_max = barrier_max(ms)
    ps_total = barrier_sum(particle_steps)
    value = ps_total / (t_max * 1e-3)

    # per-phase device times on a separate timed pass
    k_ph = min(args.steps, 10)
    phases, ph = phase_times(ctx, w, k_ph)
    line = {}
    hbm, kind = peaks()
    if rank == 0:
        pb = phase_bytes(w, ctx, ph, k_ph, mpg) if mixed else None
        roof = None
        if pb is not None:
            dominant = max(("solve", "move", "efield", "deposit"), key=lambda k: phases[k])
            kern = {"solve": "k_cg_mg" if uses_mg(w) else "k_cg_mixed", "move": "k_mixed_move_persistent",
                    "efield": "k_efield_mixed", "deposit": "k_mixed_convert"}[dominant]
            bytes_launch = pb[dominant]
            achieved = bytes_launch / (phases[dominant] * 1e-3) / 1e9
            roof = {"bound": "hbm", "kernel": kern, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved / hbm, 4), "peak_kind": kind, "traffic": read_traffic(kern, w["name"]),
                    "algorithmic_bytes_per_launch": int(bytes_launch), "ms_per_launch": round(phases[dominant], 4)}
            # the other large phase for reference
            other = "solve" if dominant == "move" else "move"
            ob = pb[other] / (phases[other] * 1e-3) / 1e9
            roof[other + "_gbs"] = round(ob, 1)
            roof[other + "_frac"] = round(ob / hbm, 4)
            roof["cg_iters_per_step"] = round(pb["iters_per_step"], 1)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if mixed else "f64",
                "precision": (("mixed: f32 push/walk, i64 fixed-point deposit, f32 "
                               + ("multigrid-preconditioned CG" if uses_mg(w) else "CG") + " inside f64 refinement")
                              if mixed else "plain f64"),
                "data": "synthetic",
                "config": {"workload": w["name"], "n_side": w["n_side"], "tets": ctx.T, "nodes": ctx.N,
                           "sort_interval": w["sort_interval"],
                           "particles": total_particles(w), "dt": w["dt"], "config_steps": w["steps"],
                           "cg_tol": 1e-10,
                           "cg_initial_guess": ["zero", "previous phi", "extrapolated 2*phi[n-1]-phi[n-2]",
                                                "extrapolated 3*phi[n-1]-3*phi[n-2]+phi[n-3]"][WARM_START],
                           "cg_preconditioner": ("geometric multigrid V-cycle (2 Jacobi sweeps per side on "
                                                 "the fine level, 1 on coarser levels, dense coarsest solve)"
                                                 if mixed and uses_mg(w) else "none"),
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "inputs larger than L2 (particle state > 129 MB), no flush"},
                "phases_ms_per_step": {k: round(v, 4) for k, v in phases.items()},
                "solver_iters_per_step": ph.solver_iters / k_ph,
                "roofline": roof, "gpu_launches": launches, "clocks": clk}
    if mixed and not args.no_plain:
        ctx.close()
        ctx = None
        # the mixed form with the plain inner CG: the FP64 form's solver family
        if uses_mg(w):
            cc = make_ctx(mpg, w, mpg.MIXED, device=local, seed_offset=rank, solver="cg")
            kc = max(1, min(args.steps, 10))
            cps, cms, cst = time_steps(cc, w, kc, 2)
            cv = barrier_sum(cps) / (barrier_max(cms) * 1e-3)
            cc.close()
        else:
            cv, kc, cms, cst = value, args.steps, ms, st
        # plain FP64 form of the same workload (the form the mixed target is measured against)
        pc = make_ctx(mpg, w, mpg.PLAIN, device=local, seed_offset=rank)
        kp = max(1, min(args.steps, 5))
        pps, pms, pst = time_steps(pc, w, kp, 2)
        pv = barrier_sum(pps) / (barrier_max(pms) * 1e-3)
        pc.close()
        if rank == 0:
            line["mixed_cg"] = {"value": cv, "unit": UNIT, "steps": kc, "ms_per_step": cms / kc,
                                "solver_iters_per_step": cst.solver_iters / kc,
                                "how": "mixed form with the unpreconditioned FP32 inner CG (the plain form's "
                                       "solver family)"}
            line["plain_fp64"] = {"value": pv, "unit": UNIT, "steps": kp, "ms_per_step": pms / kp,
                                  "solver_iters_per_step": pst.solver_iters / kp,
                                  "mixed_over_plain": value / pv, "mixed_cg_over_plain": cv / pv}
            acc, pphase = accuracy_vs_plain(mpg, w, args.accuracy_steps or w["steps"], device=local)
            line["accuracy_vs_plain_fp64"] = acc
            pb = plain_bytes(w, pc, pphase, acc["solver_iters_per_step"]["plain"])
            pl = line["plain_fp64"]
            pl["phases_ms_per_step"] = pphase
            pl["roofline"] = {
                "bound": "hbm", "kernel": "k_cg64_dia", "unit": "GB/s", "peak": hbm, "peak_kind": kind,
                "achieved": round(pb["solve"] / (pphase["solve"] * 1e-3) / 1e9, 1),
                "frac": round(pb["solve"] / (pphase["solve"] * 1e-3) / 1e9 / hbm, 4),
                "fp64_tflops": round(pb["solve_fp64_ops"] / (pphase["solve"] * 1e-3) / 1e12, 3),
                "fp64_nominal_tflops": 1.25,
                "move_gbs": round(pb["move"] / (pphase["move"] * 1e-3) / 1e9, 1),
                "compaction_gbs": round(pb["sort"] / (max(pphase["sort"], 1e-9) * 1e-3) / 1e9, 1),
                "how": "algorithmic bytes per step (bench.plain_bytes) / phase device time over the accuracy "
                       "run's steps; a fused FP64 multiply-add counts as two operations"}
        if not args.no_e2e:
            ctx = make_ctx(mpg, w, precision, device=local, seed_offset=rank)
    if not args.no_e2e and ctx is not None and mixed:
        e2e = e2e_mixed(mpg, ctx, w, args.steps, barrier_sum, barrier_max)
        if rank == 0:
            line["e2e"] = e2e
    if ctx is not None:
        ctx.close()
    if rank == 0 and world == 1 and mixed and not args.no_ensemble:
        # the ensemble part of the metric: 256 runs in the batch engine
        ens = run_ensemble(mpg, args, device=local)
        line["ensemble"] = dict(ens["ensemble"], value=ens["value"], unit=UNIT, workload=ens["config"]["workload"],
                                particles=ens["config"]["particles"], steps=ens["steps"])
    if rank == 0 and world == 1 and args.workload == "large" and not args.no_extra:
        line["standard_48"] = standard_summary(mpg, args, local)
    if rank == 0:
        if not args.no_cpu:
            try:
                line["cpu_baseline"] = cpu_baseline(w)
            except Exception as e:  # the CPU baseline is reported, never required
                line["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
