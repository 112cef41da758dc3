"""Field-solve micro-benchmark (profiling utility).

Builds an n^3 Kuhn mesh (optionally jittered), a seeded random right-hand
side (zero on the boundary), and times K solves of the selected form with
device events.  No particles, so the device holds only the mesh and the
solver (about 2 GB at n = 128).

    python minipic-crossroads_gb300/solve_bench.py --n 128 --form mixed --repeat 3
"""
import argparse
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--jitter", type=float, default=0.0)
    ap.add_argument("--form", choices=["mixed", "plain"], default="mixed")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--solver", choices=["cg", "mg"], default="cg",
                    help="mixed form: plain inner CG or multigrid-preconditioned inner CG")
    args = ap.parse_args()
    spec = importlib.util.spec_from_file_location("minipic_gb300", os.path.join(HERE, "__init__.py"))
    mpg = importlib.util.module_from_spec(spec)
    sys.modules["minipic_gb300"] = mpg
    spec.loader.exec_module(mpg)
    mpg.build()
    ctx = mpg.Ctx(0)
    ctx.mesh(args.n, split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER if args.jitter else mpg.MAP_NONE,
             jitter=args.jitter, seed=7)
    ctx.configure(precision=mpg.MIXED if args.form == "mixed" else mpg.PLAIN, deposit=mpg.DEPOSIT_LINEAR,
                  solver=mpg.SOLVER_CG_MG if args.solver == "mg" else mpg.SOLVER_CG, tol=args.tol, max_iter=20000, warm_start=0)
    b = np.random.default_rng(1).standard_normal(ctx.N)
    nodes = ctx.mesh_arrays()["boundary"]
    b[nodes == 1] = 0.0
    ctx.set_field(mpg.FIELD_RHS, b)
    out = []
    for _ in range(args.repeat):
        ctx.timer_start()
        it, res = ctx.solve()
        ms = ctx.timer_stop()
        out.append(dict(ms=ms, iters=it, resid=res, us_per_iter=1e3 * ms / max(it, 1)))
    print(json.dumps({"n": args.n, "rows": ctx.N, "form": args.form, "solver": args.solver, "jitter": args.jitter,
                      "solves": out}))


if __name__ == "__main__":
    main()
