"""Phase-time probe of the mixed-precision CG solver (profiling utility).

Builds an instrumented copy of the library (-DMPG_CG_PROFILE: SM-cycle
stamps of block 0 around the phases of the inner CG iteration) into
_build_probe/, runs steps of bench.py's standard workload and prints the mean
per-iteration split: row loop, block reduction + partial store, grid-barrier
wait, cross-block totals.  Needs a GPU.

    python minipic-crossroads_gb300/cg_probe.py [--steps 5] [--solver mg]
"""
import argparse
import ctypes
import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--solver", choices=["cg", "mg"], default="cg",
                    help="cg: split of the plain inner CG iteration; mg: per-barrier split of the "
                         "multigrid-preconditioned iteration")
    ap.add_argument("--workload", default="standard")
    args = ap.parse_args()
    spec = importlib.util.spec_from_file_location("_mpg_build", os.path.join(HERE, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    out = os.path.join(HERE, "_build_probe")
    lib_path = b.build(out_dir=out, extra_nvcc=["-DMPG_CG_PROFILE"])
    spec = importlib.util.spec_from_file_location("minipic_gb300", os.path.join(HERE, "__init__.py"))
    mpg = importlib.util.module_from_spec(spec)
    sys.modules["minipic_gb300"] = mpg
    spec.loader.exec_module(mpg)
    mpg.lib_path = lambda: lib_path  # load the instrumented build
    sys.path.insert(0, ROOT)
    import bench
    bench.MIXED_SOLVER = args.solver
    w = bench.WORKLOADS[args.workload]
    ctx = bench.make_ctx(mpg, w, mpg.MIXED)
    ctx.step(w["dt"], 3)
    L = mpg.load()
    if args.solver == "mg":
        L.mpg_probe_mg_profile.argtypes = [ctypes.c_void_p]
        p0 = (ctypes.c_ulonglong * 64)()
        L.mpg_probe_mg_profile(p0)
        ctx.step(w["dt"], args.steps)
        p1 = (ctypes.c_ulonglong * 64)()
        L.mpg_probe_mg_profile(p1)
        d = [p1[i] - p0[i] for i in range(64)]
        it = max(d[63], 1)
        f = 2.07e3  # SM cycles per microsecond at the 2070 MHz maximum clock
        rows = [{"barrier": q, "work_us": round(d[2 * q] / it / f, 3), "wait_us": round(d[2 * q + 1] / it / f, 3)}
                for q in range(31) if d[2 * q] or d[2 * q + 1]]
        print(json.dumps({"iterations": d[63], "work_us": sum(r["work_us"] for r in rows),
                          "wait_us": sum(r["wait_us"] for r in rows), "per_barrier": rows}))
        return
    L.mpg_probe_cg_profile.argtypes = [ctypes.c_void_p]
    L.mpg_probe_cg_profile_blocks.argtypes = [ctypes.c_void_p]
    p0 = (ctypes.c_ulonglong * 8)()
    b0 = (ctypes.c_ulonglong * 3072)()
    L.mpg_probe_cg_profile(p0)
    L.mpg_probe_cg_profile_blocks(b0)
    ctx.step(w["dt"], args.steps)
    p1 = (ctypes.c_ulonglong * 8)()
    b1 = (ctypes.c_ulonglong * 3072)()
    L.mpg_probe_cg_profile(p1)
    L.mpg_probe_cg_profile_blocks(b1)
    d = [p1[i] - p0[i] for i in range(6)]
    it = max(d[3], 1)
    f = 2.07e3  # SM cycles per microsecond at the 2070 MHz maximum clock
    per_block = {}
    for j, name in enumerate(("compute_reduce_us", "barrier_us", "totals_us")):
        v = sorted((b1[3 * k + j] - b0[3 * k + j]) / it / f for k in range(1024) if b1[3 * k + j] > b0[3 * k + j])
        if v:
            per_block[name] = {"blocks": len(v), "min": v[0], "median": v[len(v) // 2], "max": v[-1]}
    print(json.dumps({"iterations": d[3], "row_loop_us": d[4] / it / f, "reduce_store_us": d[5] / it / f,
                      "barrier_us": d[1] / it / f, "totals_us": d[2] / it / f,
                      "threads": os.environ.get("MPG_CG_THREADS", "512"), "per_block": per_block}))


if __name__ == "__main__":
    main()
