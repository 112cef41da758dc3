"""GPU checks of the batched ensemble engine (mpg_batch_*).

A run's field and particle state must not depend on which runs share the
batch: stepped alone or in a mix, phi and the particle set are bit-identical
(kinetic energy, a floating-point sum over particles in block order, agrees to
1e-6).  Against the single-run mixed path on the same mesh and fill (which
uses the assembled per-row FP64 matrix in the outer residual instead of the
uniform stencil): phi within 1e-7 relative, kinetic energy within 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted_state(cell, b, v):
    key = np.lexsort((v[:, 2], v[:, 1], v[:, 0], b[:, 2], b[:, 1], b[:, 0], cell))
    return cell[key], b[key], v[key]


def test_run_alone_equals_run_in_mix(mpg):
    mix = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    alone = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    mix.tuning(512, 3)
    alone.tuning(512, 3)
    a = mix.admit(8, 20000, 11, vth=0.08, steps=20)
    s_mix = mix.admit(12, 60000, 22, vth=0.05, steps=20)
    c = mix.admit(10, 30000, 33, vth=0.1, drift=(0.1, 0, 0), steps=20)
    s_alone = alone.admit(12, 60000, 22, vth=0.05, steps=20)
    for _ in range(8):
        st = mix.step(1)
        assert st.rc == 0
        assert alone.step(1).rc == 0
    p1, p2 = mix.phi(s_mix), alone.phi(s_alone)
    assert (p1.view(np.uint64) == p2.view(np.uint64)).all()
    x1 = _sorted_state(*mix.particles(s_mix))
    x2 = _sorted_state(*alone.particles(s_alone))
    assert len(x1[0]) == len(x2[0])
    for u, w in zip(x1, x2):
        assert (u == w).all()
    i1, i2 = mix.info(s_mix), alone.info(s_alone)
    assert i1.n_alive == i2.n_alive and i1.steps_done == i2.steps_done == 8
    assert i1.solver_iters == i2.solver_iters
    assert abs(i1.ke - i2.ke) <= 1e-6 * i2.ke
    assert mix.info(a).steps_done == 8 and mix.info(c).steps_done == 8


def test_run_admitted_mid_flight_equals_run_alone(mpg):
    """Continuous batching: run B is prepared on the host while run A is
    resident, admitted after A has taken 5 steps, then both step together.
    B's phi and particle set equal those of B stepped alone in its own batch
    (admitted from the same preparation), bit for bit."""
    mix = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    alone = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    mix.tuning(512, 3)
    alone.tuning(512, 3)
    a = mix.admit(10, 50000, 41, vth=0.08, drift=(0.05, 0, 0), steps=30)
    for _ in range(5):
        assert mix.step(1).rc == 0
    prep = mpg.RunPrep(12, 60000, 42, vth=0.05, steps=12)
    b_mix = mix.admit_prepared(prep)
    b_alone = alone.admit_prepared(prep)
    prep.close()
    assert b_mix is not None and b_alone is not None
    for _ in range(8):
        assert mix.step(1).rc == 0
        assert alone.step(1).rc == 0
    p1, p2 = mix.phi(b_mix), alone.phi(b_alone)
    assert (p1.view(np.uint64) == p2.view(np.uint64)).all()
    x1 = _sorted_state(*mix.particles(b_mix))
    x2 = _sorted_state(*alone.particles(b_alone))
    assert len(x1[0]) == len(x2[0])
    for u, w in zip(x1, x2):
        assert (u == w).all()
    i1, i2 = mix.info(b_mix), alone.info(b_alone)
    assert i1.n_alive == i2.n_alive and i1.steps_done == i2.steps_done == 8
    assert i1.solver_iters == i2.solver_iters
    assert mix.info(a).steps_done == 13


def test_fused_step_equals_one_launch_per_phase(mpg):
    """One persistent launch per batch step (phases behind grid barriers)
    against one launch per phase, same runs: phi and the particle sets are
    bit-identical, and a fused step launches one kernel."""
    bts = []
    for fused in (True, False):
        bt = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
        bt.tuning(512, 3, fused=fused)
        slots = [bt.admit(8, 20000, 61, vth=0.08, steps=20), bt.admit(12, 50000, 62, vth=0.05, steps=20),
                 bt.admit(10, 30000, 63, vth=0.1, drift=(0.1, 0, 0), steps=20)]
        bts.append((bt, slots))
    for k in range(7):
        sts = [bt.step(1) for bt, _ in bts]
        assert all(st.rc == 0 for st in sts)
        if k == 6:
            assert sts[0].graph == 1 and sts[0].n_launches <= 1 + 10  # one step launch (+ a sort's kernels)
    (f, fs), (u, us) = bts
    for a, b in zip(fs, us):
        assert (f.phi(a).view(np.uint64) == u.phi(b).view(np.uint64)).all()
        x1, x2 = _sorted_state(*f.particles(a)), _sorted_state(*u.particles(b))
        for p, q in zip(x1, x2):
            assert (p == q).all()
        i1, i2 = f.info(a), u.info(b)
        assert i1.n_alive == i2.n_alive and i1.solver_iters == i2.solver_iters
        assert abs(i1.ke - i2.ke) <= 1e-6 * i2.ke


def test_batch_run_matches_single_run(mpg):
    n_side, n, seed, dt = 10, 40000, 5, 0.01
    bt = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    bt.tuning(512, 0)
    s = bt.admit(n_side, n, seed, vth=0.05, dt=dt, steps=10)
    ctx = mpg.Ctx(0)
    ctx.mesh(n_side, split=mpg.SPLIT_KUHN6)
    ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10, max_iter=5000,
                  warm_start=1, kill_on_wall=1, rho_background=1.0)
    ctx.reserve(n)
    ctx.fill_uniform(n, seed, 0, 1.0 / n, vth=0.05)
    for k in range(5):
        bst = bt.step(1)
        sst = ctx.step(dt, 1)
        bi = bt.info(s)
        assert abs(bi.ke - sst.ke) <= 1e-5 * sst.ke, (k, bi.ke, sst.ke)
        assert abs(bi.n_alive - sst.n_alive) <= 2
    pb = bt.phi(s)
    pc = ctx.get_field(mpg.FIELD_PHI)
    assert np.abs(pb - pc).max() <= 1e-7 * np.abs(pc).max()


def test_budget_slots_finish_and_reuse(mpg):
    bt = mpg.Batch(0, budget_bytes=64 << 20, max_runs=2, particle_capacity=200000)
    s0 = bt.admit(8, 10000, 1, steps=3)
    s1 = bt.admit(8, 10000, 2, steps=5)
    assert bt.admit(8, 10000, 3, steps=5, allow=(mpg.ERR_CAPACITY,)) is None   # no free slot
    st = bt.step(4)
    assert st.rc == 0
    i0, i1 = bt.info(s0), bt.info(s1)
    assert i0.finished == 1 and i0.steps_done == 3 and i0.active == 0
    assert i1.steps_done == 4 and i1.active == 1
    bt.retire(s0)
    s2 = bt.admit(8, 10000, 4, steps=2)
    assert s2 == s0                      # slot reused, old particles gone
    cell, b, v = bt.particles(s2)
    assert len(cell) == 10000
    bt.step(2)
    assert bt.info(s2).finished == 1 and bt.info(s1).finished == 1
    big = mpg.Batch(0, budget_bytes=1 << 20, particle_capacity=1000)
    assert big.admit(16, 500, 1, allow=(mpg.ERR_CAPACITY,)) is None       # budget


def test_jittered_run_matches_single_run_and_mix(mpg):
    """A run on a mesh with jittered interior nodes carries its per-row
    15-diagonal operator: against the single-run mixed path on the same
    mesh and fill, phi within 1e-7 relative and kinetic energy within 1e-5;
    stepped alone or beside uniform runs, phi and the particle set are
    bit-identical."""
    n_side, n, seed, dt, jit = 10, 40000, 7, 0.01, 0.2
    bt = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    bt.tuning(512, 0)
    s = bt.admit(n_side, n, seed, vth=0.05, dt=dt, steps=10, jitter=jit, mesh_seed=9)
    mix = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
    mix.tuning(512, 0)
    mix.admit(8, 20000, 3, vth=0.08, dt=dt, steps=10)
    s_mix = mix.admit(n_side, n, seed, vth=0.05, dt=dt, steps=10, jitter=jit, mesh_seed=9)
    mix.admit(12, 30000, 4, vth=0.05, dt=dt, steps=10, jitter=0.1, mesh_seed=2)
    ctx = mpg.Ctx(0)
    ctx.mesh(n_side, split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER, jitter=jit, seed=9)
    ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10, max_iter=5000,
                  warm_start=1, kill_on_wall=1, rho_background=1.0)
    ctx.reserve(n)
    ctx.fill_uniform(n, seed, 0, 1.0 / n, vth=0.05)
    for k in range(5):
        assert bt.step(1).rc == 0 and mix.step(1).rc == 0
        sst = ctx.step(dt, 1)
        bi = bt.info(s)
        assert abs(bi.ke - sst.ke) <= 1e-5 * sst.ke, (k, bi.ke, sst.ke)
        assert abs(bi.n_alive - sst.n_alive) <= 2
    pb = bt.phi(s)
    pc = ctx.get_field(mpg.FIELD_PHI)
    assert np.abs(pb - pc).max() <= 1e-7 * np.abs(pc).max()
    assert (mix.phi(s_mix).view(np.uint64) == pb.view(np.uint64)).all()
    x1, x2 = _sorted_state(*mix.particles(s_mix)), _sorted_state(*bt.particles(s))
    for u, w in zip(x1, x2):
        assert (u == w).all()


def test_multigrid_runs_match_single_run_and_cg(mpg, monkeypatch):
    """Runs whose grid coarsens (here 16^3 and 24^3, one of them jittered)
    solve with the multigrid-preconditioned CG on one CTA: against the
    single-run mixed path (phi within 1e-7 relative, kinetic energy within
    1e-5) and against the batch's own plain inner CG (MPG_BATCH_MG=0, phi
    within 1e-7), with several times fewer iterations; stepped alone or in a
    mix, bit-identical."""
    dt = 0.01
    specs = [dict(n_side=16, n=60000, seed=31, jitter=0.0), dict(n_side=24, n=80000, seed=32, jitter=0.15)]

    def batch(specs_in, mg=True):
        monkeypatch.setenv("MPG_BATCH_MG", "1" if mg else "0")
        bt = mpg.Batch(0, budget_bytes=4 << 30, particle_capacity=1 << 20)
        bt.tuning(512, 0)
        slots = [bt.admit(s["n_side"], s["n"], s["seed"], vth=0.05, dt=dt, steps=10, jitter=s["jitter"], mesh_seed=5)
                 for s in specs_in]
        return bt, slots

    bt, slots = batch(specs)
    cg, cg_slots = batch(specs, mg=False)
    mix, mix_slots = batch([dict(n_side=9, n=10000, seed=3, jitter=0.0)] + specs)
    ctxs = []
    for s in specs:
        ctx = mpg.Ctx(0)
        ctx.mesh(s["n_side"], split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER if s["jitter"] else mpg.MAP_NONE,
                 jitter=s["jitter"], seed=5)
        ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10,
                      max_iter=5000, warm_start=1, kill_on_wall=1, rho_background=1.0)
        ctx.reserve(s["n"])
        ctx.fill_uniform(s["n"], s["seed"], 0, 1.0 / s["n"], vth=0.05)
        ctxs.append(ctx)
    for k in range(4):
        assert bt.step(1).rc == 0 and cg.step(1).rc == 0 and mix.step(1).rc == 0
        sts = [ctx.step(dt, 1) for ctx in ctxs]
        for s, st in zip(slots, sts):
            bi = bt.info(s)
            assert abs(bi.ke - st.ke) <= 1e-5 * st.ke, (k, bi.ke, st.ke)
    for s, c, ctx in zip(slots, cg_slots, ctxs):
        pb, pc, pcg = bt.phi(s), ctx.get_field(mpg.FIELD_PHI), cg.phi(c)
        assert np.abs(pb - pc).max() <= 1e-7 * np.abs(pc).max()
        assert np.abs(pb - pcg).max() <= 1e-7 * np.abs(pcg).max()
        assert 3 * bt.info(s).solver_iters < cg.info(c).solver_iters, (bt.info(s).solver_iters, cg.info(c).solver_iters)
    for s, m in zip(slots, mix_slots[1:]):
        assert (bt.phi(s).view(np.uint64) == mix.phi(m).view(np.uint64)).all()
        x1, x2 = _sorted_state(*bt.particles(s)), _sorted_state(*mix.particles(m))
        for u, w in zip(x1, x2):
            assert (u == w).all()
