"""GPU parity of the plain FP64 form against the CPU oracle (through the C ABI).

Bit-exact: mesh arrays, CSR, reference fill (cell, x, x_ref), per-tet E, the
re-synced push + walk (cell ids, exit counts, x, v), compaction order.
Tolerance (FP64 atomics / reduction order): deposit 1e-13 relative, solver
solutions 1e-9 relative, end-to-end KE 1e-10 relative per step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mesh_pair(mpg, orc, n, split, lo, hi, mapping=0, jitter=0.0, seed=0):
    ctx = mpg.Ctx(0)
    ctx.mesh(n, split=split, lo=lo, hi=hi, mapping=mapping, jitter=jitter, seed=seed)
    m = orc.Mesh(n, split=split, lo=lo, hi=hi, mapping=mapping, jitter=jitter, seed=seed)
    return ctx, m


MESHES = [(4, 5, -1.0, 1.0, 0, 0.0), (5, 6, 0.0, 1.0, 0, 0.0), (6, 6, 0.0, 1.0, 4, 0.2), (3, 5, -1.0, 1.0, 2, 0.0)]


@pytest.mark.parametrize("n,split,lo,hi,mapping,jit", MESHES)
def test_mesh_bit_exact(mpg, orc, n, split, lo, hi, mapping, jit):
    ctx, m = _mesh_pair(mpg, orc, n, split, lo, hi, mapping, jit, 9)
    a = ctx.mesh_arrays()
    assert ctx.T == m.T and ctx.N == m.N
    assert (a["tets"] == m.tets).all()
    assert (a["nbrs"] == m.nbrs).all()
    assert (a["boundary"] == m.boundary).all()
    for k in ("nodes", "jinv", "detj", "normals"):
        assert (a[k].view(np.uint64) == getattr(m, k).view(np.uint64)).all(), k


@pytest.mark.parametrize("mode", [0, 1])
def test_csr_bit_exact(mpg, orc, mode):
    ctx, m = _mesh_pair(mpg, orc, 5, 6, 0.0, 1.0, 4, 0.2, 3)
    ctx.configure(solver=mpg.SOLVER_CG if mode == 1 else mpg.SOLVER_BICGSTAB)
    rp, col, val = ctx.csr()
    orp, ocol, oval = m.assemble(mode)
    assert (rp == orp).all() and (col == ocol).all()
    assert (val.view(np.uint64) == oval.view(np.uint64)).all()


def _ref_problem(mpg, orc, n=3, nppe=4):
    ctx, m = _mesh_pair(mpg, orc, n, 5, -1.0, 1.0)
    ctx.configure(precision=mpg.PLAIN, deposit=mpg.DEPOSIT_REF_QUARTER, solver=mpg.SOLVER_BICGSTAB, tol=1e-6,
                  track_ids=1)
    cap = m.T * nppe * 3 + 1000
    ctx.reserve(cap)
    dens = 2.0 / 3.0 * np.pi ** 2
    ctx.fill_ref(nppe, 0, dens)
    ctx.fill_ref(nppe, 1, dens)
    P = orc.Particles(cap)
    P.fill_ref(m, nppe, 0, dens, mass=1.0)
    P.fill_ref(m, nppe, 1, dens, mass=1.0)
    return ctx, m, P


def test_fill_ref_matches_oracle(mpg, orc):
    ctx, m, P = _ref_problem(mpg, orc)
    d = ctx.download()
    n = P.n
    assert len(d["cell"]) == n
    assert (d["cell"] == P.cell[:n]).all()
    assert (d["xref"].view(np.uint64) == P.xref[:n].view(np.uint64)).all()
    assert (d["x"].view(np.uint64) == P.x[:n].view(np.uint64)).all()
    # velocities: Maxwellian acceptance compares against exp(); CUDA's and
    # glibc's exp may differ in the last ulp, which can flip an acceptance
    same = (d["v"] == P.v[:n]).all(axis=1)
    assert same.mean() >= 0.999
    assert (d["w"] == P.w[:n]).all()


def test_fill_uniform_matches_oracle(mpg, orc):
    ctx, m = _mesh_pair(mpg, orc, 6, 6, 0.0, 1.0, 4, 0.2, 5)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG, deposit=mpg.DEPOSIT_LINEAR)
    n = 20000
    ctx.reserve(n)
    ctx.fill_uniform(n, 77, 0, 1.0 / n, drift=(0.2, 0, 0), vth=0.05)
    P = orc.Particles(n)
    P.fill_uniform(m, n, 77, 0, 1.0 / n, drift=(0.2, 0, 0), vth=0.05)
    d = ctx.download()
    assert (d["cell"] == P.cell).all()
    assert (d["xref"].view(np.uint64) == P.xref.view(np.uint64)).all()
    assert (d["x"].view(np.uint64) == P.x.view(np.uint64)).all()
    # single-precision logf/cosf/sinf: a few ulp apart
    assert np.abs(d["v"] - P.v).max() <= 8 * np.finfo(np.float32).eps * 0.5


@pytest.mark.parametrize("mode", [0, 1])
def test_deposit_matches_oracle(mpg, orc, mode):
    ctx, m, P = _ref_problem(mpg, orc)
    cfgd = mpg.DEPOSIT_LINEAR if mode == 1 else mpg.DEPOSIT_REF_QUARTER
    ctx.configure(precision=mpg.PLAIN, deposit=cfgd, solver=mpg.SOLVER_BICGSTAB, tol=1e-6, track_ids=1)
    # identical state on both sides (velocities included)
    d = ctx.download()
    ctx.weight_charge()
    rhs = ctx.get_field(mpg.FIELD_RHS)
    P.v[: P.n] = d["v"]
    orhs = orc.deposit(m, P, mode, [-1.0, 1.0, 1.0])
    scale = np.abs(orhs).max() + 1e-300
    assert np.abs(rhs - orhs).max() <= 1e-13 * max(scale, 1.0)


def test_bicgstab_matches_oracle(mpg, orc):
    ctx, m = _mesh_pair(mpg, orc, 5, 5, -1.0, 1.0)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_BICGSTAB, tol=1e-6)
    m.assemble(0)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    ctx.set_field(mpg.FIELD_RHS, b)
    it, res = ctx.solve()
    x = ctx.get_field(mpg.FIELD_PHI)
    ox, oit, ores = orc.bicgstab(m, b, tol=1e-6)
    assert abs(it - oit) <= 1
    assert np.abs(x - ox).max() <= 1e-6 * np.abs(ox).max()
    r = b - m.spmv(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-6


def test_cg_matches_oracle(mpg, orc):
    ctx, m = _mesh_pair(mpg, orc, 7, 6, 0.0, 1.0, 4, 0.2, 2)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG, tol=1e-10, warm_start=0)
    m.assemble(1)
    rng = np.random.default_rng(4)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    ctx.set_field(mpg.FIELD_RHS, b)
    it, res = ctx.solve()
    x = ctx.get_field(mpg.FIELD_PHI)
    ox, oit, ores = orc.cg(m, b, tol=1e-10)
    assert abs(it - oit) <= 2
    assert res < 1e-10
    assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()


def test_efield_bit_exact(mpg, orc):
    ctx, m = _mesh_pair(mpg, orc, 5, 6, 0.0, 1.0, 4, 0.2, 6)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG)
    phi = np.random.default_rng(5).standard_normal(m.N)
    ctx.set_field(mpg.FIELD_PHI, phi)
    ctx.weight_efield()
    E = ctx.get_field(mpg.FIELD_E_TET)
    oE = m.efield_tet(phi)
    assert (E.view(np.uint64) == oE.view(np.uint64)).all()


@pytest.mark.parametrize("kill", [1, 0])
def test_push_walk_resynced_bit_exact(mpg, orc, kill):
    # same state + same phi -> identical cells, exits, x, x_ref, v (FP64, no FMA)
    ctx, m = _mesh_pair(mpg, orc, 6, 6, 0.0, 1.0, 4, 0.2, 8)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG, deposit=mpg.DEPOSIT_LINEAR, kill_on_wall=kill,
                  track_ids=1)
    n = 30000
    ctx.reserve(n)
    ctx.fill_uniform(n, 21, 0, 1.0 / n, vth=0.3)
    d = ctx.download()
    P = orc.Particles(n)
    P.n = n
    P.cell[:] = d["cell"]
    P.x[:] = d["x"]
    P.xref[:] = d["xref"]
    P.v[:] = d["v"]
    P.w[:] = d["w"]
    P.sp[:] = d["sp"]
    P.id[:] = d["id"]
    phi = 0.05 * np.random.default_rng(6).standard_normal(m.N)
    phi[m.boundary == 1] = 0
    ctx.set_field(mpg.FIELD_PHI, phi)
    ctx.weight_efield()
    dt = 0.2
    st = ctx.move(dt)
    Et = m.efield_tet(phi)
    E = orc.gather(m, P, 1, phi, Et)
    orc.push(m, P, E, [-1.0], dt)
    r = orc.walk(m, P, dt, kill=kill)
    assert st.n_killed == r["killed"]
    assert st.n_crossings == r["cross"]
    assert st.n_walk_limit == 0 and r["limit"] == 0
    orc.compact(P, mode=1)
    g = ctx.download()
    assert len(g["cell"]) == P.n
    assert (g["id"] == P.id[: P.n]).all()          # stable compaction order
    assert (g["cell"] == P.cell[: P.n]).all()
    for k, a in (("x", P.x), ("xref", P.xref), ("v", P.v)):
        assert (g[k].view(np.uint64) == a[: P.n].view(np.uint64)).all(), k
    ke = orc.kinetic(P, [1.0])
    assert abs(st.ke - ke) <= 1e-12 * ke


def test_reference_problem_steps_match_oracle(mpg, orc):
    # the reference's default problem: 5-split [-1,1]^3, e- and e+ per tet,
    # ref-quarter deposit, BiCGStab 1e-6, specular walls (main.cpp:89-110)
    ctx, m, P = _ref_problem(mpg, orc, n=3, nppe=4)
    d = ctx.download()
    P.v[: P.n] = d["v"]
    m.assemble(0)
    cfg = orc.StepCfg(0, 0, 1e-6, 1000, 0, 1, 0, 1000, 1, 1)
    phi = np.zeros(m.N)
    for s in range(5):
        st = ctx.step(0.1, 1)
        rc, ost, _ = orc.step(m, P, cfg, 0.1, [-1.0, 1.0, 1.0], [1.0, 1.0, 1837.0], None, phi)
        assert st.n_alive == ost.n_alive
        assert abs(st.ke - ost.ke) <= 1e-9 * abs(ost.ke)
    g = ctx.download()
    assert np.abs(g["x"] - P.x[: P.n]).max() < 1e-9


def test_config1_plain_steps_match_oracle(mpg, orc):
    # the 10^3 Kuhn plain configuration at a reduced count: Kuhn [0,1]^3, e- uniform, background, CG 1e-10,
    # absorbing walls
    n_side, n = 10, 20000
    ctx, m = _mesh_pair(mpg, orc, n_side, 6, 0.0, 1.0)
    ctx.configure(precision=mpg.PLAIN, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10,
                  warm_start=1, kill_on_wall=1, rho_background=1.0, track_ids=1)
    ctx.reserve(n)
    ctx.fill_uniform(n, 1, 0, 1.0 / n, vth=0.05)
    P = orc.Particles(n)
    P.fill_uniform(m, n, 1, 0, 1.0 / n, vth=0.05)
    d = ctx.download()
    P.v[:] = d["v"]
    m.assemble(1)
    bg = m.background(1.0)
    phi = np.zeros(m.N)
    cfg = orc.StepCfg(1, 1, 1e-10, 1000, 1, 1, 1, 1000, 1, 1)
    flips = 0
    for s in range(10):
        st = ctx.step(0.01, 1)
        rc, ost, _ = orc.step(m, P, cfg, 0.01, [-1.0], [1.0], bg, phi)
        assert abs(st.ke - ost.ke) <= 1e-10 * ost.ke
        assert abs(st.n_alive - ost.n_alive) <= 2
    g = ctx.download()
    common = np.intersect1d(g["id"], P.id[: P.n])
    gi = {int(i): k for k, i in enumerate(g["id"])}
    oi = {int(i): k for k, i in enumerate(P.id[: P.n])}
    a = np.array([gi[int(i)] for i in common])
    b = np.array([oi[int(i)] for i in common])
    flips = int((g["cell"][a] != P.cell[b]).sum())
    assert flips <= 5
    assert np.abs(g["x"][a] - P.x[b]).max() < 1e-8


def _by_id(ids, *arrays):
    order = np.argsort(ids, kind="stable")
    return (ids[order],) + tuple(a[order] for a in arrays)


def test_config1_full_run_matches_oracle(mpg, orc, capsys):
    """The plain-FP64 configuration as specified: 10^3 Kuhn cube of [0,1]^3,
    100,000 electrons uniform in volume from seed 1, v_th = 0.05, uniform
    neutralising background, phi = 0 on the boundary, absorbing walls,
    dt = 0.01, 100 steps, CG to 1e-10 -- the GPU plain form against the
    oracle from the same fill, never re-synchronised.

    Per step: survivors, wall exits and face crossings equal the oracle's
    exactly and the kinetic energy agrees to 1e-10; every 10 steps the
    surviving particles, matched by id, sit in the same cells with positions
    within 1e-9 and velocities within 1e-9 relative.  What differs between
    the two is only floating-point summation order (the GPU deposit's atomic
    order, the CG dot products' tree order), which moves phi by about the
    solver tolerance; the test reports the largest position difference and
    the cell flips it saw."""
    n_side, n, steps = 10, 100000, 100
    ctx, m = _mesh_pair(mpg, orc, n_side, 6, 0.0, 1.0)
    ctx.configure(precision=mpg.PLAIN, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10, max_iter=5000,
                  warm_start=1, kill_on_wall=1, rho_background=1.0, track_ids=1)
    ctx.reserve(n)
    ctx.fill_uniform(n, 1, 0, 1.0 / n, vth=0.05)
    P = orc.Particles(n)
    P.fill_uniform(m, n, 1, 0, 1.0 / n, vth=0.05)
    d = ctx.download()
    assert (d["cell"] == P.cell).all() and (d["xref"] == P.xref).all()
    # single-precision logf/cosf of the velocity draw may differ by an ulp
    # between CUDA and glibc: both runs start from the GPU's velocities
    P.v[:] = d["v"]
    m.assemble(1)
    bg = m.background(1.0)
    phi = np.zeros(m.N)
    cfg = orc.StepCfg(1, 1, 1e-10, 5000, 1, 1, 1, 1000, 1, 1)
    worst_x, worst_v, flips, exits = 0.0, 0.0, 0, 0
    for s in range(steps):
        st = ctx.step(0.01, 1)
        rc, ost, _ = orc.step(m, P, cfg, 0.01, [-1.0], [1.0], bg, phi)
        assert rc == 0
        assert st.n_alive == ost.n_alive, s
        assert st.n_killed == ost.n_killed, s
        assert st.n_crossings == ost.n_cross, s
        assert abs(st.ke - ost.ke) <= 1e-10 * ost.ke, s
        exits += st.n_killed
        if s % 10 == 9:
            g = ctx.download()
            gi, gc, gx, gv = _by_id(g["id"], g["cell"], g["x"], g["v"])
            oi, oc, ox, ov = _by_id(P.id[: P.n].copy(), P.cell[: P.n].copy(), P.x[: P.n].copy(),
                                    P.v[: P.n].copy())
            assert (gi == oi).all(), s
            flips += int((gc != oc).sum())
            worst_x = max(worst_x, float(np.abs(gx - ox).max()))
            worst_v = max(worst_v, float(np.abs(gv - ov).max() / np.abs(ov).max()))
    assert flips == 0
    assert worst_x <= 1e-9 and worst_v <= 1e-9
    phi_gpu = ctx.get_field(mpg.FIELD_PHI)
    assert np.abs(phi_gpu - phi).max() <= 1e-8 * np.abs(phi).max()
    with capsys.disabled():
        print(f"\nconfig 1 (100 steps): {exits} wall exits, survivors {st.n_alive}, cell flips {flips}, "
              f"max |dx| {worst_x:.2e}, max |dv|/|v| {worst_v:.2e}")


def test_capacity_and_argument_errors(mpg):
    ctx = mpg.Ctx(0)
    ctx.mesh(2, split=5, lo=-1, hi=1)
    ctx.configure()
    ctx.reserve(10)
    assert ctx.fill_ref(4, 0, 1.0) == mpg.ERR_CAPACITY
    with pytest.raises(mpg.MpgError) as e:
        ctx.mesh(0)
    assert e.value.code == mpg.ERR_ARG


def test_walk_limit_and_not_converged_are_reported(mpg):
    ctx = mpg.Ctx(0)
    ctx.mesh(4, split=6)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG, deposit=mpg.DEPOSIT_LINEAR, tol=1e-12, max_iter=1,
                  max_crossings=1, kill_on_wall=1)
    ctx.reserve(1000)
    ctx.fill_uniform(1000, 3, 0, 1e-3, vth=2.0)
    st = ctx.step(0.1, 1, allow=(mpg.ERR_NOT_CONVERGED, mpg.ERR_WALK_LIMIT))
    assert st.rc in (mpg.ERR_NOT_CONVERGED, mpg.ERR_WALK_LIMIT)
    assert st.n_walk_limit > 0
