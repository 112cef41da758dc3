"""GPU parity on meshes periodic in x (the reference's two-stream set-up:
mesh.cpp:61-76,178-189,369-392; ES.cpp:93-110,168-189; PIC.cpp:132-134;
particle_move.hpp:190-191) against the CPU oracle, through the C ABI.

Bit-exact: mesh arrays, periodic face flags and node pairs, both CSR forms
(the reference's ghost-row system and the symmetric system without the ghost
plane), the re-synced push + walk across periodic faces (cells, exits, x,
x_ref, v), the fixed-point charge and its fold onto the pair nodes.
Tolerance: solver solutions 1e-9 relative (FP64 reduction order); mixed form
against the plain form: phi 1e-6 relative over the first steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PMESHES = [(4, 5, -1.0, 1.0, 0, 0.0), (5, 6, 0.0, 1.0, 4, 0.2), ((6, 4, 5), 6, 0.0, 1.0, 0, 0.0)]


def _pair(mpg, orc, n, split, lo, hi, mapping=0, jitter=0.0, seed=0):
    ctx = mpg.Ctx(0)
    ctx.mesh(n, split=split, lo=lo, hi=hi, mapping=mapping, jitter=jitter, seed=seed, periodic=1)
    m = orc.Mesh(n, split=split, lo=lo, hi=hi, mapping=mapping, jitter=jitter, seed=seed, periodic=1)
    return ctx, m


@pytest.mark.parametrize("n,split,lo,hi,mapping,jit", PMESHES)
def test_periodic_mesh_bit_exact(mpg, orc, n, split, lo, hi, mapping, jit):
    ctx, m = _pair(mpg, orc, n, split, lo, hi, mapping, jit, 9)
    a = ctx.mesh_arrays()
    assert ctx.T == m.T and ctx.N == m.N
    assert (a["tets"] == m.tets).all()
    assert (a["nbrs"] == m.nbrs).all()
    assert (a["boundary"] == m.boundary).all()
    for k in ("nodes", "jinv", "detj", "normals"):
        assert (a[k].view(np.uint64) == getattr(m, k).view(np.uint64)).all(), k
    fp, pr = ctx.periodic_arrays()
    assert (fp == m.face_periodic).all()
    assert (pr == m.node_pairs).all()


@pytest.mark.parametrize("mode", [0, 1])
def test_periodic_csr_bit_exact(mpg, orc, mode):
    ctx, m = _pair(mpg, orc, 5, 6, 0.0, 1.0, 4, 0.2, 3)
    ctx.configure(solver=mpg.SOLVER_CG if mode == 1 else mpg.SOLVER_BICGSTAB)
    rp, col, val = ctx.csr()
    orp, ocol, oval = m.assemble(mode)
    assert len(rp) == len(orp)
    assert (rp == orp).all() and (col == ocol).all()
    assert (val.view(np.uint64) == oval.view(np.uint64)).all()


@pytest.mark.parametrize("solver", ["cg", "bicgstab", "mixed"])
def test_periodic_solves_match_oracle(mpg, orc, solver):
    ctx, m = _pair(mpg, orc, 6, 6, 0.0, 1.0, 4, 0.2, 5)
    prec = mpg.MIXED if solver == "mixed" else mpg.PLAIN
    kind = mpg.SOLVER_BICGSTAB if solver == "bicgstab" else mpg.SOLVER_CG
    ctx.configure(precision=prec, solver=kind, tol=1e-12, max_iter=3000, warm_start=0)
    rng = np.random.default_rng(11)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    b[m.node_pairs >= 0] = 0
    ctx.set_field(mpg.FIELD_RHS, b)
    ctx.solve()
    x = ctx.get_field(mpg.FIELD_PHI)
    m.assemble(1)
    ox, _, _ = orc.cg(m, b, tol=1e-13, max_iter=3000)
    assert np.abs(x - ox).max() <= 1e-9 * np.abs(ox).max()
    g = m.node_pairs >= 0
    assert (x[g] == x[m.node_pairs[g]]).all()


@pytest.mark.parametrize("jit", [0.2, 0.0])
def test_periodic_mg_solve_matches_oracle(mpg, orc, jit):
    # multigrid-preconditioned mixed solve on a 16^3 mesh periodic in x
    # (x coarsens plane by plane with wrap-around): the oracle's solution to
    # 1e-8, the ghost plane equal to its pair, far fewer iterations than the
    # plain inner CG, and bit-identical repeats
    n = 16
    m = orc.Mesh(n, split=6, lo=0.0, hi=1.0, mapping=4 if jit else 0, jitter=jit, seed=5, periodic=1)
    rng = np.random.default_rng(13)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    b[m.node_pairs >= 0] = 0

    def solve(kind):
        ctx = mpg.Ctx(0)
        ctx.mesh(n, split=6, lo=0.0, hi=1.0, mapping=4 if jit else 0, jitter=jit, seed=5, periodic=1)
        ctx.configure(precision=mpg.MIXED, solver=kind, tol=1e-11, max_iter=3000, warm_start=0)
        ctx.set_field(mpg.FIELD_RHS, b)
        it, _ = ctx.solve()
        return ctx.get_field(mpg.FIELD_PHI), it

    x, it_mg = solve(mpg.SOLVER_CG_MG)
    x2, it2 = solve(mpg.SOLVER_CG_MG)
    assert it2 == it_mg and (x2.view(np.uint64) == x.view(np.uint64)).all()
    m.assemble(1)
    ox, _, _ = orc.cg(m, b, tol=1e-13, max_iter=3000)
    assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()
    g = m.node_pairs >= 0
    assert (x[g] == x[m.node_pairs[g]]).all()
    _, it_cg = solve(mpg.SOLVER_CG)
    assert 2 * it_mg < it_cg, (it_mg, it_cg)


def test_periodic_mg_steps_track_plain(mpg):
    # the two counter-streaming beams of test_periodic_mixed_tracks_plain on a
    # 16^3 mesh, mixed form with the multigrid-preconditioned solver
    def make(prec, kind):
        ctx = mpg.Ctx(0)
        ctx.mesh(16, split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER, jitter=0.2, seed=3, periodic=1)
        ctx.configure(precision=prec, deposit=mpg.DEPOSIT_LINEAR, solver=kind, tol=1e-10, warm_start=2,
                      kill_on_wall=1, rho_background=1.0)
        n = 60000
        ctx.reserve(n)
        ctx.fill_uniform(n // 2, 1, 0, 1.0 / n, drift=(0.3, 0.0, 0.0), vth=0.02)
        ctx.fill_uniform(n // 2, 2, 0, 1.0 / n, drift=(-0.3, 0.0, 0.0), vth=0.02)
        return ctx
    mixed, plain = make(mpg.MIXED, mpg.SOLVER_CG_MG), make(mpg.PLAIN, mpg.SOLVER_CG)
    errs = []
    for s in range(5):
        sm = mixed.step(0.02, 1)
        sp = plain.step(0.02, 1)
        pm = mixed.get_field(mpg.FIELD_PHI)
        pp = plain.get_field(mpg.FIELD_PHI)
        errs.append(np.abs(pm - pp).max() / np.abs(pp).max())
        assert abs(sm.n_alive - sp.n_alive) <= 3
        assert sm.solver_iters < sp.solver_iters
    assert max(errs) <= 1e-6, errs


@pytest.mark.parametrize("mesh", [(4, 5, -1.0, 1.0, 0, 0.0), (6, 6, 0.0, 1.0, 4, 0.2)])
@pytest.mark.parametrize("kill", [1, 0])
def test_periodic_push_walk_resynced_bit_exact(mpg, orc, mesh, kill):
    # same state + same phi -> identical cells, exits, x, x_ref, v, with
    # particles crossing the periodic faces in both directions
    n_side, split, lo, hi, mapping, jit = mesh
    ctx, m = _pair(mpg, orc, n_side, split, lo, hi, mapping, jit, 8)
    ctx.configure(precision=mpg.PLAIN, solver=mpg.SOLVER_CG, deposit=mpg.DEPOSIT_LINEAR, kill_on_wall=kill,
                  track_ids=1)
    n = 30000
    ctx.reserve(n)
    ctx.fill_uniform(n, 21, 0, 1.0 / n, drift=(0.6 * (hi - lo), 0.0, 0.0), vth=0.2 * (hi - lo))
    d = ctx.download()
    P = orc.Particles(n)
    P.n = n
    for k in ("cell", "x", "xref", "v", "w", "sp", "id"):
        getattr(P, k)[:] = d[k]
    phi = 0.05 * np.random.default_rng(6).standard_normal(m.N)
    phi[m.boundary == 1] = 0
    g = m.node_pairs >= 0
    phi[g] = phi[m.node_pairs[g]]
    ctx.set_field(mpg.FIELD_PHI, phi)
    ctx.weight_efield()
    dt = 0.5
    st = ctx.move(dt)
    Et = m.efield_tet(phi)
    E = orc.gather(m, P, 1, phi, Et)
    orc.push(m, P, E, [-1.0], dt)
    x0 = P.x[:n, 0].copy()
    r = orc.walk(m, P, dt, kill=kill)
    assert st.n_killed == r["killed"]
    assert st.n_crossings == r["cross"]
    wrapped = int((np.abs(P.x[:n, 0] - x0) > 0.5 * (hi - lo))[P.cell[:n] >= 0].sum())
    assert wrapped > 100
    orc.compact(P, mode=1)
    gd = ctx.download()
    assert len(gd["cell"]) == P.n
    assert (gd["id"] == P.id[: P.n]).all()
    assert (gd["cell"] == P.cell[: P.n]).all()
    for k, a in (("x", P.x), ("xref", P.xref), ("v", P.v)):
        assert (gd[k].view(np.uint64) == a[: P.n].view(np.uint64)).all(), k


def test_periodic_mixed_charge_folds_onto_pairs(mpg, orc):
    # the fixed-point accumulator matches the oracle node by node (ghosts
    # included); the conversion moves ghost quanta onto their pairs exactly
    ctx, m = _pair(mpg, orc, 6, 6, 0.0, 1.0, 4, 0.2, 2)
    ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10)
    n = 40000
    ctx.reserve(n)
    ctx.fill_uniform(n, 4, 0, 1.0 / n, vth=0.1)
    acc, quantum, qfix = ctx.charge()
    cs, b, v = ctx.mixed_download()
    assert (acc == orc.deposit_fixed(m, cs, b, qfix)).all()
    g = np.nonzero(m.node_pairs >= 0)[0]
    assert np.abs(acc[g]).sum() > 0
    folded = acc.copy()
    folded[m.node_pairs[g]] += acc[g]
    folded[g] = 0
    live = cs != mpg.DEAD
    assert folded.sum() == int(qfix[0]) * int(live.sum())
    ctx.weight_charge()
    rhs = ctx.get_field(mpg.FIELD_RHS)
    want = -(folded.astype(np.float64) * quantum)
    want[m.boundary == 1] = 0.0
    want[g] = 0.0
    assert (rhs.view(np.uint64) == want.view(np.uint64)).all()


def test_periodic_mixed_tracks_plain(mpg):
    # two counter-streaming beams on a periodic jittered Kuhn mesh; both forms
    # from the same fill: phi within 1e-6 relative, same survivors
    def make(prec):
        ctx = mpg.Ctx(0)
        ctx.mesh(8, split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER, jitter=0.2, seed=3, periodic=1)
        ctx.configure(precision=prec, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10, warm_start=2,
                      kill_on_wall=1, rho_background=1.0)
        n = 40000
        ctx.reserve(n)
        ctx.fill_uniform(n // 2, 1, 0, 1.0 / n, drift=(0.3, 0.0, 0.0), vth=0.02)
        ctx.fill_uniform(n // 2, 2, 0, 1.0 / n, drift=(-0.3, 0.0, 0.0), vth=0.02)
        return ctx
    mixed, plain = make(mpg.MIXED), make(mpg.PLAIN)
    errs = []
    for s in range(5):
        sm = mixed.step(0.02, 1)
        sp = plain.step(0.02, 1)
        pm = mixed.get_field(mpg.FIELD_PHI)
        pp = plain.get_field(mpg.FIELD_PHI)
        errs.append(np.abs(pm - pp).max() / np.abs(pp).max())
        # a few particles on the y/z walls may exit in one form only (FP32 vs
        # FP64 exit test), so KE is compared per surviving particle
        assert abs(sm.n_alive - sp.n_alive) <= 3
        assert abs(sm.ke / sm.n_alive - sp.ke / sp.n_alive) <= 1e-5 * sp.ke / sp.n_alive
        assert sm.n_crossings > 0
    assert max(errs) <= 1e-6, errs


@pytest.mark.parametrize("yz", [(0.41, 0.57), (0.41, 0.96), (0.04, 0.93)])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_periodic_crossing_known_answer(mpg, orc, form, yz):
    # one particle at x = 0.97 moving +x by 0.1 with E = 0 ends at x = 0.07;
    # the last two start in cells whose x faces touch the y/z walls
    m = orc.Mesh(4, split=6, periodic=1)
    x0 = np.array([0.97, yz[0], yz[1]])
    for t in range(m.T):
        X = m.nodes[m.tets[t]]
        xr = np.linalg.solve((X[1:] - X[0]).T, x0 - X[0])
        if (xr >= 0).all() and xr.sum() <= 1:
            break
    ctx = mpg.Ctx(0)
    ctx.mesh(4, split=mpg.SPLIT_KUHN6, periodic=1)
    ctx.configure(precision=mpg.MIXED if form == "mixed" else mpg.PLAIN, deposit=mpg.DEPOSIT_LINEAR,
                  solver=mpg.SOLVER_CG, kill_on_wall=1)
    ctx.reserve(4)
    ctx.fill_uniform(1, 1, 0, 1.0, vth=0.0)  # sets the species weight; replaced below
    v = np.array([[0.1, 0.0, 0.0]])
    if form == "plain":
        ctx.upload(np.array([t], np.int32), x0[None], xr[None], v, w=np.ones(1), sp=np.zeros(1, np.int32))
    else:
        ctx.mixed_upload(np.array([t], np.uint32), xr[None].astype(np.float32), v.astype(np.float32))
    ctx.set_field(mpg.FIELD_PHI, np.zeros(m.N))
    ctx.weight_efield()
    st = ctx.move(1.0)
    assert st.n_killed == 0 and st.n_crossings >= 1
    if form == "plain":
        d = ctx.download()
        x = d["x"][0]
        tol = 1e-13
    else:
        cs, b, _ = ctx.mixed_download()
        cell = int(cs[0] & 0xFFFFFF)
        lam = np.array([1 - b[0].astype(np.float64).sum(), *b[0].astype(np.float64)])
        x = lam @ m.nodes[m.tets[cell]]
        tol = 2e-6
    assert np.allclose(x, [0.07, yz[0], yz[1]], atol=tol), x
