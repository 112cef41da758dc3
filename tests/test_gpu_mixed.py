"""GPU checks of the mixed form (FP32 push/walk, int64 fixed-point deposit,
FP32 CG inside FP64 refinement).

Bit-exact: fill positions (cell, barycentrics), the fixed-point charge
accumulator against the oracle's integer restatement, its invariance under
particle permutation, and the exact total charge.
Tolerance against the FP64 plain form on the same initial state: phi
relative error <= 1e-6 over the first steps (stated per check below).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(mpg, n_side=8, precision=None, jitter=0.2, **cfg):
    ctx = mpg.Ctx(0)
    ctx.mesh(n_side, split=mpg.SPLIT_KUHN6, lo=0.0, hi=1.0, mapping=mpg.MAP_JITTER if jitter else 0,
             jitter=jitter, seed=4)
    base = dict(precision=mpg.MIXED if precision is None else precision, deposit=mpg.DEPOSIT_LINEAR,
                solver=mpg.SOLVER_CG, tol=1e-10, warm_start=1, kill_on_wall=1)
    base.update(cfg)
    ctx.configure(**base)
    return ctx


def _two_species(ctx, n):
    ctx.species(0, -1.0, 1.0)
    ctx.species(1, 1.0, 100.0)
    ctx.reserve(2 * n)
    ctx.fill_uniform(n, 11, 0, 1.0 / n, vth=0.05)
    ctx.fill_uniform(n, 12, 1, 1.0 / n, vth=0.005)


def test_mixed_fill_positions_match_oracle(mpg, orc):
    ctx = _ctx(mpg)
    m = orc.Mesh(8, split=6, mapping=4, jitter=0.2, seed=4)
    n = 20000
    ctx.reserve(n)
    ctx.fill_uniform(n, 5, 0, 1.0 / n, drift=(0.2, 0, 0), vth=0.02)
    cs, b, v = ctx.mixed_download()
    P = orc.Particles(n)
    P.fill_uniform(m, n, 5, 0, 1.0 / n, drift=(0.2, 0, 0), vth=0.02)
    assert ((cs & 0xFFFFFF) == P.cell).all() and ((cs >> 24) == 0).all()
    assert (b == P.xref.astype(np.float32)).all()
    assert np.abs(v - P.v.astype(np.float32)).max() <= 8 * np.finfo(np.float32).eps * 0.3


def test_fixed_point_deposit_bit_exact_and_exact_charge(mpg, orc):
    ctx = _ctx(mpg)
    m = orc.Mesh(8, split=6, mapping=4, jitter=0.2, seed=4)
    _two_species(ctx, 30000)
    acc, quantum, qfix = ctx.charge()
    cs, b, v = ctx.mixed_download()
    oacc = orc.deposit_fixed(m, cs, b, qfix)
    assert (acc == oacc).all()
    live = cs != mpg.DEAD
    assert acc.sum() == sum(int(qfix[s]) for s in (cs[live] >> 24))
    # order independence: permute the particles and deposit again
    perm = np.random.default_rng(1).permutation(len(cs))
    ctx.mixed_upload(cs[perm], b[perm], v[perm])
    acc2, _, _ = ctx.charge()
    assert (acc2 == acc).all()


@pytest.mark.parametrize("n_side", [10, 56])
@pytest.mark.parametrize("jitter", [0.2, 0.0])
def test_mixed_solve_reaches_fp64_tolerance(mpg, orc, jitter, n_side):
    # jitter 0.2: stored FP32 operator with Jacobi scaling; jitter 0: uniform
    # mesh, constant-stencil FP32 operator.  56^3 has more rows than solver
    # threads, so the rows are walked along j with the register window.
    ctx = _ctx(mpg, n_side=n_side, warm_start=0, jitter=jitter)
    m = orc.Mesh(n_side, split=6, mapping=4 if jitter else 0, jitter=jitter, seed=4)
    m.assemble(1)
    rng = np.random.default_rng(7)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    ctx.set_field(mpg.FIELD_RHS, b)
    it, res = ctx.solve()
    x = ctx.get_field(mpg.FIELD_PHI)
    r = b - m.spmv(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-10
    ox, _, _ = orc.cg(m, b, tol=1e-12, max_iter=5000, nthreads=8)
    assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()


@pytest.mark.parametrize("n_side,split", [(16, 6), (24, 5), (56, 6), (31, 6), ((32, 19, 24), 6), (9, 6)])
@pytest.mark.parametrize("jitter", [0.2, 0.0])
def test_mg_preconditioned_solve_reaches_fp64_tolerance(mpg, orc, jitter, n_side, split):
    # the multigrid-preconditioned inner CG reaches the same FP64 tolerance
    # in far fewer iterations (31 cells per side: odd counts coarsen too); 9
    # cells per side are few enough (512 unknowns) to stay unpreconditioned
    def solve(kind):
        ctx = mpg.Ctx(0)
        ctx.mesh(n_side, split=split, lo=0.0, hi=1.0, mapping=mpg.MAP_JITTER if jitter else 0, jitter=jitter,
                 seed=4)
        ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=kind, tol=1e-10, warm_start=0)
        ctx.set_field(mpg.FIELD_RHS, b)
        it, _ = ctx.solve()
        return ctx.get_field(mpg.FIELD_PHI), it
    m = orc.Mesh(n_side, split=split, mapping=4 if jitter else 0, jitter=jitter, seed=4)
    m.assemble(1)
    rng = np.random.default_rng(7)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    x, it_mg = solve(mpg.SOLVER_CG_MG)
    x2, it2 = solve(mpg.SOLVER_CG_MG)
    assert it2 == it_mg and (x2.view(np.uint64) == x.view(np.uint64)).all()  # deterministic
    r = b - m.spmv(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-10
    ox, _, _ = orc.cg(m, b, tol=1e-12, max_iter=5000, nthreads=8)
    assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()
    _, it_cg = solve(mpg.SOLVER_CG)
    if n_side != 9:  # rectangular meshes coarsen per axis (19 cells: 20 -> 11 -> 6 nodes)
        assert 2 * it_mg < it_cg, (it_mg, it_cg)
    else:
        assert it_mg == it_cg


def test_mg_steps_track_plain_form(mpg):
    n = 40000
    mixed = _ctx(mpg, n_side=16, solver=mpg.SOLVER_CG_MG, warm_start=2)
    plain = _ctx(mpg, n_side=16, precision=mpg.PLAIN, warm_start=2)
    for c in (mixed, plain):
        _two_species(c, n)
    phis = []
    for s in range(5):
        sm = mixed.step(0.01, 1)
        sp = plain.step(0.01, 1)
        pm = mixed.get_field(mpg.FIELD_PHI)
        pp = plain.get_field(mpg.FIELD_PHI)
        phis.append(np.abs(pm - pp).max() / np.abs(pp).max())
        assert abs(sm.ke - sp.ke) <= 1e-5 * sp.ke
        assert abs(sm.n_alive - sp.n_alive) <= max(3, 1e-3 * n)
        assert sm.solver_iters < sp.solver_iters
    assert max(phis) <= 1e-6, phis


def test_mixed_steps_track_plain_form(mpg):
    n = 40000
    mixed = _ctx(mpg, n_side=8)
    plain = _ctx(mpg, n_side=8, precision=mpg.PLAIN)
    for c in (mixed, plain):
        _two_species(c, n)
    phis = []
    for s in range(5):
        sm = mixed.step(0.01, 1)
        sp = plain.step(0.01, 1)
        pm = mixed.get_field(mpg.FIELD_PHI)
        pp = plain.get_field(mpg.FIELD_PHI)
        err = np.abs(pm - pp).max() / np.abs(pp).max()
        phis.append(err)
        assert abs(sm.ke - sp.ke) <= 1e-5 * sp.ke
        assert abs(sm.n_alive - sp.n_alive) <= max(3, 1e-3 * n)
    assert max(phis) <= 1e-6, phis


def test_mixed_sort_orders_cells_and_drops_dead(mpg):
    ctx = _ctx(mpg, n_side=6, sort_interval=0)
    n = 20000
    ctx.reserve(n)
    ctx.fill_uniform(n, 8, 0, 1.0 / n, vth=0.5)
    ctx.step(0.05, 1)
    cs0, b0, v0 = ctx.mixed_download()
    live0 = cs0 != mpg.DEAD
    ctx.sort()
    cs, b, v = ctx.mixed_download()
    assert len(cs) == live0.sum()
    assert (np.diff((cs & 0xFFFFFF).astype(np.int64)) >= 0).all()
    key0 = np.sort(np.round(b0[live0].astype(np.float64) * 1e7).sum(axis=1))
    key = np.sort(np.round(b.astype(np.float64) * 1e7).sum(axis=1))
    assert (key0 == key).all()
    assert ctx.count() == len(cs)


def test_mixed_walk_known_answer(mpg):
    # one particle moving along +x for one step through a uniform Kuhn mesh
    ctx = _ctx(mpg, n_side=4, jitter=0.0, kill_on_wall=1)
    ctx.reserve(1)
    ctx.fill_uniform(1, 1, 0, 1.0, vth=0.0)
    cs, b, v = ctx.mixed_download()
    ctx.species(0, 0.0, 1.0)  # no force
    v = np.array([[0.1, 0.0, 0.0]], np.float32)
    ctx.mixed_upload(cs, b, v)
    d0 = ctx.download()
    x0 = d0["x"][0]
    st = ctx.move(1.0)
    d = ctx.download()
    if x0[0] + 0.1 < 1.0:
        assert st.n_killed == 0
        assert np.allclose(d["x"][0], x0 + [0.1, 0, 0], atol=2e-6)
    else:
        assert st.n_killed == 1


def test_mixed_upload_rejects_bad_words_and_keeps_state(mpg):
    # the upload is validated on the device before it replaces the resident
    # state: a cell out of range is an argument error, a species without a
    # weight a state error, and a rejected upload changes nothing
    ctx = _ctx(mpg, n_side=4)
    ctx.reserve(1000)
    ctx.fill_uniform(1000, 3, 0, 1e-3, vth=0.05)
    cs, b, v = ctx.mixed_download()
    n0 = ctx.count()
    bad = cs.copy()
    bad[777] = (bad[777] & 0xFF000000) | ctx.T  # cell index = T
    with pytest.raises(mpg.MpgError) as e:
        ctx.mixed_upload(bad, b, v)
    assert e.value.code == mpg.ERR_ARG and "777" in str(e.value)
    bad = cs.copy()
    bad[5] = (5 << 24) | (bad[5] & 0xFFFFFF)  # species 5 has no weight
    bad[9] = (bad[9] & 0xFF000000) | ctx.T
    with pytest.raises(mpg.MpgError) as e:
        ctx.mixed_upload(bad, b, v)
    assert e.value.code == mpg.ERR_STATE  # lowest bad index (5) is reported
    assert ctx.count() == n0
    cs2, b2, v2 = ctx.mixed_download()
    assert (cs2 == cs).all() and (b2.view(np.uint32) == b.view(np.uint32)).all()
    dead = cs.copy()
    dead[::3] = mpg.DEAD
    ctx.mixed_upload(dead, b, v)
    assert ctx.count() == int((dead != mpg.DEAD).sum())
    out = (np.empty_like(cs), np.empty_like(b), np.empty_like(v))
    cs3, b3, v3 = ctx.mixed_download(out=out)
    assert cs3.base is out[0] or cs3 is out[0]
    assert (cs3 == dead).all() and (b3.view(np.uint32) == b.view(np.uint32)).all()


@pytest.mark.parametrize("ws", [2, 3])
@pytest.mark.parametrize("form", ["mixed", "plain"])
def test_extrapolated_initial_guess_same_solution(mpg, form, ws):
    # warm_start 2 starts each solve at 2 phi[n-1] - phi[n-2]; the converged
    # phi must agree with the previous-phi start to the solver tolerance
    # (both stop at |b - A x| <= 1e-10 |b|; phi differences stay below
    # 1e-8 max|phi| over the first steps), and KE to 1e-9 relative
    n = 40000
    prec = mpg.MIXED if form == "mixed" else mpg.PLAIN
    a = _ctx(mpg, n_side=8, precision=prec, warm_start=1)
    b = _ctx(mpg, n_side=8, precision=prec, warm_start=ws)
    for c in (a, b):
        _two_species(c, n)
    ia = ib = 0
    for s in range(6):
        sa = a.step(0.01, 1)
        sb = b.step(0.01, 1)
        pa = a.get_field(mpg.FIELD_PHI)
        pb = b.get_field(mpg.FIELD_PHI)
        assert np.abs(pa - pb).max() <= 1e-8 * np.abs(pa).max(), s
        assert abs(sa.ke - sb.ke) <= 1e-9 * sa.ke
        assert sa.n_alive == sb.n_alive
        if s >= 2:
            ia += sa.solver_iters
            ib += sb.solver_iters
    # the extrapolated start is closer: never more iterations in total
    assert ib <= ia, (ia, ib)


@pytest.mark.parametrize("shape", [12, (10, 7, 13)])
def test_kuhn_table_walk_equals_per_tet_records(mpg, monkeypatch, shape):
    """On a uniform Kuhn mesh the mixed walk reads J^-1 and the neighbours from
    the 6-type table and E is formed per hex; against the per-tet records
    (MPG_KUHN_WALK=0) the state, the per-node charge, phi, E and the counts
    after several steps with many crossings and wall exits are bit-identical
    (a cube, and a box with three different cell counts)."""
    runs = []
    for kw in ("1", "0"):
        monkeypatch.setenv("MPG_KUHN_WALK", kw)
        ctx = mpg.Ctx(0)
        ctx.mesh(shape, split=mpg.SPLIT_KUHN6)
        ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG_MG, tol=1e-10,
                      warm_start=2, kill_on_wall=1, sort_interval=3, rho_background=1.0)
        n = 60000
        ctx.reserve(n)
        ctx.fill_uniform(n // 2, 4, 0, 1.0 / n, drift=(0.3, 0, 0), vth=0.1)
        ctx.fill_uniform(n // 2, 5, 0, 1.0 / n, drift=(-0.3, 0, 0), vth=0.1)
        sts = [ctx.step(0.02, 1) for _ in range(7)]
        runs.append((ctx.mixed_download() + (ctx.charge()[0],), ctx.get_field(mpg.FIELD_PHI),
                     ctx.get_field(mpg.FIELD_E_TET), [(s.n_alive, s.n_crossings, s.n_killed) for s in sts]))
        ctx.close()
    (a, pa, ea, ca), (b, pb, eb, cb) = runs
    assert ca == cb and sum(k for _, _, k in ca) > 0 and sum(c for _, c, _ in ca) > 0
    for u, v in zip(a, b):
        assert (u.view(np.uint8) == v.view(np.uint8)).all()
    assert (pa.view(np.uint64) == pb.view(np.uint64)).all()
    assert (ea.view(np.uint64) == eb.view(np.uint64)).all()


@pytest.mark.parametrize("n_side,n", [(12, 40000), (40, 400000)])
def test_kuhn_move_deposit_matches_oracle(mpg, orc, n_side, n):
    """The fused move deposits the new positions (warp runs into per-(cell,
    corner) slots, walk on the 6-type Kuhn table with the multiply-shift hex
    split); after steps with crossings, wall exits and a sort in between,
    the per-node charge equals the oracle's fixed-point deposit of the
    particle state, bit for bit."""
    ctx = mpg.Ctx(0)
    ctx.mesh(n_side, split=mpg.SPLIT_KUHN6)
    ctx.configure(precision=mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG_MG, tol=1e-10,
                  warm_start=2, kill_on_wall=1, sort_interval=2, rho_background=1.0)
    ctx.reserve(n)
    ctx.fill_uniform(n // 2, 7, 0, 1.0 / n, drift=(0.4, 0, 0), vth=0.1)
    ctx.fill_uniform(n // 2, 8, 0, 1.0 / n, drift=(-0.4, 0, 0), vth=0.1)
    m = orc.Mesh(n_side, split=6)
    killed = 0
    for _ in range(3):
        st = ctx.step(0.02, 1)
        killed += st.n_killed
        acc, quantum, qfix = ctx.charge()
        cs, b, v = ctx.mixed_download()
        assert (acc == orc.deposit_fixed(m, cs, b, qfix)).all()
    assert killed > 0
    ctx.close()


def test_mixed_upload_download_from_mapped_host_memory(mpg):
    """Page-locked mapped host buffers (cudaHostAlloc, here through torch's
    pinned allocator) are validated, packed and unpacked by the device
    directly over the host link: the same particle state as through staged
    copies of pageable buffers, and a rejected upload (a cell out of range)
    leaves the resident state unchanged."""
    torch = pytest.importorskip("torch")
    ctx = _ctx(mpg, n_side=10, jitter=0.0)
    n = 50000
    ctx.reserve(n)
    ctx.fill_uniform(n, 9, 0, 1.0 / n, drift=(0.2, 0, 0), vth=0.05)
    ctx.step(0.01, 2)
    cs, b, v = ctx.mixed_download()

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(a.dtype).reshape(a.shape)
        np.copyto(t, a)
        return t

    pc, pb, pv = pinned(cs), pinned(b), pinned(v)
    out = tuple(pinned(np.zeros_like(a)) for a in (cs, b, v))
    c2, b2, v2 = ctx.mixed_download(out=out)
    assert (c2 == cs).all() and (b2 == b).all() and (v2 == v).all()
    bad = pinned(cs)
    bad[123] = (bad[123] & 0xFF000000) | 0xFFFFF0
    with pytest.raises(mpg.MpgError):
        ctx.mixed_upload(bad, pb, pv)
    c3, b3, v3 = ctx.mixed_download()
    assert (c3 == cs).all() and (b3 == b).all() and (v3 == v).all()
    # a modified state goes in through the mapped buffers and comes back the same
    pb[:, 0] *= 0.5
    ctx.mixed_upload(pc, pb, pv)
    acc_mapped = ctx.charge()[0]  # deposited by the upload's own pass
    c4, b4, v4 = ctx.mixed_download()
    assert (c4 == pc).all() and (b4 == pb).all() and (v4 == pv).all()
    # and steps on exactly as the same state uploaded from pageable copies
    ctx.mixed_upload(pc, pb, pv)
    ctx.step(0.01, 1)
    c5, b5, v5 = ctx.mixed_download(out=out)
    ctx.mixed_upload(np.array(pc), np.array(pb), np.array(pv))
    assert (ctx.charge()[0] == acc_mapped).all()  # deposited by the deposit kernel
    ctx.step(0.01, 1)
    c6, b6, v6 = ctx.mixed_download()
    assert (c5 == c6).all() and (b5 == b6).all() and (v5 == v6).all()
    ctx.close()
