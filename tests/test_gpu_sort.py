"""GPU checks of the stable cell sort (ParticleList::sort and
compute_start_particles_by_element, particle_list.cpp:90-146).

Bit-exact against the oracle's std::stable_sort by cell (dead particles
dropped): the permutation of the particle list, every record moved with its
particle, and the start offsets per cell.  Inside a cell the list keeps its
input order, so on a fill whose list is in id order the result is the
(cell, id) order, and the same on every run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(mpg, precision, n_side=8, jitter=0.0, **cfg):
    ctx = mpg.Ctx(0)
    ctx.mesh(n_side, split=mpg.SPLIT_KUHN6, mapping=mpg.MAP_JITTER if jitter else mpg.MAP_NONE, jitter=jitter,
             seed=3)
    base = dict(precision=precision, deposit=mpg.DEPOSIT_LINEAR, solver=mpg.SOLVER_CG, tol=1e-10, warm_start=1,
                kill_on_wall=1, sort_interval=0, track_ids=1, rho_background=1.0)
    base.update(cfg)
    ctx.configure(**base)
    return ctx


@pytest.mark.parametrize("form", ["mixed", "plain"])
def test_sort_permutation_matches_oracle_stable_sort(mpg, orc, form):
    precision = mpg.MIXED if form == "mixed" else mpg.PLAIN
    ctx = _ctx(mpg, precision, jitter=0.2)
    n = 40000
    ctx.reserve(n)
    ctx.fill_uniform(n, 21, 0, 1.0 / n, vth=0.3)
    # after a few steps the list is out of cell order and (mixed) holds dead slots
    ctx.step(0.02, 3)
    before = ctx.download()
    perm, start = orc.sort_by_cell(before["cell"], ctx.T)
    ctx.sort()
    after = ctx.download()
    assert len(after["cell"]) == len(perm) == ctx.count()
    assert (after["id"] == before["id"][perm]).all()
    assert (after["cell"] == before["cell"][perm]).all()
    for k in ("x", "xref", "v", "w", "sp"):
        assert (after[k] == before[k][perm]).all(), k
    assert (ctx.cell_starts() == start).all()


def test_sort_of_a_fresh_fill_is_cell_then_id_order(mpg, orc):
    ctx = _ctx(mpg, mpg.MIXED, n_side=6)
    n = 30000
    ctx.reserve(n)
    ctx.fill_uniform(n, 5, 0, 1.0 / n, vth=0.05)
    ctx.sort()
    d = ctx.download()
    order = np.lexsort((d["id"], d["cell"]))
    assert (order == np.arange(len(order))).all()
    assert (np.sort(d["id"]) == np.arange(n)).all()


def test_sort_long_cell_ranges_and_repeatability(mpg, orc):
    """Cells holding more particles than one thread sorts (a 9000-particle
    cell spans three shared-memory tiles and two merge passes) and a
    shuffled input with dead slots: the mixed form keeps every cell's input
    order, bit for bit, on two runs."""
    ctx = _ctx(mpg, mpg.MIXED, n_side=4)
    T = ctx.T
    rng = np.random.default_rng(8)
    n = 20000
    cells = rng.integers(0, T, n).astype(np.uint32)
    cells[rng.choice(n, 9000, replace=False)] = 7
    cells[rng.choice(n, 600, replace=False)] = 11
    dead = rng.choice(n, 500, replace=False)
    cs = cells.copy()
    cs[dead] = mpg.DEAD
    b = np.full((n, 3), 0.25, np.float32)
    v = np.zeros((n, 3), np.float32)
    v[:, 0] = np.arange(n, dtype=np.float32)  # the input index, exact in FP32 below 2^24
    ctx.species(0, -1.0, 1.0)
    ctx.reserve(n)
    ctx.fill_uniform(1, 1, 0, 1.0, vth=0.0)  # gives species 0 its weight
    cell_oracle = np.where(cs == mpg.DEAD, -1, cs.astype(np.int64)).astype(np.int32)
    perm, start = orc.sort_by_cell(cell_oracle, T)
    runs = []
    for _ in range(2):
        ctx.mixed_upload(cs, b, v)
        ctx.sort()
        cs2, b2, v2 = ctx.mixed_download()
        runs.append((cs2.copy(), v2.copy()))
        assert (v2[:, 0].astype(np.int64) == perm).all()
        assert (cs2 == cs[perm]).all()
        assert (ctx.cell_starts() == start).all()
    assert (runs[0][0] == runs[1][0]).all() and (runs[0][1] == runs[1][1]).all()


def test_sort_gather_fused_into_next_move(mpg):
    """mpg_step leaves the gather of its cell sort to the next move, which
    reads the particles through the permutation into the other buffer; any
    other use of the list completes the gather first.  Nine steps in one call
    (sorts after steps 3 and 6 fused into the moves of steps 4 and 7) equal
    nine single steps with a download after each (every gather completed on
    its own), bit for bit: particle state, charge, phi."""
    runs = []
    for single in (False, True):
        ctx = _ctx(mpg, mpg.MIXED, n_side=10, jitter=0.2, sort_interval=3, track_ids=1)
        n = 60000
        ctx.reserve(n)
        ctx.fill_uniform(n // 2, 41, 0, 1.0 / n, drift=(0.3, 0, 0), vth=0.1)
        ctx.fill_uniform(n // 2, 42, 0, 1.0 / n, drift=(-0.3, 0, 0), vth=0.1)
        if single:
            for _ in range(9):
                ctx.step(0.02, 1)
                ctx.mixed_download()
        else:
            ctx.step(0.02, 9)
        runs.append((ctx.mixed_download(), ctx.download()["id"], ctx.charge()[0], ctx.get_field(mpg.FIELD_PHI)))
        ctx.close()
    (a, ida, qa, pa), (b, idb, qb, pb) = runs
    for u, v in zip(a, b):
        assert (u.view(np.uint8) == v.view(np.uint8)).all()
    assert (ida == idb).all() and (qa == qb).all()
    assert (pa.view(np.uint64) == pb.view(np.uint64)).all()


def test_step_sort_counts_from_the_move_equal_a_separate_sort(mpg):
    """A step that ends with a cell sort takes the sort's particles per cell
    from the move's deposit runs instead of a counting pass: three steps
    with sort_interval=3 (sorted before step 1 and after step 3) equal, bit
    for bit, a sort, three unsorted steps and a sort by mpg_sort (its own
    counting pass): the permutation (ids), every record, the cell starts and
    the charge."""
    runs = []
    for fused in (True, False):
        ctx = _ctx(mpg, mpg.MIXED, n_side=10, jitter=0.2, sort_interval=3 if fused else 0, track_ids=1)
        n = 60000
        ctx.reserve(n)
        ctx.fill_uniform(n // 2, 51, 0, 1.0 / n, drift=(0.3, 0, 0), vth=0.2)
        ctx.fill_uniform(n // 2, 52, 0, 1.0 / n, drift=(-0.3, 0, 0), vth=0.2)
        if fused:
            ctx.step(0.02, 3)
        else:
            ctx.sort()
            ctx.step(0.02, 3)
            ctx.sort()
        runs.append((ctx.mixed_download(), ctx.download()["id"], ctx.cell_starts(), ctx.charge()[0]))
        ctx.close()
    (a, ida, sa, qa), (b, idb, sb, qb) = runs
    assert len(ida) == len(idb)
    for u, v in zip(a, b):
        assert (u.view(np.uint8) == v.view(np.uint8)).all()
    assert (ida == idb).all() and (sa == sb).all() and (qa == qb).all()
