"""CPU tests of the oracle: pins against the reference's own code and invariants.

The reference ships no tests.  What pins the oracle:
  * golden vectors from the reference's random.hpp compiled here
    (tests/golden/ref_random.json, made by tests/golden/make_golden.py);
  * the reference's own assert() invariants of the mesh generator
    (mesh.cpp:163,171,119-120,278,399,641-647,692);
  * closed-form answers (P1 patch test, single-particle walks, charge sums).
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_random.json")


@pytest.fixture(scope="module")
def gold():
    with open(GOLD) as f:
        return json.load(f)


def test_lcg_matches_reference_random_hpp(orc, gold):
    for case in gold["lcg"]:
        r, d = orc.ref_lcg(case["seed"], 8)
        assert [int(x) for x in r] == case["rand"]
        assert [int(x) for x in d.view(np.uint64)] == case["drand_bits"]


@pytest.mark.parametrize("ng,split,n", [(6000, 6, 10), (5000, 5, 10), (40, 5, 2)])
def test_fill_seed_and_rejection_match_reference(orc, gold, ng, split, n):
    # particle_fill.hpp:147-156: seed per (elem, ipart, type), 10 burned draws, x_ref rejection
    m = orc.Mesh(n, split=split, lo=-1.0, hi=1.0)
    assert m.T == ng
    cases = [c for c in gold["fill"] if c["n_global_elem"] == ng]
    assert cases
    nppe = max(c["ipart"] for c in cases) + 1
    for typ in sorted({c["type"] for c in cases}):
        P = orc.Particles(m.T * nppe)
        P.fill_ref(m, nppe, typ, 1.0, temp=0.0)
        for c in (c for c in cases if c["type"] == typ):
            k = c["elem"] * nppe + c["ipart"]
            assert P.cell[k] == c["elem"]
            assert [int(x) for x in P.xref[k].view(np.uint64)] == c["xref_bits"]


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_mesh_counts_match_reference_asserts(orc, n):
    m = orc.Mesh(n, split=5, lo=-1.0, hi=1.0)
    nx = ny = nz = n
    assert m.T == 5 * nx * ny * nz                                   # mesh.cpp:163
    assert m.N == (nx + 1) * (ny + 1) * (nz + 1)                     # mesh.cpp:171
    assert m.n_faces == 4 * nx * ny * nz + 2 * (nx * ny * (nz + 1) + nx * (ny + 1) * nz + (nx + 1) * ny * nz)
    assert m.n_bfaces == 2 * (2 * nx * ny + 2 * nx * nz + 2 * ny * nz)  # mesh.cpp:641
    assert (m.detj > 0).all()                                        # mesh.cpp:692
    # every interior face is shared by exactly two tets, symmetrically (mesh.cpp:399-404)
    nb = m.nbrs
    assert (nb >= -1).all()
    for t in range(m.T):
        for f in range(4):
            o = nb[t, f]
            if o >= 0:
                assert t in nb[o]
    assert (nb == -1).sum() == m.n_bfaces


@pytest.mark.parametrize("n", [1, 3, 4])
def test_kuhn_mesh_invariants(orc, n):
    m = orc.Mesh(n, split=6)
    assert m.T == 6 * n ** 3 and m.N == (n + 1) ** 3
    assert m.n_faces == 6 * n ** 3 + 2 * 3 * n * n * (n + 1)
    assert m.n_bfaces == 2 * 6 * n * n
    assert np.allclose(m.detj, (1.0 / n) ** 3)
    assert abs(m.detj.sum() / 6 - 1.0) < 1e-12


def test_jittered_mesh_positive_and_volume_preserving(orc):
    m = orc.Mesh(12, split=6, mapping=4, jitter=0.2, seed=7)
    assert (m.detj > 0).all()
    assert abs(m.detj.sum() / 6 - 1.0) < 1e-12
    # boundary nodes do not move
    b = m.boundary.astype(bool)
    g = np.round(m.nodes[b] * 12)
    assert np.allclose(m.nodes[b] * 12, g)


def test_reference_mappings_build(orc):
    for mp in (1, 2, 3):
        m = orc.Mesh(4, split=5, lo=-1, hi=1, mapping=mp)
        assert (m.detj > 0).all()


def test_p1_patch_test(orc):
    # a linear field is reproduced exactly: (A u)_i = 0 at interior nodes for linear u
    m = orc.Mesh(6, split=6, mapping=4, jitter=0.15, seed=3)
    m.assemble(0)
    u = 0.3 + 1.7 * m.nodes[:, 0] - 0.4 * m.nodes[:, 1] + 2.2 * m.nodes[:, 2]
    y = m.spmv(u)
    inner = m.boundary == 0
    assert np.abs(y[inner]).max() < 1e-12
    # the per-tet E of a linear phi is its exact gradient
    E = m.efield_tet(u)
    assert np.allclose(E, [1.7, -0.4, 2.2], atol=1e-10)


def test_cg_matches_scipy(orc):
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    m = orc.Mesh(8, split=6, mapping=4, jitter=0.2, seed=11)
    rp, col, val = m.assemble(1)
    A = sp.csr_matrix((val, col, rp), shape=(m.N, m.N))
    rng = np.random.default_rng(0)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    x, it, res = orc.cg(m, b, tol=1e-12)
    xs = spl.spsolve(A.tocsc(), b)
    assert res < 1e-12
    assert np.abs(x - xs).max() / np.abs(xs).max() < 1e-9
    assert abs(A - A.T).max() < 1e-14 * abs(A).max()  # symmetric form


def test_bicgstab_reference_solves(orc):
    m = orc.Mesh(5, split=5, lo=-1, hi=1)
    m.assemble(0)
    rng = np.random.default_rng(1)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    x, it, res = orc.bicgstab(m, b, tol=1e-6)
    r = b - m.spmv(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-6
    assert res < 1e-6


def test_deposit_charge_conservation(orc):
    m = orc.Mesh(5, split=6)
    P = orc.Particles(5000)
    P.fill_uniform(m, 5000, 3, 0, 2e-4, vth=0.1)
    for mode in (0, 1):
        rhs_full = orc.deposit(m, P, mode, [-1.0])
        # undo the Dirichlet zeroing by depositing with no boundary: compare sums via cell nodes
        assert rhs_full.shape == (m.N,)
    # linear deposit, no Dirichlet: total = -sum w q
    tot = 0.0
    for p in range(P.n):
        tot += -(P.w[p] * -1.0)
    rhs = orc.deposit(m, P, 1, [-1.0])
    inner = m.boundary == 0
    # interior sum plus the zeroed boundary part equals the total; check fixed-point exactness instead
    cs = (P.cell[: P.n].astype(np.uint32)) | np.uint32(0)
    b = P.xref[: P.n].astype(np.float32)
    acc = orc.deposit_fixed(m, cs, b, [123456789])
    assert acc.sum() == 123456789 * P.n
    assert np.isfinite(rhs[inner]).all()


def test_fixed_point_deposit_order_independent(orc):
    m = orc.Mesh(4, split=6)
    P = orc.Particles(3000)
    P.fill_uniform(m, 3000, 5, 0, 1.0)
    cs = P.cell[: P.n].astype(np.uint32)
    b = P.xref[: P.n].astype(np.float32)
    a1 = orc.deposit_fixed(m, cs, b, [1 << 30])
    perm = np.random.default_rng(2).permutation(P.n)
    a2 = orc.deposit_fixed(m, cs[perm], b[perm], [1 << 30])
    assert (a1 == a2).all()
    assert a1.sum() == (1 << 30) * P.n


def _single(orc, m, cell, xref, v):
    P = orc.Particles(1)
    P.n = 1
    P.cell[0] = cell
    P.xref[0] = xref
    lam = np.array([1 - sum(xref), *xref])
    P.x[0] = lam @ m.nodes[m.tets[cell]]
    P.v[0] = v
    P.w[0] = 1.0
    return P


def test_walk_straight_line_known_answer(orc):
    # a particle moving along +x through a uniform Kuhn mesh ends at x0 + v dt
    m = orc.Mesh(4, split=6)
    P = orc.Particles(1)
    x0 = np.array([0.13, 0.41, 0.57])
    v = np.array([0.5, 0.0, 0.0])
    # locate the tet: barycentric coordinates all >= 0
    for t in range(m.T):
        X = m.nodes[m.tets[t]]
        J = (X[1:] - X[0]).T
        xr = np.linalg.solve(J, x0 - X[0])
        if (xr >= 0).all() and xr.sum() <= 1:
            break
    P = _single(orc, m, t, xr, v)
    orc.push(m, P, np.zeros((1, 3)), [-1.0], 1.0)
    r = orc.walk(m, P, 1.0, kill=1)
    assert r["killed"] == 0 and r["limit"] == 0
    assert np.allclose(P.x[0], x0 + v, atol=1e-13)
    X = m.nodes[m.tets[P.cell[0]]]
    lam = np.array([1 - P.xref[0].sum(), *P.xref[0]])
    assert np.allclose(lam @ X, P.x[0], atol=1e-13)
    assert r["cross"] >= 2


def test_walk_wall_kill_and_reflect(orc):
    m = orc.Mesh(3, split=6)
    x0 = np.array([0.9, 0.5, 0.5])
    for t in range(m.T):
        X = m.nodes[m.tets[t]]
        xr = np.linalg.solve((X[1:] - X[0]).T, x0 - X[0])
        if (xr >= -1e-15).all() and xr.sum() <= 1 + 1e-15:
            break
    v = np.array([0.2, 0.0, 0.0])
    P = _single(orc, m, t, xr, v)
    orc.push(m, P, np.zeros((1, 3)), [-1.0], 1.0)
    r = orc.walk(m, P, 1.0, kill=1)
    assert r["killed"] == 1 and P.cell[0] == -1
    assert abs(P.x[0, 0] - 1.0) < 1e-13  # stopped on the wall
    P = _single(orc, m, t, xr, v)
    orc.push(m, P, np.zeros((1, 3)), [-1.0], 1.0)
    r = orc.walk(m, P, 1.0, kill=0)
    assert r["killed"] == 0
    assert np.allclose(P.v[0], [-0.2, 0, 0], atol=1e-15)
    assert np.allclose(P.x[0], [0.9, 0.5, 0.5], atol=1e-13)  # 0.1 to the wall, 0.1 back


def test_compaction_modes(orc):
    P = orc.Particles(10)
    P.n = 10
    P.cell[:10] = [0, -1, 2, -1, 4, 5, -1, 7, 8, -1]
    P.id[:10] = np.arange(10)
    P2 = orc.Particles(10)
    P2.n = 10
    P2.cell[:] = P.cell
    P2.id[:] = P.id
    orc.compact(P, mode=1)
    assert list(P.id[: P.n]) == [0, 2, 4, 5, 7, 8]
    orc.compact(P2, mode=0)
    # tail fill: hole 1 <- 8, hole 3 <- 7, hole 6 >= new count: skipped
    assert sorted(P2.id[: P2.n]) == [0, 2, 4, 5, 7, 8]
    assert list(P2.id[: P2.n]) == [0, 8, 2, 7, 4, 5]


def test_sort_by_cell_known_answer(orc):
    # ParticleList::sort + compute_start_particles_by_element: stable by cell,
    # dead (-1) dropped, start = lower_bound of each element (particle_list.cpp:118-133)
    cell = np.array([3, 1, -1, 1, 0, 3, 2, -1, 1], np.int32)
    perm, start = orc.sort_by_cell(cell, 5)
    assert perm.tolist() == [4, 1, 3, 8, 6, 0, 5]
    assert start.tolist() == [0, 1, 4, 5, 7, 7]
    rng = np.random.default_rng(3)
    cell = rng.integers(-1, 50, 5000).astype(np.int32)
    perm, start = orc.sort_by_cell(cell, 50)
    live = np.flatnonzero(cell >= 0)
    assert (perm == live[np.argsort(cell[live], kind="stable")]).all()
    assert (start == np.searchsorted(cell[perm], np.arange(51), side="left")).all()


def test_gather_ref_vs_per_tet(orc):
    # the reference's 48-term gather equals E_tet * sum(lambda): a few ulp apart
    m = orc.Mesh(6, split=6, mapping=4, jitter=0.2, seed=5)
    rng = np.random.default_rng(4)
    phi = rng.standard_normal(m.N)
    P = orc.Particles(2000)
    P.fill_uniform(m, 2000, 9, 0, 1.0)
    Et = m.efield_tet(phi)
    E0 = orc.gather(m, P, 0, phi)
    E1 = orc.gather(m, P, 1, phi, Et)
    scale = np.abs(E1).max()
    assert np.abs(E0 - E1).max() <= 64 * np.finfo(float).eps * scale


def test_full_step_runs_and_conserves(orc):
    m = orc.Mesh(6, split=6)
    m.assemble(1)
    n = 20000
    P = orc.Particles(n)
    P.fill_uniform(m, n, 1, 0, 1.0 / n, vth=0.05)
    bg = m.background(1.0)
    phi = np.zeros(m.N)
    cfg = orc.StepCfg(1, 1, 1e-10, 1000, 1, 1, 1, 1000, 1, 1)
    ke0 = orc.kinetic(P, [1.0])
    for _ in range(3):
        rc, st, rhs = orc.step(m, P, cfg, 0.01, [-1.0], [1.0], bg, phi)
        assert rc == 0 and st.solver_resid < 1e-10
    assert P.n == st.n_alive and P.n <= n
    assert 0.5 * ke0 < st.ke < 2 * ke0


# ---------------------------------------------------------------------------
# periodic-in-x meshes (the reference's --problem two-stream set-up)
@pytest.mark.parametrize("split,n,lo,hi", [(5, 4, -1.0, 1.0), (6, 3, 0.0, 1.0), (6, (4, 3, 5), 0.0, 1.0)])
def test_periodic_mesh_invariants(orc, split, n, lo, hi):
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    m = orc.Mesh(n, split=split, lo=lo, hi=hi, periodic=1)
    per_hex = 4 if split == 5 else 6
    # mesh.cpp:119-120: the x = hi faces are merged with the x = lo faces
    total = per_hex * nx * ny * nz + 2 * (nx * ny * (nz + 1) + nx * (ny + 1) * nz + (nx + 1) * ny * nz) - 2 * ny * nz
    assert m.n_faces == total
    assert m.n_bfaces == 4 * nx * (ny + nz)          # only the y and z walls
    g = np.arange(m.N)
    i, j, k = g // ((ny + 1) * (nz + 1)), (g // (nz + 1)) % (ny + 1), g % (nz + 1)
    bnd = (j == 0) | (j == ny) | (k == 0) | (k == nz)
    assert (m.boundary == bnd).all()
    ghost = (i == nx) & ~bnd
    assert (m.node_pairs[ghost] == g[ghost] - nx * (ny + 1) * (nz + 1)).all()
    assert (m.node_pairs[~ghost] == -1).all()
    # neighbours are mutual, including across the periodic faces
    for t in range(m.T):
        for f in range(4):
            b = m.nbrs[t, f]
            if b >= 0:
                assert t in m.nbrs[b]
    # both sides of every x-plane triangle are flagged (mesh.cpp:369-392)
    assert (m.face_periodic != 0).sum() == 2 * 2 * ny * nz
    assert (m.nbrs[m.face_periodic != 0] >= 0).all()


def test_periodic_five_tet_needs_even_nx(orc):
    with pytest.raises(ValueError):
        orc.Mesh(3, split=5, lo=-1.0, hi=1.0, periodic=1)


def test_periodic_walk_wraps_known_answer(orc):
    # crossing x = hi reappears at x = lo (particle_move.hpp:190-191)
    m = orc.Mesh(4, split=6, periodic=1)
    x0 = np.array([0.97, 0.41, 0.57])
    for t in range(m.T):
        X = m.nodes[m.tets[t]]
        xr = np.linalg.solve((X[1:] - X[0]).T, x0 - X[0])
        if (xr >= 0).all() and xr.sum() <= 1:
            break
    P = _single(orc, m, t, xr, np.array([0.1, 0.0, 0.0]))
    orc.push(m, P, np.zeros((1, 3)), [-1.0], 1.0)
    r = orc.walk(m, P, 1.0, kill=1)
    assert r["killed"] == 0 and r["limit"] == 0
    assert np.allclose(P.x[0], [0.07, 0.41, 0.57], atol=1e-13)
    X = m.nodes[m.tets[P.cell[0]]]
    lam = np.array([1 - P.xref[0].sum(), *P.xref[0]])
    assert np.allclose(lam @ X, P.x[0], atol=1e-13)
    # and back across x = lo
    P.v[0] = [-0.2, 0.0, 0.0]
    orc.push(m, P, np.zeros((1, 3)), [-1.0], 1.0)
    P.vref[0] = np.linalg.solve((m.nodes[m.tets[P.cell[0]]][1:] - m.nodes[m.tets[P.cell[0]]][0]).T, P.v[0])
    r = orc.walk(m, P, 1.0, kill=1)
    assert r["killed"] == 0
    assert np.allclose(P.x[0], [0.87, 0.41, 0.57], atol=1e-13)


def test_periodic_assembly_and_solves_agree(orc):
    # mode 1 (symmetric, ghost plane left out) is symmetric with zero row sums
    # away from the walls; mode 0 BiCGStab (reference ghost rows) and mode 1
    # CG give the same phi
    import scipy.sparse as sp
    n = 6
    m = orc.Mesh(n, split=6, mapping=4, jitter=0.2, seed=5, periodic=1)
    plane = (n + 1) ** 2
    rp, col, val = m.assemble(1)
    R = len(rp) - 1
    assert R == m.N - plane
    A = sp.csr_matrix((val, col, rp), shape=(R, R))
    assert abs(A - A.T).max() < 1e-15
    # rows two or more cells away from the y and z walls (all x planes,
    # including the two coupled through the periodic faces)
    r = np.arange(R)
    j, k = (r // (n + 1)) % (n + 1), r % (n + 1)
    inner = (j >= 2) & (j <= n - 2) & (k >= 2) & (k <= n - 2)
    rs = np.asarray(A.sum(axis=1)).ravel()
    assert np.abs(rs[inner]).max() < 1e-12 * np.abs(val).max()
    rng = np.random.default_rng(3)
    b = rng.standard_normal(m.N)
    b[m.boundary == 1] = 0
    b[m.node_pairs >= 0] = 0          # ghost rows carry no charge (PIC.cpp:132-134)
    x1, it1, _ = orc.cg(m, b, tol=1e-12, max_iter=2000)
    m.assemble(0)
    x0, it0, _ = orc.bicgstab(m, b, tol=1e-12, max_iter=2000)
    assert np.abs(x0 - x1).max() <= 1e-8 * np.abs(x1).max()
    g = m.node_pairs >= 0
    assert (x1[g] == x1[m.node_pairs[g]]).all() and (x0[g] == x0[m.node_pairs[g]]).all()
