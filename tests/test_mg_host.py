"""CPU checks of the multigrid hierarchy behind MPG_SOLVER_CG_MG (host set-up
only, no GPU): each coarse operator equals the Galerkin product P^T A P of the
oracle's assembled symmetric system with trilinear interpolation P (to FP32
rounding of the stored stencil), level 0's D^-1 and Dirichlet flags match the
system, odd cell counts coarsen with a one-cell last interval, and meshes
periodic in x coarsen plane by plane with wrap-around.

The preconditioner is not part of the reference (its CG is unpreconditioned);
the converged solution is checked against the oracle CG on the GPU
(test_gpu_mixed.py, test_gpu_periodic.py)."""
import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")

MESHES = [
    # (n, split, mapping, jitter, periodic, dense_max)
    (8, 6, 0, 0.0, 0, 100),
    ((8, 6, 10), 6, 4, 0.2, 0, 100),
    (8, 5, 0, 0.0, 0, 100),
    (9, 6, 0, 0.0, 0, 100),             # odd cell counts: the last coarse interval is one fine cell
    ((9, 7, 12), 6, 4, 0.2, 0, 60),
    (16, 6, 4, 0.2, 1, 0),
    (16, 6, 0, 0.0, 1, 0),
    ((16, 9, 11), 6, 4, 0.2, 1, 300),
]


def _extents(n, periodic):
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    return (nx if periodic else nx + 1, ny + 1, nz + 1)


def _interp(fine, coarse, periodic):
    """Trilinear P (fine rows x coarse columns) between interior nodes."""
    gx, gy, gz = fine
    cx, cy, cz = coarse

    def bnd(i, j, k, ex):
        return (not periodic and (i == 0 or i == ex[0] - 1)) or j in (0, ex[1] - 1) or k in (0, ex[2] - 1)

    rows, cols, vals = [], [], []
    for I in range(cx):
        for J in range(cy):
            for K in range(cz):
                if bnd(I, J, K, coarse):
                    continue
                C = (I * cy + J) * cz + K
                for di in (-1, 0, 1):
                    fi = 2 * I + di
                    if periodic:
                        fi %= gx
                    for dj in (-1, 0, 1):
                        for dk in (-1, 0, 1):
                            fj, fk = 2 * J + dj, 2 * K + dk
                            if bnd(fi, fj, fk, fine):
                                continue
                            rows.append((fi * gy + fj) * gz + fk)
                            cols.append(C)
                            vals.append((0.5 if di else 1.0) * (0.5 if dj else 1.0) * (0.5 if dk else 1.0))
    n_f, n_c = gx * gy * gz, cx * cy * cz
    return scipy_sparse.csr_matrix((vals, (rows, cols)), shape=(n_f, n_c))


def _stencil_matrix(val, ext, bnd, periodic):
    cx, cy, cz = ext
    n = cx * cy * cz
    rows, cols, vals = [], [], []
    for C in range(n):
        if bnd[C]:
            continue
        I, J, K = C // (cy * cz), (C // cz) % cy, C % cz
        for d in range(27):
            di, dj, dk = d // 9 - 1, (d // 3) % 3 - 1, d % 3 - 1
            i2 = (I + di) % cx if periodic else I + di
            C2 = (i2 * cy + J + dj) * cz + K + dk
            if bnd[C2] or val[d, C] == 0.0:
                continue
            rows.append(C)
            cols.append(C2)
            vals.append(float(val[d, C]))
    return scipy_sparse.csr_matrix((vals, (rows, cols)), shape=(n, n))


@pytest.mark.parametrize("n,split,mapping,jit,periodic,dense_max", MESHES)
def test_coarse_operators_are_galerkin_products(mpg, orc, n, split, mapping, jit, periodic, dense_max):
    m = orc.Mesh(n, split=split, mapping=mapping, jitter=jit, seed=5, periodic=periodic)
    rp, col, val = m.assemble(1)
    R = len(rp) - 1
    A = scipy_sparse.csr_matrix((val, col, rp), shape=(R, R))
    h0 = mpg.mg_hierarchy(n, split=split, mapping=mapping, jitter=jit, seed=5, periodic=periodic,
                          dense_max=dense_max, level=0)
    assert h0["extent"] == _extents(n, periodic)
    assert h0["nlev"] >= 2
    # level 0: Dirichlet rows and D^-1 of the system
    diag = A.diagonal()
    bnd0 = m.boundary[:R] == 1
    assert ((h0["bnd"] == 1) == bnd0).all()
    assert np.allclose(h0["dinv"][~bnd0], (1.0 / diag[~bnd0]).astype(np.float32), rtol=1e-7)
    Af, fine = A, h0["extent"]
    for lev in range(1, h0["nlev"]):
        h = mpg.mg_hierarchy(n, split=split, mapping=mapping, jitter=jit, seed=5, periodic=periodic,
                             dense_max=dense_max, level=lev)
        ext = h["extent"]
        if periodic:
            assert ext == (fine[0] // 2, fine[1] // 2 + 1, fine[2] // 2 + 1)
        else:
            assert ext == tuple(g // 2 + 1 for g in fine)
        P = _interp(fine, ext, periodic)
        Ac = (P.T @ Af @ P).tocsr()
        Ms = _stencil_matrix(h["val"], ext, h["bnd"], periodic)
        scale = np.abs(Ac).max()
        assert np.abs((Ac - Ms).toarray()).max() <= 1e-6 * scale
        # symmetric, positive diagonal, D^-1 of the stored stencil
        assert np.abs((Ms - Ms.T).toarray()).max() <= 1e-6 * scale
        inner = h["bnd"] == 0
        assert (h["val"][13][inner] > 0).all()
        assert np.allclose(h["dinv"][inner], 1.0 / h["val"][13][inner].astype(np.float64), rtol=1e-6)
        Af, fine = Ac, ext


def test_too_small_grid_is_not_coarsened(mpg):
    # 3 cells per side: 4 nodes, fewer than the 5 a halving needs
    with pytest.raises(mpg.MpgError):
        mpg.mg_hierarchy(3, dense_max=1, level=0)


@pytest.mark.parametrize("n,periodic", [(32, 0), (31, 0), (24, 1), (16, 0)])
def test_bench_level_model_matches_library(mpg, n, periodic):
    # bench.py's algorithmic-bytes model of the multigrid iteration uses the
    # same level extents the library builds
    import bench
    model = bench.mg_levels(n, periodic)
    h = mpg.mg_hierarchy(n, periodic=periodic, level=len(model) - 1)
    assert len(model) == h["nlev"]
    x, g, _ = model[-1]
    assert h["extent"] == (x, g, g)
