"""The C++ driver (the reference's main.cpp shape) runs the reference problem
end to end through include/minipic_gb300.hpp and prints the reference's lines."""
import glob
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rows(path):
    with open(path) as f:
        return [ln.split() for ln in f if ln.strip()]


def _faces_edges(tets, nx, ny, nz, periodic):
    """Faces and edges in the reference's gid order (sorted node tuples,
    lexicographic; periodic x = nx faces renamed to x = 0, mesh.cpp:61-76)."""
    plane = (ny + 1) * (nz + 1)
    fidx = np.array([[0, 1, 3], [1, 2, 3], [0, 3, 2], [0, 2, 1]])
    f = tets[:, fidx].reshape(-1, 3).astype(np.int64)
    if periodic:
        on = (f // plane == nx).all(axis=1)
        f[on] -= nx * plane
    f = np.unique(np.sort(f, axis=1), axis=0)
    pairs = [(j, k) for j in range(3) for k in range(j + 1, 4)]
    e = np.stack([tets[:, [j, k]] for j, k in pairs], axis=1).reshape(-1, 2).astype(np.int64)
    e = np.unique(np.sort(e, axis=1), axis=0)
    return f, e


def test_driver_reference_problem(mpg, tmp_path):
    drv = os.path.join(os.path.dirname(mpg.lib_path()), "minipic_gb300")
    assert os.path.exists(drv)
    (tmp_path / "brick.txt").write_text("3 3 3 0\n")
    p = subprocess.run([drv, "--nparts=4", "--dt=0.1", "--tfinal=0.3", "--output=1", "--dump_mesh=1"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    out = p.stdout
    assert "Fill time" in out and "for 1080 particles" in out
    assert out.count("Total KE is") == 3
    assert "updates/second" in out and "Timers are:" in out
    assert any(f.name.startswith("output.") for f in tmp_path.iterdir())


def test_driver_dump_and_output_files_match_the_mesh_and_fill(mpg, orc, tmp_path):
    """--dump_mesh writes the eight files of Mesh::dump_data (mesh.cpp:794-910)
    and --output the particle samples of main.cpp:125-136; their contents are
    checked against the mesh arrays, an independent face/edge numbering, the
    reference's own boundary counts (mesh.cpp:641-646) and the oracle's
    reference fill."""
    drv = os.path.join(os.path.dirname(mpg.lib_path()), "minipic_gb300")
    n, nppe = 3, 4
    (tmp_path / "brick.txt").write_text(f"{n} {n} {n} 0\n")
    p = subprocess.run([drv, f"--nparts={nppe}", "--dt=0.1", "--steps=2", "--output=1", "--dump_mesh=1"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    ctx = mpg.Ctx(0)
    ctx.mesh(n, split=mpg.SPLIT_REF5, lo=-1.0, hi=1.0)
    mesh = ctx.mesh_arrays()
    nodes = _rows(tmp_path / "nodes-000.dat")
    assert [int(r[0]) for r in nodes] == list(range(ctx.N))
    assert np.allclose(np.array([[float(v) for v in r[1:]] for r in nodes]), mesh["nodes"], atol=1e-5)
    elems = np.array([[int(v) for v in r] for r in _rows(tmp_path / "elems-000.dat")])
    assert (elems[:, 0] == np.arange(ctx.T)).all() and (elems[:, 1:] == mesh["tets"]).all()
    f, e = _faces_edges(mesh["tets"], n, n, n, False)
    faces = np.array([[int(v) for v in r] for r in _rows(tmp_path / "faces-000.dat")])
    edges = np.array([[int(v) for v in r] for r in _rows(tmp_path / "edges-000.dat")])
    assert (faces[:, 0] == np.arange(len(f))).all() and (faces[:, 1:] == f).all()
    assert (edges[:, 0] == np.arange(len(e))).all() and (edges[:, 1:] == e).all()
    om = orc.Mesh(n, split=5, lo=-1.0, hi=1.0)
    assert len(f) == om.n_faces
    assert [int(r[0]) for r in _rows(tmp_path / "owned-faces-000.dat")] == list(range(len(f)))
    assert [int(r[0]) for r in _rows(tmp_path / "owned-edges-000.dat")] == list(range(len(e)))
    bf = [int(r[0]) for r in _rows(tmp_path / "boundary-faces-000.dat")]
    be = [int(r[0]) for r in _rows(tmp_path / "boundary-edges-000.dat")]
    nx = ny = nz = n
    assert len(bf) == 2 * (2 * nx * ny + 2 * nx * nz + 2 * ny * nz) == om.n_bfaces
    assert len(be) == (2 * (5 * nx * ny - nx * (ny - 1) - ny * (nx - 1) + 5 * nx * nz - nx * (nz - 1) - nz * (nx - 1)
                            + 5 * ny * nz - ny * (nz - 1) - nz * (ny - 1)) - 4 * (nx + ny + nz))
    xyz = mesh["nodes"]
    for g in bf:
        c = xyz[f[g]].mean(axis=0)
        assert (np.abs(c) >= 0.99999999).any()
    # output.<t> at t = 0: every nppe-th particle of type 0 of the reference fill
    outs = sorted(glob.glob(str(tmp_path / "output.*")))
    assert len(outs) == 2
    first = np.array([[float(v) for v in r] for r in _rows(tmp_path / "output.0.000000")])
    P = orc.Particles(2 * nppe * ctx.T)
    dens = 2.0 / 3.0 * np.pi ** 2
    P.fill_ref(om, nppe, 0, dens, mass=1.0)
    P.fill_ref(om, nppe, 1, dens, mass=1.0)
    pick = [i for i in range(0, P.n, nppe) if P.sp[i] == 0]
    assert first.shape == (len(pick), 6)
    # positions against the oracle (the fill is positionally bit-exact);
    # velocities against the same device fill (the Maxwellian acceptance test
    # uses exp(), whose last bit may differ between CUDA and glibc)
    assert np.allclose(first[:, :3], P.x[pick], rtol=1e-5, atol=1e-6)
    g = mpg.Ctx(0)
    g.mesh(n, split=mpg.SPLIT_REF5, lo=-1.0, hi=1.0)
    g.configure()
    g.reserve(2 * nppe * ctx.T)
    g.fill_ref(nppe, 0, dens)
    g.fill_ref(nppe, 1, dens)
    d = g.download()
    assert np.allclose(first[:, 3:], d["v"][pick], rtol=1e-5, atol=1e-6)


def test_driver_mixed_linear_cg(mpg, tmp_path):
    drv = os.path.join(os.path.dirname(mpg.lib_path()), "minipic_gb300")
    (tmp_path / "brick.txt").write_text("4 4 4 0\n")
    p = subprocess.run([drv, "--nparts=8", "--dt=0.05", "--steps=4", "--precision=mixed", "--solver=cg",
                        "--deposit=linear", "--tol=1e-10", "--kill-particles=1"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.count("Total KE is") == 4


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_driver_two_stream_periodic(mpg, tmp_path, precision):
    # main.cpp:89-106: --problem two-stream builds the periodic mesh and the
    # two counter-streaming beams; nothing leaves through x, so the only
    # losses are at the y/z walls
    drv = os.path.join(os.path.dirname(mpg.lib_path()), "minipic_gb300")
    (tmp_path / "brick.txt").write_text("4 4 4 0\n")
    args = [drv, "--nparts=8", "--dt=0.05", "--steps=4", "--problem=two-stream", "--kill-particles=1",
            "--precision=" + precision]
    if precision == "mixed":
        args += ["--solver=cg", "--deposit=linear", "--tol=1e-10"]
    p = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    out = p.stdout
    # 5 * 4^3 tets, 4 + 4 beam electrons and 8 ions per tet
    assert "for 5120 particles" in out
    assert out.count("Total KE is") == 4
