"""The C++ driver (the reference's main.cpp shape) runs the reference problem
end to end through include/minipic_gb300.hpp and prints the reference's lines."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


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
    assert (tmp_path / "nodes-000.dat").exists() and (tmp_path / "elems-000.dat").exists()
    assert any(f.name.startswith("output.") for f in tmp_path.iterdir())


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
