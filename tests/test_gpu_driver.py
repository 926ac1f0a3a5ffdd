"""The C++ host driver (openrbc_gb300/driver/openrbc_gpu.cpp) with the
reference's command line: -i trimesh -m PREFIX builds the cell from mesh
files through init_rbc's network and the GPU lipid placement, minimises and
runs; -i vesicle runs the synthetic red cell."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, geodesic_mesh

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(ROOT, "openrbc_gb300", "openrbc_gpu")


def _run(args):
    r = subprocess.run([DRIVER] + args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    return r.returncode, r.stdout


def test_driver_runs_a_cell_from_mesh_files(tmp_path):
    v, e, f = geodesic_mesh(2)
    prefix = str(tmp_path / "ico42")
    np.savetxt(prefix + ".vert.txt", v, fmt="%.9f", delimiter="\t")
    np.savetxt(prefix + ".bond.txt", e, fmt="%d", delimiter="\t")
    np.savetxt(prefix + ".face.txt", f, fmt="%d", delimiter="\t")
    rc, out = _run(["-i", "trimesh", "-m", prefix, "-t", "0.2", "-k", "0.01", "-D", "10", "-E", "100"])
    assert rc == 0, out
    assert "particle-steps/s" in out
    temps = [float(line.split("T =")[1].split()[0]) for line in out.splitlines() if line.startswith("t =")]
    assert len(temps) == 2 and all(np.isfinite(temps))


def test_driver_refuses_missing_mesh_files(tmp_path):
    rc, out = _run(["-i", "trimesh", "-m", str(tmp_path / "nothing"), "-t", "0.1"])
    assert rc != 0 and "mesh" in out


def test_driver_runs_the_synthetic_cell():
    rc, out = _run(["-i", "vesicle", "--n-lipid", "100000", "--mesh-frequency", "8", "-t", "0.1", "-D", "5"])
    assert rc == 0, out
    assert "particle-steps/s" in out
