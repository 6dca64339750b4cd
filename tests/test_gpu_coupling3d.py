"""The 3-D coupling pieces on the GPU (rhoPJ CalcJfx, QWPlacement; usefulsubs
EAtXYZ) against the reference's vectors and the oracle (needs a GPU)."""

import numpy as np
import pytest
import torch

from oracle import sbe_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def _bits(z):
    return np.ascontiguousarray(z).view(np.int64)


def test_vs_reference_vectors():
    from pulsesuite_gb300 import rhoPJ, usefulsubs
    g = golden("coupling3d")
    J = rhoPJ.CalcJfx(g["rn"], g["rp"], float(g["dt"]), float(g["dx"]))
    assert np.max(np.abs(J - g["J"])) <= 1e-13 * np.max(np.abs(g["J"]))
    grid = np.zeros(g["grid"].shape, dtype=complex)
    rhoPJ.QWPlacement(g["fw"], g["gx"], g["gy"], g["gz"], grid)
    assert np.array_equal(_bits(grid), _bits(g["grid"]))            # bit-exact
    val = usefulsubs.EAtXYZ_points(g["f"], g["x"], g["y"], g["z"], g["pts"])
    assert np.array_equal(_bits(val), _bits(g["val"]))              # bit-exact
    assert usefulsubs.EAtXYZ(g["f"], g["x"], g["y"], g["z"], *g["pts"][7]) == g["val"][7]


def test_large_sizes_vs_oracle():
    """CalcJfx over 100k points (scan against the serial recurrence), QWPlacement on a
    256 x 64 x 64 grid and EAtXYZ at 20k points, device tensors in and out."""
    from pulsesuite_gb300 import rhoPJ, usefulsubs
    rng = np.random.default_rng(5)
    n = 100003
    rn = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    rp = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    J = rhoPJ.CalcJfx(torch.as_tensor(rn).cuda(), torch.as_tensor(rp).cuda(), 1e-16, 5e-9)
    ref = O.calc_jfx(rn, rp, 1e-16, 5e-9)
    assert float(np.max(np.abs(J.cpu().numpy() - ref))) <= 1e-12 * np.max(np.abs(ref))
    nx, ny, nz = 256, 64, 64
    fw = rng.standard_normal(nx) + 1j * rng.standard_normal(nx)
    gx, gy, gz = rng.uniform(0, 1, nx), rng.uniform(-1, 1, ny), rng.uniform(0, 1, nz)
    grid = torch.empty((nx, ny, nz), dtype=torch.complex128, device="cuda")
    rhoPJ.QWPlacement(torch.as_tensor(fw).cuda(), gx, gy, gz, grid)
    assert np.array_equal(_bits(grid.cpu().numpy()), _bits(O.qw_placement(fw, gx, gy, gz)))
    x = np.sort(rng.uniform(0, 1, 40))
    y = np.linspace(0, 1, 30)
    z = np.array([0.25])                     # a singleton axis
    f = rng.standard_normal((40, 30, 1)) + 1j * rng.standard_normal((40, 30, 1))
    pts = rng.uniform(-0.1, 1.1, (20000, 3))
    val = usefulsubs.EAtXYZ_points(f, x, y, z, pts)
    want = np.array([O.e_at_xyz(f, x, y, z, *p) for p in pts])
    assert np.array_equal(_bits(val), _bits(want))
