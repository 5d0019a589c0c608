"""The five workloads as stated for the benchmark and the parity tests (no GPU),
checked against their descriptions: grids and domains in the reference's axis order
(ni, nj_wall, nk) with the walls at j = 1 and j = nj; fluid properties, time steps
and run lengths; the sessile drop's lower wall a 60/120 deg checkerboard of 0.125 x
0.125 squares starting at the domain's origin, its upper wall uniform; the
128x64x64 rollout's per-wall-cell angles 75 + N(0, 5^2) deg; the drop a spherical
cap of radius 0.3 centred 0.15 above the lower wall."""
import numpy as np
import pytest

from fmf import config as C


def test_grids_domains_and_properties():
    want = {
        # name: (ni, nj, nk, dt, steps, rhol/rhog, rmul/rmug)
        "couette32": (32, 32, 16, 1e-4, 100, 1.0, 1.0),
        "couette256": (256, 128, 128, 2e-5, 1000, 10.0, 10.0),
        "droplet512": (512, 256, 256, 1e-5, 500, 1000.0, 100.0),
        "couette128": (128, 64, 64, 1e-4, 200, 1.0, 1.0),
        "droplet256": (256, 128, 128, 1e-5, 500, 1000.0, 100.0),
    }
    for name, (ni, nj, nk, dt, steps, rr, mr) in want.items():
        c = C.get(name)
        assert (c.ni, c.nj, c.nk) == (ni, nj, nk), name
        assert (c.xl, c.yl, c.zl) == (2.0, 1.0, 1.0), name
        assert c.dt == dt and c.steps == steps, name
        assert c.rhol / c.rhog == pytest.approx(rr) and c.rmul / c.rmug == pytest.approx(mr), name
        assert c.cells == ni * nj * nk
    for name in ("droplet512", "droplet256"):
        assert C.get(name).uwall == 0.0


@pytest.mark.parametrize("name", ["droplet512", "droplet256"])
def test_checkerboard_lower_wall(name):
    c = C.get(name)
    th = C.wall_arrays(c)[0]
    n = c.checker_cells
    assert n * c.dx == pytest.approx(0.125) and n * c.dz == pytest.approx(0.125)
    low = th[3:c.nk + 3, 3, 3:c.ni + 3]  # k, i interior of the j = 1 plane
    assert set(np.unique(low)) == {60.0, 120.0}
    # constant on each 0.125 x 0.125 square (squares start at x = 0 and z = 0)
    blocks = low.reshape(c.nk // n, n, c.ni // n, n)
    assert np.all(blocks == blocks[:, :1, :, :1])
    corner = blocks[:, 0, :, 0]
    # neighbouring squares differ, along x and along z
    assert np.all(corner[:, 1:] != corner[:, :-1]) and np.all(corner[1:, :] != corner[:-1, :])
    # the upper wall is uniform
    assert np.all(th[3:c.nk + 3, c.nj + 2, 3:c.ni + 3] == c.theta_hi)


def test_rollout_wall_angles():
    c = C.get("couette128")
    th = C.wall_arrays(c)[0]
    vals = np.concatenate([th[:, 3, :].ravel(), th[:, c.nj + 2, :].ravel()])
    assert vals.size == 2 * (c.nk + 6) * (c.ni + 6)
    assert abs(vals.mean() - 75.0) < 0.2 and abs(vals.std() - 5.0) < 0.2
    assert np.array_equal(th, C.wall_arrays(c)[0])  # seeded


def test_droplet_cap():
    c = C.get("droplet256").scaled(64, 32, 32, checker_cells=4)
    phi = C.phi_interior(c)  # phi = 0 inside the drop
    x = (np.arange(1, c.ni + 1) - 0.5) * c.dx
    y = (np.arange(1, c.nj + 1) - 0.5) * c.dy
    z = (np.arange(1, c.nk + 1) - 0.5) * c.dz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt((X - 1.0) ** 2 + (Y - 0.15) ** 2 + (Z - 0.5) ** 2)
    # a tanh profile of width 1.5 cells: 0.5 (1 - tanh(4 / 1.5)) = 0.005 four cells from the surface
    assert np.all(phi[r < 0.3 - 4 * c.dx] < 1e-2) and np.all(phi[r > 0.3 + 4 * c.dx] > 1 - 1e-2)
    # the cap's volume: the sphere of radius 0.3 above the wall at y = 0, on the
    # workload's own 256x128x128 grid (the smeared surface adds a second-order
    # excess: 4.5 % at 64x32x32, 1.1 % at 128x64x64, 0.28 % here)
    c = C.get("droplet256")
    vol = (1.0 - C.phi_interior(c)).sum() * c.dx * c.dy * c.dz
    h = 0.3 + 0.15  # the cap's height above the wall
    cap = np.pi * h * h * (3 * 0.3 - h) / 3.0
    assert vol == pytest.approx(cap, rel=0.01)
