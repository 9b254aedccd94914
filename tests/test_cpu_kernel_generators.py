"""Collection-kernel table generators (collision/kernel.py:793-942) against the
reference's own output (tests/golden/kernel_generators.npz): the Beard
velocities, the kernel grid K(R1, R2), the mass and radius grids, bit for
bit."""
import numpy as np
import pytest

from conftest import golden, sub


@pytest.mark.parametrize("kt", ["Long_Bott", "Hall_Bott"])
@pytest.mark.parametrize("n10", [10, 20])
def test_kernel_grid_generators_vs_reference(kt, n10):
    from lacmopy_gb300 import tables
    d = sub(golden("kernel_generators.npz"), f"{kt}_{n10}")
    R_low, R_high, nb10, rho = d["args"]
    gen = {"Long_Bott": tables.generate_kernel_grid_Long_Bott_np,
           "Hall_Bott": tables.generate_kernel_grid_Hall_Bott_np}[kt]
    K, vel, mass, rg = gen(R_low, R_high, int(nb10), rho)
    np.testing.assert_array_equal(rg, d["radius"])
    np.testing.assert_array_equal(vel, d["vel"])
    np.testing.assert_array_equal(mass, d["mass"])
    np.testing.assert_array_equal(K, d["K"])


def test_generate_and_save_writes_the_reference_files(tmp_path):
    from lacmopy_gb300 import tables
    d = sub(golden("kernel_generators.npz"), "Long_Bott_10")
    R_low, R_high, nb10, rho = d["args"]
    tables.generate_and_save_kernel_grid(R_low, R_high, int(nb10), rho, "Long_Bott",
                                         str(tmp_path) + "/")
    for fn, key in (("kernel_grid.npy", "K"), ("velocity_grid.npy", "vel"),
                    ("mass_grid_out.npy", "mass"), ("radius_grid_out.npy", "radius")):
        np.testing.assert_array_equal(np.load(tmp_path / fn), d[key])
    nb, m_lo, bf = tables.kernel_grid_m_parameters(d["mass"])
    assert nb == d["mass"].size and np.isclose(np.exp(m_lo), d["mass"][0])
