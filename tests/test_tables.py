"""Rate tables saved by the reference (scattering_struct::save, src/monte_carlo/scattering_struct.h:
56-94) are read back as they were written: the four grids one value per line, the rates after a
four-line header, theta-major.  Armadillo prints vectors in scientific notation with leading
blanks; values written at full precision come back bit for bit."""
import os

import numpy as np

from cnt_film_monte_carlo_gb300 import tables
from oracle import oracle as O

GRID = ([0, 180, 21], [1.5e-9, 10e-9, 11], [-10e-9, 10e-9, 11], [-10e-9, 10e-9, 11])


def save_like_reference(tab, directory, fmt="%.17g", grid_fmt="   %.17e"):
    """Write tab in the layout of scattering_struct::save."""
    base = os.path.join(directory, "scat_table")
    for name, g in zip(("theta", "z_shift", "axis_shift_1", "axis_shift_2"), tab["grids"]):
        with open(base + f".{name}.dat", "w") as f:
            f.write("".join(grid_fmt % x + "\n" for x in g))
    r = tab["rate"]
    with open(base + ".rates.dat", "w") as f:
        f.write("sizes:\ntheta, z_shift, axis_shift_1, axis_shift_2\n")
        f.write(",".join(str(n) for n in r.shape) + "\n\n")
        f.write("".join(fmt % x + "\n" for x in r.ravel()))


def test_saved_table_reads_back_exactly(tmp_path):
    tab = O.forster_table(1e15, *GRID)
    save_like_reference(tab, str(tmp_path))
    t = tables.read_reference_table(str(tmp_path))
    assert t["kind"] == 4 and t["rate"].shape == (21, 11, 11, 11)
    for a, b in zip(t["grids"], tab["grids"]):
        assert np.array_equal(a, b)
    assert np.array_equal(t["rate"], tab["rate"])


def test_saved_table_at_stream_precision(tmp_path):
    # the reference writes the rates with the stream's default precision (6 significant digits)
    tab = O.forster_table(1e13, *GRID)
    save_like_reference(tab, str(tmp_path), fmt="%g", grid_fmt="   %.4e")
    t = tables.read_reference_table(str(tmp_path))
    np.testing.assert_allclose(t["rate"], tab["rate"], rtol=5e-6)
    np.testing.assert_allclose(t["grids"][0], tab["grids"][0], rtol=1e-4)


def test_forster_2d_table_is_the_formula():
    # gamma_0 cos^2(theta) (1 nm / d)^6 on the 2-D grids, built by the library for both drivers
    t = tables.forster_2d(1e15, (0.5e-9, 10e-9, 96), (0.0, 90.0, 91))
    d, th = t["grids"]
    assert t["kind"] == 2 and t["rate"].shape == (96, 91)
    assert np.array_equal(d, tables.linspace(0.5e-9, 10e-9, 96))
    assert np.array_equal(th, tables.linspace(0.0, 90.0, 91) * (tables.REF_PI / 180))
    want = 1e15 * np.cos(th)[None, :] ** 2 * (1e-9 / d[:, None]) ** 6
    np.testing.assert_allclose(t["rate"], want, rtol=1e-14, atol=1e-300)
    assert t["rate"][0, 0] == 1e15 * (1e-9 / 0.5e-9) ** 6


def test_oracle_2d_table_equals_library_table():
    # the oracle builds the benchmark films' table on its own (the CPU reference arm of bench.py
    # never loads the library); it must be the library's table bit for bit
    for args in (((0.5e-9, 10e-9, 96), (0.0, 90.0, 91)), ((0.3e-9, 12e-9, 17), (0.0, 90.0, 7))):
        t = tables.forster_2d(1e15, *args)
        o = O.forster2d_table(1e15, *args)
        assert o["kind"] == t["kind"] == 2
        for a, b in zip(o["grids"], t["grids"]):
            assert np.array_equal(a, b)
        assert np.array_equal(o["rate"], t["rate"])
