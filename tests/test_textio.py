"""The reference driver's text formats (host only, runs without a GPU):
file names, boundary-data pairs with their size line, density pairs, the
distance grid and the result log, as the reference writes and reads them
(large3Dexample2.c:405-424, 1236-1252, 1333-1335, 3097-3129, 3446-3474,
1885-1896)."""
import os

import numpy as np
import pytest


def test_file_names(hz):
    names = hz.reference_file_names(64, 5.0)
    assert names == {"b": "Rel_bN64k5.txt", "bimg": "Rel_bimgN64k5.txt", "density": "Rel_DensityN64k5.txt",
                     "densityimg": "Rel_DensityimgN64k5.txt", "result": "Rel_Result_N64k5.txt",
                     "distance": "distance64.txt"}


def test_rhs_files_reference_format(hz, tmp_path):
    rng = np.random.default_rng(0)
    b = rng.standard_normal(37) + 1j * rng.standard_normal(37)
    pr, pi = str(tmp_path / "b.txt"), str(tmp_path / "bimg.txt")
    hz.write_rhs_files(pr, pi, b)
    # byte-for-byte the reference's print_f output: "%d\n" then "%.15lf\n"
    expect = "%d\n" % len(b) + "".join("%.15f\n" % v for v in b.real)
    assert open(pr).read() == expect
    back = hz.read_rhs_files(pr, pi, len(b))
    assert np.max(np.abs(back - b)) < 1e-15 * 10
    with pytest.raises(hz.HzError):
        hz.read_rhs_files(pr, pi, len(b) + 1)  # the reference's size check


def test_density_files(hz, tmp_path):
    x = np.array([1.25, -3.5e-3, 7.0]) + 1j * np.array([0.5, 2.0, -1.0])
    pr, pi = str(tmp_path / "d.txt"), str(tmp_path / "dimg.txt")
    hz.write_density_files(pr, pi, x)
    assert open(pr).read() == "".join("%.15f " % v for v in x.real)
    assert np.array_equal(hz.read_density_files(pr, pi, 3), x)
    open(pr, "w").write("1.0 nan 2.0")
    with pytest.raises(hz.HzError):
        hz.read_density_files(pr, pi, 3)


def test_distance_file_round_trip(hz, tmp_path):
    from helmholtz_3d_torrone_gb300 import geometry as G
    d = G.sphere(12, radius=0.5)
    p = str(tmp_path / "distance12.txt")
    hz.write_distance_file(p, 12, d)
    assert np.array_equal(hz.read_distance_file(p, 12), d)
    # a whitespace-separated file as the reference reads it with fscanf("%lf")
    open(p, "w").write(" ".join("%.12f" % v for v in d.ravel()))
    assert np.max(np.abs(hz.read_distance_file(p, 12) - d)) < 1e-12
    open(p, "w").write("0.5 0.25")
    with pytest.raises(hz.HzError):
        hz.read_distance_file(p, 12)


def test_result_file(hz, tmp_path):
    p = str(tmp_path / "res.txt")
    hz.write_result_file(p, 1.0 + 2.0j, 1.1 + 1.9j)
    lines = open(p).read().splitlines()
    assert lines[0] == "Real: exact = 1.000000, trad_approxu = 1.100000, error %.2E" % (0.1 / 1.0)
    assert lines[2].startswith("Norm: exact = %f" % abs(1.0 + 2.0j))
