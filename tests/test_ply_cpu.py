"""The library's PLY importer (sky_ply_read_host, no GPU) against the
restatement of the reference's load() in oracle/ply.py: 3DGS files of SH
degree 0, 1 and 3 (with the f_rest ordering and rot_0 = w), xyz + rgb point
clouds (with the reference's double division of uchar colours by 255),
plain xyz clouds with the reference's defaults, and the files it rejects."""
import numpy as np
import pytest

from oracle import ply as O


def gauss_props(deg):
    rest = 3 * ((deg + 1) ** 2 - 1)
    props = [("float", a) for a in ("x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2")]
    props += [("float", f"f_rest_{k}") for k in range(rest)]
    props += [("float", a) for a in ("opacity", "scale_0", "scale_1", "scale_2",
                                     "rot_0", "rot_1", "rot_2", "rot_3")]
    return props


@pytest.mark.parametrize("deg", [0, 1, 3])
def test_gaussian_ply(sky, tmp_path, deg):
    rng = np.random.default_rng(deg)
    props = gauss_props(deg)
    rows = rng.normal(size=(300, len(props))).tolist()
    path = tmp_path / "g.ply"
    O.write_ply(path, props, rows)
    planes, d, ext = sky._lib.read_ply(path)
    want, wd, wext = O.expected_planes(props, rows)
    assert d == wd == deg
    assert np.array_equal(planes, want)
    assert ext == pytest.approx(wext, rel=0, abs=0)


def test_rgb_point_cloud_defaults(sky, tmp_path):
    props = [("float", "x"), ("float", "y"), ("float", "z"),
             ("uchar", "red"), ("uchar", "green"), ("uchar", "blue")]
    rows = [[0.1, 0.2, 0.3, 255, 128, 0], [-1.0, 2.0, 0.5, 10, 20, 30]]
    path = tmp_path / "pc.ply"
    O.write_ply(path, props, rows)
    planes, d, ext = sky._lib.read_ply(path)
    want, _, wext = O.expected_planes(props, rows)
    assert d == 0
    assert np.array_equal(planes, want)
    assert ext == pytest.approx(wext)
    # the reference divides uchar colours by 255 twice: red 255 -> 1/255
    assert planes[11, 0] == O.f16((1.0 / 255.0 - 0.5) / O.SH_C0)
    # default rotation halves (0, 0, 0, 1) read as quaternion (0, 0, 1, 0)
    assert planes[6:10, 0].tolist() == [0.0, 0.0, 1.0, 0.0]


def test_xyz_only(sky, tmp_path):
    props = [("float", "x"), ("float", "y"), ("float", "z")]
    rows = [[1.0, 2.0, 3.0]]
    path = tmp_path / "xyz.ply"
    O.write_ply(path, props, rows)
    planes, d, _ = sky._lib.read_ply(path)
    want, _, _ = O.expected_planes(props, rows)
    assert np.array_equal(planes, want)
    assert not planes[11:14].any()


def test_rejected_files(sky, tmp_path):
    p = tmp_path / "d.ply"
    O.write_ply(p, [("double", "x"), ("float", "y"), ("float", "z")], [[1.0, 2.0, 3.0]])
    with pytest.raises(sky.SkyError):
        sky._lib.read_ply(p)
    a = tmp_path / "a.ply"
    a.write_text("ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nend_header\n1.0\n")
    with pytest.raises(sky.SkyError):
        sky._lib.read_ply(a)
    t = tmp_path / "t.ply"
    O.write_ply(t, [("float", "x"), ("float", "y"), ("float", "z")], [[1.0, 2.0, 3.0]] * 4)
    t.write_bytes(t.read_bytes()[:-5])
    with pytest.raises(sky.SkyError):
        sky._lib.read_ply(t)
    with pytest.raises(sky.SkyError):
        sky._lib.read_ply(tmp_path / "missing.ply")
