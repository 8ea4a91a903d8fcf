"""Configuration and checkpoint files (InputOutput.f90) through the engine library's host entry
points, against the oracle's restatement of the formats (oracle/state_io_oracle.py). Host only:
no GPU. Text output must be byte-identical; numbers read back must be identical (bit for bit)."""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FRAMES = os.path.join(HERE, "golden", "reference_frames.npz")


@pytest.fixture(scope="module")
def sio(pkg):
    pkg.build_lib.build()
    return pkg.state_io


@pytest.fixture(scope="module")
def so():
    import __graft_entry__ as ge

    ge.load_oracle()
    import state_io_oracle

    return state_io_oracle


def molecules(rng, nw, L):
    O = rng.uniform(-L / 2, L / 2, size=(nw, 3))
    H1 = O + rng.normal(scale=0.6, size=(nw, 3))
    H2 = O + rng.normal(scale=0.6, size=(nw, 3))
    return np.stack([O, H1, H2], axis=1).reshape(-1, 3)


@pytest.mark.parametrize("layout", ["box_first", "count_first", "one_record"])
@pytest.mark.parametrize("read_method", [0, 1])
def test_read_xyz_layouts(sio, so, tmp_path, layout, read_method):
    rng = np.random.default_rng(11)
    nw, L = 7, 12.3456
    RR = molecules(rng, nw, L)
    sym = ["O", "H", "H"] * nw
    order = list(range(3 * nw)) if read_method == 1 else [3 * i for i in range(nw)] + [
        3 * i + k for i in range(nw) for k in (1, 2)]
    head = {"box_first": "%.6f %.6f %.6f\n%d\n" % (L, L, L, 3 * nw),
            "count_first": "  %d\n%.6f  %.6f  %.6f\n" % (3 * nw, L, L, L),
            "one_record": "%d %.6f %.6f %.6f\n\n" % (3 * nw, L, L, L)}[layout]
    body = "".join("%s %.9f %.9f\t%.9f\n" % (sym[i], *RR[i]) for i in order)
    path = str(tmp_path / "frame.xyz")
    open(path, "w").write(head + body)
    n, nb, t, box = sio.read_config_header(path)
    assert (n, nb, t) == (3 * nw, 0, 0.0) and np.allclose(box, L)
    b1, R1 = sio.read_xyz(path, read_method)
    b2, R2 = so.read_xyz(path, read_method)
    assert np.array_equal(b1, b2) and np.array_equal(R1, R2)
    if read_method == 1:
        assert np.abs(R1.mean(axis=0)).max() < 1e-12
    else:  # the read_method 0 loop accumulates no mean: coordinates as read
        assert np.allclose(R1, np.round(RR, 9), atol=1e-12)


def test_write_xyz_bytes(sio, so, tmp_path):
    rng = np.random.default_rng(3)
    RR = molecules(rng, 5, 10.0)
    RR[0, 0] = -0.0000004  # rounds to -0.000000, written with its sign as Fortran does
    RR[1, 1] = 1.0e9       # does not fit f12.6: asterisks
    path = str(tmp_path / "out.xyz")
    sio.write_xyz(path, RR)
    sio.write_xyz(path, RR[::-1].copy(), append=True)
    got = open(path).read()
    assert got == so.format_xyz(RR) + so.format_xyz(RR[::-1].copy())
    assert "************" in got and " -0.000000" in got


@pytest.mark.parametrize("with_nh", [False, True])
def test_image_round_trip(sio, so, tmp_path, with_nh):
    rng = np.random.default_rng(7)
    nw, P, L, mO, mH = 4, 3, 11.0, 15.9994, 1.008
    base = molecules(rng, nw, L)
    RRt = base[None] + rng.normal(scale=0.05, size=(P, 3 * nw, 3))
    RRt[:, 0, 0] += 0.9 * L  # a centroid outside the box: the loader shifts the ring back
    PPt = rng.normal(scale=3.0, size=(P, 3 * nw, 3))
    vb = rng.normal(size=(3, P, 3 * nw, 2)) * np.array([1e-7, 12.5]) if with_nh else None
    vg = np.array([0.1, -3.3e-5]) if with_nh else None
    path = str(tmp_path / "state.img")
    sio.save_image(path, 1.25, (L, L, L), RRt, PPt, mO, mH, vb, vg)
    assert open(path).read() == so.format_image(1.25, (L, L, L), RRt, PPt, mO, mH, vb, vg)
    got = sio.load_image(path, mO, mH, n_vxi_beads=with_nh, n_vxi_global=2 if with_nh else 0)
    ref = so.parse_image(path, mO, mH, vxi_beads=with_nh, n_vxi_global=2 if with_nh else 0)
    for k in ("RRt", "PPt", "RRc", "box"):
        assert np.array_equal(got[k], ref[k]), k
    assert got["time"] == ref["time"] == 1.25
    # the file keeps 6 decimals of positions and velocities; chain velocities all digits
    shift = got["RRt"] - RRt
    assert np.abs(shift - np.round(shift / L) * L).max() <= 5.1e-7
    assert np.abs(got["RRc"][0, 0]) < L / 2 + 0.2
    im = np.where(np.arange(3 * nw) % 3 == 0, 1 / mO, 1 / mH)[None, :, None]
    assert np.abs(got["PPt"] * im - PPt * im).max() <= 5.1e-7
    if with_nh:
        assert np.array_equal(got["vxi_beads"], vb) and np.array_equal(got["vxi_global"], vg)


def test_image_rejects_wrong_sizes(sio, pkg, tmp_path):
    RRt = np.zeros((2, 6, 3))
    path = str(tmp_path / "s.img")
    sio.save_image(path, 0.0, (9.0, 9.0, 9.0), RRt, RRt, 16.0, 1.0)
    L = pkg.engine.load()
    buf = np.zeros(3 * 6 * 3)
    p = buf.ctypes.data_as(pkg.engine._D)
    box = np.zeros(3)
    # three beads asked for, two in the file (the reference aborts, InputOutput.f90:90-94)
    assert L.pimd_load_image(path.encode(), 6, 3, 16.0, 1.0, None, box.ctypes.data_as(pkg.engine._D), p, p, None,
                             None, 0, None, 0) == 1
    assert L.pimd_read_config_header(str(tmp_path / "missing.xyz").encode(), pkg.engine._I(), None, None,
                                     box.ctypes.data_as(pkg.engine._D)) == 1


def test_reference_frames_fixture(sio, so):
    """The committed frames are the reference's files as both readers read them (checked where
    the reference tree is named by PIMD_REFERENCE_DIR; else the fixture's own consistency)."""
    d = np.load(FRAMES)
    names = sorted({k.rsplit("_", 1)[0] for k in d.files})
    assert names == ["4nm", "input_128", "input_32", "input_512"]
    for n in names:
        assert d[n + "_RRc"].shape[0] % 3 == 0 and d[n + "_box"].shape == (3,)
    ref = os.environ.get("PIMD_REFERENCE_DIR")
    if not ref:
        pytest.skip("PIMD_REFERENCE_DIR not set: fixture not re-read from the reference tree")
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_frames", os.path.join(HERE, "golden", "make_frames.py"))
    mf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mf)
    for n, relpath in mf.FRAMES.items():
        path = os.path.join(ref, relpath)
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == str(d[n + "_sha256"])
        box, RRc = sio.read_xyz(path)
        assert np.array_equal(box, d[n + "_box"]) and np.array_equal(RRc, d[n + "_RRc"])
        obox, oR = so.read_xyz(path)
        assert np.array_equal(oR, RRc)
