"""The reference's input files through the library's host readers (no GPU):
PETSc binary vectors (restart fields), xyz.dat / grid.dat grids and UCD
surfaces, checked against files written here with numpy in the formats the
reference reads (Source/main.c:376-935, Source/init.c:254-366,
Source/ibm_io.c:782-1011)."""
import os

import numpy as np
import pytest



def _reference_cases():
    """Instructional_Cases of the reference tree: VFS_REFERENCE_DIR, else the
    tree the reference pin was built from (oracle/_ref), else none."""
    import reference
    root = os.environ.get("VFS_REFERENCE_DIR") or reference.reference_dir()
    return os.path.join(root, "Instructional_Cases") if root else ""


REF_CASES = _reference_cases()


@pytest.fixture(scope="module")
def V(cuda_lib):
    import vfs_poisson
    return vfs_poisson


def test_petsc_vec_round_trip(V, tmp_path):
    rng = np.random.default_rng(0)
    v = rng.standard_normal(1000)
    p = str(tmp_path / "vfield000010_0.dat")
    V.write_petsc_vec(p, v)
    raw = open(p, "rb").read()
    assert raw[:4] == (1211214).to_bytes(4, "big") and raw[4:8] == (1000).to_bytes(4, "big")
    assert np.frombuffer(raw[8:], ">f8").tolist() == v.tolist()
    np.testing.assert_array_equal(V.read_petsc_vec(p), v)


def test_petsc_vec_written_elsewhere(V, tmp_path):
    # a Cmpnts DA field as VecView writes it on one rank: interleaved x,y,z
    u = np.arange(4 * 3 * 5 * 3, dtype=np.float64).reshape(4, 3, 5, 3) * 0.5 - 7
    p = tmp_path / "f.dat"
    with open(p, "wb") as f:
        f.write(np.array([1211214, u.size], ">i4").tobytes())
        f.write(u.astype(">f8").tobytes())
    np.testing.assert_array_equal(V.read_petsc_vec(str(p)).reshape(u.shape), u)
    bad = tmp_path / "bad.dat"
    bad.write_bytes(np.array([1211215, 1], ">i4").tobytes() + np.zeros(1, ">f8").tobytes())
    with pytest.raises(V.VfsError):
        V.read_petsc_vec(str(bad))


def test_xyz_grid(V, tmp_path):
    X, Y, Z = np.linspace(0, 2, 5), np.linspace(-1, 1, 4) ** 3, np.linspace(0, 1, 3)
    p = tmp_path / "xyz.dat"
    with open(p, "w") as f:
        f.write(f"{len(X)} {len(Y)} {len(Z)}\n")
        for x in X:
            f.write(f"{x:.17e} 0 0\n")
        for y in Y:
            f.write(f"0 {y:.17e} 0\n")
        for z in Z:
            f.write(f"0 0 {z:.17e}\n")
    coor = V.read_grid(str(p), V.GRID_XYZ, L_dim=2.0, cl=4.0)
    assert coor.shape == (len(Z) + 1, len(Y) + 1, len(X) + 1, 3)
    np.testing.assert_array_equal(coor[:-1, :-1, :-1, 0], np.broadcast_to(X / 4.0 * 2.0, (3, 4, 5)))
    np.testing.assert_array_equal(coor[:-1, :-1, :-1, 1], np.broadcast_to((Y / 4.0 * 2.0)[None, :, None], (3, 4, 5)))
    np.testing.assert_array_equal(coor[:-1, :-1, :-1, 2], np.broadcast_to((Z / 4.0 * 2.0)[:, None, None], (3, 4, 5)))
    assert np.all(coor[-1] == 0) and np.all(coor[:, -1] == 0) and np.all(coor[:, :, -1] == 0)


@pytest.mark.parametrize("binary", [False, True])
def test_grid_dat_blocks(V, tmp_path, binary):
    rng = np.random.default_rng(1)
    blocks = [rng.standard_normal((3, 4, 3, 5)), rng.standard_normal((3, 3, 2, 4))]  # [xyz][k][j][i]
    p = tmp_path / "grid.dat"
    if binary:
        with open(p, "wb") as f:
            f.write(np.array([2], np.int32).tobytes())
            for bk in blocks:
                _, KM, JM, IM = bk.shape
                f.write(np.array([IM, JM, KM], np.int32).tobytes())
                f.write(np.ascontiguousarray(bk).tobytes())
    else:
        with open(p, "w") as f:
            f.write("2\n")
            for bk in blocks:
                _, KM, JM, IM = bk.shape
                f.write(f"{IM} {JM} {KM}\n")
                for v in bk.ravel():
                    f.write(f"{v:.17e}\n")
    for bi, bk in enumerate(blocks):
        coor = V.read_grid(str(p), V.GRID_BINARY if binary else V.GRID_TEXT, block=bi)
        _, KM, JM, IM = bk.shape
        assert coor.shape == (KM + 1, JM + 1, IM + 1, 3)
        np.testing.assert_array_equal(coor[:KM, :JM, :IM].transpose(3, 0, 1, 2), bk)


def _write_ucd(path, xyz, tri):
    with open(path, "w") as f:
        f.write("# UCD\n#\n#\n")
        f.write(f"{len(xyz)} {len(tri)} 0 0 0\n")
        for q, (x, y, z) in enumerate(xyz):
            f.write(f"{q + 1} {x:.17e} {y:.17e} {z:.17e}\n")
        for e, (a, b, c) in enumerate(tri):
            f.write(f"{e + 1} 0 tri {a + 1} {b + 1} {c + 1}\n")


def test_ucd_surface(V, tmp_path):
    from vfs_poisson import configs as CF
    xyz, tri = CF.rod_surface((0.1, 0.2, 0.3), (0, 1, 0), 0.5, 0.05, 12, 3)
    p = tmp_path / "ibmdata00"
    _write_ucd(p, xyz, tri)
    x2, t2 = V.read_ucd(str(p))
    np.testing.assert_array_equal(x2, xyz)
    np.testing.assert_array_equal(t2, tri)
    # placement: scale, offset, then rotations about x, y, z in turn
    L, cm, r, ang = 2.0, (1.0, -1.0, 0.5), (0.3, 0.2, 0.1), (0.2, -0.4, 0.7)
    x3, _ = V.read_ucd(str(p), L_dim=L, cm=cm, centre=r, angles=ang)
    x = xyz * L + np.asarray(cm)
    X, Y, Z = x[:, 0].copy(), x[:, 1].copy(), x[:, 2].copy()
    Y, Z = r[1] + (Y - r[1]) * np.cos(ang[0]) - (Z - r[2]) * np.sin(ang[0]), \
        r[2] + (Y - r[1]) * np.sin(ang[0]) + (Z - r[2]) * np.cos(ang[0])
    X, Z = r[0] + (Z - r[2]) * np.sin(ang[1]) + (X - r[0]) * np.cos(ang[1]), \
        r[2] + (Z - r[2]) * np.cos(ang[1]) - (X - r[0]) * np.sin(ang[1])
    X, Y = r[0] + (X - r[0]) * np.cos(ang[2]) - (Y - r[1]) * np.sin(ang[2]), \
        r[1] + (X - r[0]) * np.sin(ang[2]) + (Y - r[1]) * np.cos(ang[2])
    np.testing.assert_allclose(x3, np.stack([X, Y, Z], 1), rtol=0, atol=1e-14)


@pytest.mark.skipif(not os.path.isdir(REF_CASES), reason="reference instructional cases not present")
def test_reference_instructional_files(V):
    """The reference's own input files (read in place; nothing is copied)."""
    ucd = os.path.join(REF_CASES, "Test_02_VIV_Mounted_Cyll", "ibmdata00")
    if os.path.exists(ucd):
        xyz, tri = V.read_ucd(ucd)
        assert xyz.shape == (484, 3) and tri.shape == (964, 3)
        assert tri.min() >= 0 and tri.max() < 484
    for case in sorted(os.listdir(REF_CASES)):
        p = os.path.join(REF_CASES, case, "xyz.dat")
        if os.path.exists(p):
            with open(p) as f:
                IM, JM, KM = (int(v) for v in f.readline().split()[:3])
            coor = V.read_grid(p, V.GRID_XYZ)
            assert coor.shape == (KM + 1, JM + 1, IM + 1, 3)
            assert np.all(np.diff(coor[0, 0, :IM, 0]) > 0)
            break
