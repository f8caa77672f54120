"""Mesh files (vtkSurface::CreateFromFile / WriteToFile, Common/vtkSurface.cxx:1958-2136):
round trips through every written format, hand-written files in the variants the
readers accept, and the error paths.  Host code only."""
import os

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import engine as E
from acvd_gb300 import synth

TET_P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.5]])
TET_F = np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], dtype=np.int32)


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


@pytest.mark.parametrize("ext", ["ply", "off", "obj", "vtk", "PLY"])
def test_round_trip(tmp_path, ext):
    m = synth.torus(20, 10, seed=1)
    p = str(tmp_path / f"m.{ext}")
    E.write_mesh(p, m.points, m.faces)
    pts, tri = E.read_mesh(p)
    np.testing.assert_array_equal(tri, m.faces)
    # PLY stores float points (as the reference's float vtkPoints); the text formats keep doubles
    np.testing.assert_array_equal(pts, _f32(m.points) if ext.lower() == "ply" else m.points)


def test_stl_merges_corners(tmp_path):
    m = synth.torus(20, 10, seed=1)
    p = str(tmp_path / "m.stl")
    E.write_mesh(p, m.points, m.faces)
    pts, tri = E.read_mesh(p)
    assert pts.shape == m.points.shape and tri.shape == m.faces.shape
    np.testing.assert_array_equal(pts[tri], _f32(m.points)[m.faces])
    # vertices numbered by first appearance in the facets
    first = []
    for v in m.faces.reshape(-1):
        if v not in first:
            first.append(v)
    np.testing.assert_array_equal(pts, _f32(m.points)[first])


def test_ascii_stl_and_surface_api(tmp_path):
    p = tmp_path / "t.stl"
    lines = ["solid t"]
    for f in TET_F:
        lines += ["facet normal 0 0 0", "outer loop"] + [f"vertex {x} {y} {z}" for x, y, z in TET_P[f]] + \
                 ["endloop", "endfacet"]
    p.write_text("\n".join(lines + ["endsolid t"]) + "\n")
    s = acvd_gb300.Surface.CreateFromFile(str(p))
    assert s.GetNumberOfPoints() == 4 and s.GetNumberOfCells() == 4 and s.GetNumberOfEdges() == 6
    np.testing.assert_array_equal(s.points[s.faces], TET_P[TET_F])


def test_ply_variants(tmp_path):
    # ascii, extra properties and elements, uint indices
    head = ("ply\nformat ascii 1.0\ncomment test\nelement vertex 4\nproperty double x\nproperty double y\n"
            "property double z\nproperty uchar red\nelement face 4\nproperty list uchar uint vertex_indices\n"
            "property float quality\nelement edge 1\nproperty int vertex1\nproperty int vertex2\nend_header\n")
    body = "".join(f"{x} {y} {z} 7\n" for x, y, z in TET_P) + "".join(f"3 {a} {b} {c} 0.5\n" for a, b, c in TET_F)
    p = tmp_path / "a.ply"
    p.write_text(head + body + "0 1\n")
    pts, tri = E.read_mesh(str(p))
    np.testing.assert_array_equal(pts, TET_P)
    np.testing.assert_array_equal(tri, TET_F)
    # binary big endian, int count, vertex_index name, normals before the coordinates
    head = ("ply\nformat binary_big_endian 1.0\nelement vertex 4\nproperty float nx\nproperty float x\n"
            "property float y\nproperty float z\nelement face 4\nproperty list int int vertex_index\nend_header\n")
    raw = bytearray(head.encode())
    for x, y, z in TET_P:
        raw += np.array([9, x, y, z], dtype=">f4").tobytes()
    for f in TET_F:
        raw += np.array([3, *f], dtype=">i4").tobytes()
    p = tmp_path / "b.ply"
    p.write_bytes(bytes(raw))
    pts, tri = E.read_mesh(str(p))
    np.testing.assert_array_equal(pts, _f32(TET_P))
    np.testing.assert_array_equal(tri, TET_F)


def test_obj_off_vtk_variants(tmp_path):
    obj = tmp_path / "a.obj"
    obj.write_text("# c\no x\n" + "".join(f"v {x} {y} {z}\n" for x, y, z in TET_P) + "vn 0 0 1\n" +
                   "f 1/1/1 2/2/1 3/3/1\nf 1//1 4//1 2//1\nf -4 -2 -1\nf 2 4 3\n")
    pts, tri = E.read_mesh(str(obj))
    np.testing.assert_array_equal(pts, TET_P)
    np.testing.assert_array_equal(tri, TET_F)
    off = tmp_path / "a.off"
    off.write_text("OFF 4 4 6\n# comment\n" + "".join(f"{x} {y} {z}\n" for x, y, z in TET_P) +
                   "".join(f"3 {a} {b} {c} 255 0 0\n" for a, b, c in TET_F))
    pts, tri = E.read_mesh(str(off))
    np.testing.assert_array_equal(pts, TET_P)
    np.testing.assert_array_equal(tri, TET_F)
    vtk = tmp_path / "a.vtk"
    vtk.write_text("# vtk DataFile Version 5.1\nt\nASCII\nDATASET POLYDATA\nPOINTS 4 float\n" +
                   " ".join(f"{x} {y} {z}" for x, y, z in TET_P) +
                   "\nPOLYGONS 5 12\nOFFSETS vtktypeint64\n0 3 6 9 12\nCONNECTIVITY vtktypeint64\n" +
                   " ".join(str(v) for v in TET_F.reshape(-1)) + "\nPOINT_DATA 4\n")
    pts, tri = E.read_mesh(str(vtk))
    np.testing.assert_array_equal(pts, TET_P)
    np.testing.assert_array_equal(tri, TET_F)


def test_errors(tmp_path):
    quad = tmp_path / "q.obj"
    quad.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    with pytest.raises(acvd_gb300.AcvdError) as ei:
        E.read_mesh(str(quad))
    assert ei.value.code == 5
    bad = tmp_path / "b.off"
    bad.write_text("OFF\n3 1 0\n0 0 0\n1 0 0\n0 1 0\n3 0 1 7\n")
    with pytest.raises(acvd_gb300.AcvdError):
        E.read_mesh(str(bad))
    for name in ("x.vtp", "x.wrl", "x.xyz"):   # an empty .vtp is no VTK XML file
        (tmp_path / name).write_text("")
        with pytest.raises(acvd_gb300.AcvdError):
            E.read_mesh(str(tmp_path / name))
    with pytest.raises(acvd_gb300.AcvdError):
        E.read_mesh(str(tmp_path / "missing.ply"))
    with pytest.raises(acvd_gb300.AcvdError):
        E.write_mesh(str(tmp_path / "o.ply"), TET_P, np.array([[0, 1, 9]]))


def test_cli_rejects_unbuilt_options():
    from acvd_gb300 import cli
    with pytest.raises(SystemExit):
        cli.main_acvd(["x.ply", "100", "0", "-w", "1"])
    with pytest.raises(SystemExit):
        cli.main_acvdq(["x.ply", "100", "0", "-d", "1"])
    with pytest.raises(SystemExit):
        cli.main_acvd(["x.ply"])


def test_acvdq_fixed_vertex_files(tmp_path):
    """-fv reads vertex ids until one does not parse; -ft marks the vertices of the listed
    faces; the last of the two given wins (ACVDQ.cxx:246-280)."""
    from acvd_gb300 import cli
    mesh = acvd_gb300.Surface(TET_P, np.array([[0, 1, 2], [0, 3, 1], [1, 3, 2], [2, 3, 0]], dtype=np.int32))
    (tmp_path / "v.txt").write_text("3 1\n2 x 0\n")
    (tmp_path / "f.txt").write_text("1\n")
    opts = cli._parse(["m.ply", "10", "0", "-fv", str(tmp_path / "v.txt")], "ACVDQ")
    np.testing.assert_array_equal(cli._fixed_vertices(opts, mesh), [3, 1, 2])
    opts = cli._parse(["m.ply", "10", "0", "-fv", str(tmp_path / "v.txt"), "-ft", str(tmp_path / "f.txt")], "ACVDQ")
    np.testing.assert_array_equal(cli._fixed_vertices(opts, mesh), [0, 1, 3])
    opts = cli._parse(["m.ply", "10", "0", "-fv", str(tmp_path / "missing.txt")], "ACVDQ")
    assert cli._fixed_vertices(opts, mesh).size == 0
    assert cli._fixed_vertices(cli._parse(["m.ply", "10", "0"], "ACVDQ"), mesh) is None


def test_native_programs_parse_like_the_reference():
    """The native ACVD / ACVDQ programs (csrc/acvd_cli.cpp) are built beside the library;
    without arguments they print the usage, an option that needs an unbuilt part stops
    them before any file or device is touched."""
    import subprocess
    from acvd_gb300 import build as B
    for name in ("acvd", "acvdq", "anisotropic_remeshing_q"):
        exe = os.path.join(B.OUT, name)
        assert os.access(exe, os.X_OK)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0 and "Usage" in r.stdout
        r = subprocess.run([exe, "missing.ply", "100", "0", "-w", "1"], capture_output=True, text=True)
        assert r.returncode == 1 and "-w" in r.stderr


def test_checkpoint_files_round_trip(tmp_path):
    """clustering.dat / curvature.dat as the reference's FileLoadSaveOption writes them:
    raw int32 and float64 per item."""
    r = acvd_gb300.QIsotropicDiscreteRemeshing()
    lab = np.arange(50, dtype=np.int32) % 7
    ind = np.linspace(0.1, 2.0, 50)
    r.Clustering = lab
    r.Indicator = ind
    r.SaveClustering(str(tmp_path / "clustering.dat"))
    r.SaveCurvature(str(tmp_path / "curvature.dat"))
    assert (tmp_path / "clustering.dat").stat().st_size == 4 * 50
    assert (tmp_path / "curvature.dat").stat().st_size == 8 * 50
    r2 = acvd_gb300.QIsotropicDiscreteRemeshing()
    np.testing.assert_array_equal(r2.LoadClustering(str(tmp_path / "clustering.dat")), lab)
    np.testing.assert_array_equal(r2.InitialClustering, lab)
    np.testing.assert_array_equal(r2.LoadCurvature(str(tmp_path / "curvature.dat")), ind)
    np.testing.assert_array_equal(r2.Indicator, ind)


def test_split_long_edges_follows_the_reference_order():
    """vtkSurface::SplitLongEdges worked by hand on one triangle (edges 4, sqrt(17), 1;
    threshold = their mean): edges 0 and 1 get midpoints 3 and 4 in edge order, and the
    face splits by the reference's Split3(f, v2, v3, v1, v23, v12) case, its first part in
    the face's slot."""
    pts = np.array([[0, 0, 0], [4, 0, 0], [0, 1, 0]], dtype=np.float64)
    p, t = E.split_long_edges(pts, np.array([[0, 1, 2]], dtype=np.int32), 1.0)
    np.testing.assert_array_equal(p, [[0, 0, 0], [4, 0, 0], [0, 1, 0], [2, 0, 0], [2, 0.5, 0]])
    np.testing.assert_array_equal(t, [[1, 4, 3], [4, 2, 0], [0, 3, 4]])


def _edges(tri):
    e = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
    u, cnt = np.unique(e, axis=0, return_counts=True)
    return u, cnt


def _area(p, t):
    return 0.5 * np.linalg.norm(np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]]), axis=1).sum()


@pytest.mark.parametrize("ratio", [0.6, 1.0, 1.5])
def test_split_long_edges_properties(ratio):
    m = synth.torus(20, 6, seed=3)              # long edges around the tube's length
    pts = m.points.astype(np.float32).astype(np.float64)
    e0, _ = _edges(m.faces)
    mean = np.linalg.norm(pts[e0[:, 0]] - pts[e0[:, 1]], axis=1).mean()
    p, t = E.split_long_edges(pts, m.faces, ratio)
    np.testing.assert_array_equal(p[: pts.shape[0]], pts)          # vertices keep their ids
    np.testing.assert_array_equal(p, p.astype(np.float32))         # midpoints stored as floats
    e, cnt = _edges(t)
    assert np.all(cnt == 2)                                        # still closed and manifold
    assert np.linalg.norm(p[e[:, 0]] - p[e[:, 1]], axis=1).max() <= ratio * mean
    assert p.shape[0] - t.shape[0] // 2 == pts.shape[0] - m.faces.shape[0] // 2   # Euler: V - F/2 kept
    assert abs(_area(p, t) - _area(pts, m.faces)) < 1e-5 * _area(pts, m.faces)
    if ratio < 1.5:
        assert p.shape[0] > pts.shape[0]
    elif np.linalg.norm(pts[e0[:, 0]] - pts[e0[:, 1]], axis=1).max() <= ratio * mean:
        np.testing.assert_array_equal(t, m.faces)                  # nothing to split: unchanged
    # orientation kept: every interior edge is used once in each direction
    d = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    assert len({tuple(x) for x in d.tolist()}) == d.shape[0]


def test_split_long_edges_option_order(tmp_path):
    """-l before -ft: the face ids refer to the split mesh (the reference's argument loop)."""
    from acvd_gb300 import cli
    pts = np.array([[0, 0, 0], [4, 0, 0], [0, 1, 0]], dtype=np.float64)
    mesh = acvd_gb300.Surface(pts, np.array([[0, 1, 2]], dtype=np.int32))
    (tmp_path / "f.txt").write_text("2\n")
    opts = cli._parse(["m.ply", "3", "0", "-l", "1", "-ft", str(tmp_path / "f.txt")], "ACVDQ")
    out, fixed = cli._mesh_options(opts, mesh, True)
    assert out.GetNumberOfPoints() == 5
    np.testing.assert_array_equal(fixed, [0, 3, 4])               # face 2 of the split mesh: (0, 3, 4)
    opts = cli._parse(["m.ply", "3", "0", "-ft", str(tmp_path / "f.txt"), "-l", "1"], "ACVDQ")
    with pytest.raises(IndexError):                                # face 2 does not exist before the split
        cli._mesh_options(opts, mesh, True)


def _density_volume(tmp_path, kind):
    """A 7 x 5 x 4 float volume, origin (-1.5, -1, -0.8), spacing (0.5, 0.5, 0.6)."""
    import zlib
    dims = (7, 5, 4)
    vol = np.arange(np.prod(dims), dtype=np.float32).reshape(dims[::-1]) * 10.0   # z, y, x
    head = ("ObjectType = Image\nNDims = 3\nDimSize = 7 5 4\nElementSpacing = 0.5 0.5 0.6\n"
            "Offset = -1.5 -1 -0.8\nElementNumberOfChannels = 1\n")
    if kind == "mhd_raw":
        (tmp_path / "d.raw").write_bytes(vol.astype(">f4").tobytes())
        (tmp_path / "d.mhd").write_text(head + "ElementType = MET_FLOAT\nElementByteOrderMSB = True\n"
                                        "ElementDataFile = d.raw\n")
        return str(tmp_path / "d.mhd"), vol
    data = zlib.compress(vol.astype(np.uint16).tobytes())
    (tmp_path / "d.mha").write_bytes((head + "ElementType = MET_USHORT\nCompressedData = True\n"
                                      f"CompressedDataSize = {len(data)}\nElementDataFile = LOCAL\n").encode() + data)
    return str(tmp_path / "d.mha"), vol.astype(np.uint16).astype(np.float64)


@pytest.mark.parametrize("kind", ["mhd_raw", "mha_zlib"])
def test_custom_density_indicator(tmp_path, kind):
    """vtkDiscreteRemeshing's InputDensityFile: the voxel at the cell holding each vertex
    (the last cell at the upper face, 0 outside), mapped to max(cmax - value * cf, cmin)."""
    path, vol = _density_volume(tmp_path, kind)
    origin, spacing, dims = np.array([-1.5, -1, -0.8]), np.array([0.5, 0.5, 0.6]), np.array([7, 5, 4])
    rng = np.random.default_rng(0)
    pts = rng.uniform(origin - 0.3, origin + spacing * (dims - 1) + 0.3, size=(400, 3))
    pts[0] = origin + spacing * (dims - 1)          # the upper corner: last cell
    pts[1] = origin                                  # the lower corner
    got = E.density_indicator(path, pts, 60.0, 0.5, 0.25)
    d = (pts - origin) / spacing
    inside = np.all((d >= 0) & (d <= dims - 1), axis=1)
    ijk = np.minimum(np.floor(d).astype(int), dims - 2)
    val = np.where(inside, vol[ijk[:, 2].clip(0, 3), ijk[:, 1].clip(0, 4), ijk[:, 0].clip(0, 6)], 0.0)
    want = np.maximum(60.0 - val * 0.25, 0.5)
    np.testing.assert_array_equal(got, want)
    assert inside.sum() > 100 and (~inside).sum() > 20
    with pytest.raises(acvd_gb300.AcvdError):
        E.density_indicator(str(tmp_path / "v.mnc"), pts)



@pytest.mark.parametrize("header", [
    "DimSize = 4294967296 4294967296 16\n",                        # 2^68 voxels: the byte count would wrap
    "DimSize = 7 5 4\nElementNumberOfChannels = 4611686018427387904\n",   # channels x size would wrap
    "DimSize = 100000 100000 100000\n",                             # above the voxel cap
])
def test_oversized_density_volume_is_refused(tmp_path, header):
    """DimSize / ElementNumberOfChannels whose byte count would overflow are refused
    before any data is read (ACVD_ERR_ARG), not wrapped into a short read."""
    (tmp_path / "big.mha").write_bytes((
        "ObjectType = Image\nNDims = 3\n" + header + "ElementType = MET_UCHAR\nElementDataFile = LOCAL\n").encode()
        + bytes(64))
    with pytest.raises(acvd_gb300.AcvdError):
        E.density_indicator(str(tmp_path / "big.mha"), np.zeros((3, 3)))
