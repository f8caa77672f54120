"""The ACVD / ACVDQ command-line drivers end to end on the GPU: file in, remesh
(with subdivision, ForceManifold, boundary fixing and the quadric post-placement as the
options ask), file out."""
import os

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import cli, synth
from acvd_gb300 import engine as E

pytestmark = pytest.mark.gpu


def test_acvd_program(tmp_path):
    m = synth.torus(80, 40, seed=2)
    src = str(tmp_path / "in.ply")
    E.write_mesh(src, m.points, m.faces)
    out = str(tmp_path / "out")
    os.makedirs(out)
    assert cli.main_acvd([src, "300", "0.5", "-o", out, "-of", "coarse.obj", "-q", "2"]) == 0
    smooth = E.read_mesh(out + "smooth_coarse.obj")           # written before the post-placement
    final = E.read_mesh(os.path.join(out, "coarse.obj"))
    assert smooth[0].shape == final[0].shape == (300, 3)
    np.testing.assert_array_equal(smooth[1], final[1])
    assert not np.array_equal(smooth[0], final[0])


def test_acvdq_program_with_subdivision_and_options(tmp_path):
    h = synth.heightfield(30, seed=2)                          # 900 vertices, open
    src = str(tmp_path / "in.off")
    E.write_mesh(src, h.points, h.faces)
    dst = str(tmp_path) + "/"
    assert cli.main_acvdq([src, "200", "0", "-o", dst, "-of", "q.vtk", "-m", "1", "-b", "1", "-q", "2"]) == 0
    # 900 < 10 x 200: subdivided twice before clustering; written as PLY whatever the name
    raw = open(dst + "q.vtk", "rb").read(3)
    assert raw == b"ply"
    os.replace(dst + "q.vtk", dst + "q.ply")
    pts, tri = E.read_mesh(dst + "q.ply")
    assert pts.shape[0] > 200                                  # boundary vertices appended
    assert tri.max() < pts.shape[0]


@pytest.mark.parametrize("prog,args", [
    ("acvd", ["300", "0.5", "-q", "2"]),
    ("acvdq", ["200", "0", "-m", "1", "-b", "1", "-q", "2"]),
    ("anisotropic_remeshing_q", ["300", "0.5", "-b", "1", "-q", "2", "-m", "1"]),
    ("acvd", ["300", "0.5", "-l", "0.9", "-q", "1"]),
    ("acvdq", ["200", "1.5", "-cd", "DENSITY", "-cmax", "2", "-cmin", "0.2", "-cf", "0.01"]),
])
def test_native_programs_match_the_python_drivers(tmp_path, prog, args):
    """The native programs (C++ over the C ABI) and the Python drivers run the same steps:
    their output files are byte for byte the same."""
    import subprocess
    from acvd_gb300 import build as B
    mesh = {"acvd": lambda: synth.torus(80, 40, seed=2), "acvdq": lambda: synth.heightfield(30, seed=2),
            "anisotropic_remeshing_q": lambda: synth.heightfield(64, seed=4)}[prog]()
    src = str(tmp_path / "in.ply")
    E.write_mesh(src, mesh.points, mesh.faces)
    if "DENSITY" in args:   # a volume over the mesh's bounding box
        vol = np.arange(8 * 8 * 8, dtype=np.float32) % 97
        lo = mesh.points.min(axis=0) - 0.01
        sp = (mesh.points.max(axis=0) + 0.01 - lo) / 7
        (tmp_path / "d.raw").write_bytes(vol.tobytes())
        (tmp_path / "d.mhd").write_text("ObjectType = Image\nNDims = 3\nDimSize = 8 8 8\n"
                                        f"ElementSpacing = {sp[0]!r} {sp[1]!r} {sp[2]!r}\n"
                                        f"Offset = {lo[0]!r} {lo[1]!r} {lo[2]!r}\n"
                                        "ElementType = MET_FLOAT\nElementDataFile = d.raw\n")
        args = [str(tmp_path / "d.mhd") if a == "DENSITY" else a for a in args]
    native, python = tmp_path / "native", tmp_path / "python"
    native.mkdir()
    python.mkdir()
    r = subprocess.run([os.path.join(B.OUT, prog), src] + args + ["-o", str(native) + "/"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    main = {"acvd": cli.main_acvd, "acvdq": cli.main_acvdq,
            "anisotropic_remeshing_q": cli.main_anisotropic_remeshing_q}[prog]
    assert main([src] + args + ["-o", str(python) + "/"]) == 0
    names = sorted(os.listdir(native))
    assert names == sorted(os.listdir(python)) and names
    for n in names:
        assert (native / n).read_bytes() == (python / n).read_bytes(), n


@pytest.mark.parametrize("key", ["-fv", "-ft"])
def test_acvdq_fixed_vertices(tmp_path, key, capfd):
    """ACVDQ -fv / -ft (ACVDQ.cxx:246-280, 327-363): the fixed vertices are the first
    output vertices, unchanged; the native program and the Python driver write the same
    file."""
    import subprocess
    from acvd_gb300 import build as B
    m = synth.torus(80, 40, seed=2)
    src = str(tmp_path / "in.ply")
    E.write_mesh(src, m.points, m.faces)
    pts, tri = E.read_mesh(src)                                 # as stored (float)
    if key == "-fv":
        fixed = np.array([5, 77, 400, 1203, 2900], dtype=np.int32)
        (tmp_path / "ids.txt").write_text(" ".join(str(v) for v in fixed) + "\n")
    else:
        faces = np.array([10, 3000, 5100], dtype=np.int32)
        fixed = np.unique(tri[faces].reshape(-1)).astype(np.int32)
        (tmp_path / "ids.txt").write_text("\n".join(str(f) for f in faces))
    native, python = tmp_path / "native", tmp_path / "python"
    native.mkdir()
    python.mkdir()
    args = [src, "250", "0.5", key, str(tmp_path / "ids.txt")]
    r = subprocess.run([os.path.join(B.OUT, "acvdq")] + args + ["-o", str(native) + "/"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert "Constraints on vertices have been checked" in r.stdout
    assert cli.main_acvdq(args + ["-o", str(python) + "/"]) == 0
    assert "Constraints on vertices have been checked" in capfd.readouterr().out
    out_pts, _ = E.read_mesh(str(python / "simplification.ply"))
    assert out_pts.shape[0] == 250 + len(fixed)
    np.testing.assert_array_equal(out_pts[: len(fixed)], pts[fixed])
    assert (native / "simplification.ply").read_bytes() == (python / "simplification.ply").read_bytes()


def test_resume_from_a_saved_clustering(tmp_path):
    """A clustering saved to clustering.dat and loaded again (the reference's load path:
    no minimisation) gives the same clustering and the same coarse mesh."""
    m = synth.torus(60, 30, seed=5)
    r = acvd_gb300.QIsotropicDiscreteRemeshing()
    r.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r.SetNumberOfClusters(150)
    r.Remesh()
    r.SaveClustering(str(tmp_path / "clustering.dat"))
    r2 = acvd_gb300.QIsotropicDiscreteRemeshing()
    r2.SetInput(acvd_gb300.Surface(m.points, m.faces))
    r2.SetNumberOfClusters(150)
    r2.LoadClustering(str(tmp_path / "clustering.dat"))
    r2.Remesh()
    np.testing.assert_array_equal(r2.GetClustering(), r.GetClustering())
    assert r2.Stats is None                                     # nothing was minimised
    np.testing.assert_array_equal(r2.GetOutput().points, r.GetOutput().points)
    np.testing.assert_array_equal(r2.GetOutput().faces, r.GetOutput().faces)
