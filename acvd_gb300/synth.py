"""Seeded synthetic triangle meshes for the clustering workloads.

The reference's own smoke script fetches public scanned models over the network
(`test.sh:1-10`); none of them is available here, so these generators stand in
for them.  Every generator returns a `SynthMesh` with

* ``points``  float64 (nV, 3) coordinates (already rounded through float32 when
  the workload asks for fp32 positions, so every consumer sees the same values),
* ``faces``   int32 (nF, 3) triangles, consistently oriented,
* ``indicator`` float64 (nV,) per-vertex curvature indicator or density
  (None when the workload has gradation 0),
* ``principal_dirs`` float32 (nV, 6) principal directions scaled by
  sqrt(|kappa|), largest |kappa| first (None unless the anisotropic metric needs
  them).

The curvature data are computed analytically from the smooth parametric surface
(not by the reference's polynomial fitting in `Common/vtkCurvatureMeasure.cxx:188`),
following the output convention of `vtkCurvatureMeasure.cxx:440-482`: indicator =
sqrt(k1^2 + k2^2), direction j = sqrt(|k_j|) * e_j, swapped so that the larger
|k| comes first.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class SynthMesh:
    name: str
    points: np.ndarray
    faces: np.ndarray
    indicator: np.ndarray | None = None
    principal_dirs: np.ndarray | None = None
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.faces.shape[0])


# --------------------------------------------------------------------------
# curvature from first/second fundamental forms
# --------------------------------------------------------------------------

def _principal_from_forms(Pu, Pv, Puu, Puv, Pvv):
    """Principal curvatures/directions from parametric derivatives (vectorised).

    Returns (indicator, dirs6) with dirs6 = [sqrt|k1| e1, sqrt|k2| e2], |k1|>=|k2|.
    """
    n = np.cross(Pu, Pv)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    E = np.einsum("ij,ij->i", Pu, Pu)
    F = np.einsum("ij,ij->i", Pu, Pv)
    G = np.einsum("ij,ij->i", Pv, Pv)
    L = np.einsum("ij,ij->i", Puu, n)
    M = np.einsum("ij,ij->i", Puv, n)
    N = np.einsum("ij,ij->i", Pvv, n)
    det = E * G - F * F
    # shape operator S = I^-1 II (2x2, not symmetric in this basis)
    s11 = (G * L - F * M) / det
    s12 = (G * M - F * N) / det
    s21 = (E * M - F * L) / det
    s22 = (E * N - F * M) / det
    tr = s11 + s22
    dt = s11 * s22 - s12 * s21
    disc = np.sqrt(np.maximum(tr * tr / 4.0 - dt, 0.0))
    k1 = tr / 2.0 + disc
    k2 = tr / 2.0 - disc
    # eigenvector of S for eigenvalue k: (s12, k - s11) or (k - s22, s21)
    def evec(k):
        a1, b1 = s12, k - s11
        a2, b2 = k - s22, s21
        use2 = (a2 * a2 + b2 * b2) > (a1 * a1 + b1 * b1)
        a = np.where(use2, a2, a1)
        b = np.where(use2, b2, b1)
        d = a[:, None] * Pu + b[:, None] * Pv
        nrm = np.linalg.norm(d, axis=1, keepdims=True)
        # umbilic points: any unit tangent
        fallback = Pu / np.linalg.norm(Pu, axis=1, keepdims=True)
        bad = (nrm[:, 0] < 1e-300)
        d = np.where(bad[:, None], fallback, d / np.where(bad[:, None], 1.0, nrm))
        return d
    e1 = evec(k1)
    # second direction: orthogonal to e1 in the tangent plane
    e2 = np.cross(n, e1)
    swap = np.abs(k1) < np.abs(k2)
    ka = np.where(swap, k2, k1)
    kb = np.where(swap, k1, k2)
    ea = np.where(swap[:, None], e2, e1)
    eb = np.where(swap[:, None], e1, e2)
    dirs = np.concatenate([np.sqrt(np.abs(ka))[:, None] * ea,
                           np.sqrt(np.abs(kb))[:, None] * eb], axis=1)
    ind = np.sqrt(k1 * k1 + k2 * k2)
    return ind, dirs.astype(np.float32)


# --------------------------------------------------------------------------
# icosphere (configuration: isotropic ACVD, 10,242 vertices at level 5)
# --------------------------------------------------------------------------

def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def _subdivide_sphere(v, f):
    """One 1->4 split; midpoints are projected back onto the unit sphere."""
    nv = v.shape[0]
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    key = np.sort(e, axis=1)
    uniq, inv = np.unique(key[:, 0] * (nv + 1) + key[:, 1], return_inverse=True)
    a = uniq // (nv + 1)
    b = uniq % (nv + 1)
    mid = v[a] + v[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    nF = f.shape[0]
    m01 = nv + inv[:nF]
    m12 = nv + inv[nF:2 * nF]
    m20 = nv + inv[2 * nF:]
    f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
    nf = np.stack([
        np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
        np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=1).reshape(-1, 3)
    return np.concatenate([v, mid], axis=0), nf


def icosphere(level: int = 5, seed: int = 0, noise: float = 0.002,
              fp32: bool = False, with_curvature: bool = False) -> SynthMesh:
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide_sphere(v, f)
    rng = np.random.default_rng(seed)
    d = rng.uniform(-noise, noise, size=v.shape[0])
    v = v * (1.0 + d)[:, None]          # along the (radial) normal of the unit sphere
    if fp32:
        v = v.astype(np.float32).astype(np.float64)
    m = SynthMesh(f"icosphere{level}", v, f.astype(np.int32),
                  meta={"kind": "icosphere", "level": level, "seed": seed, "noise": noise})
    if with_curvature:
        # curvature of the underlying unit sphere: umbilic, k1 = k2 = 1
        n = v / np.linalg.norm(v, axis=1, keepdims=True)
        ref = np.where(np.abs(n[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
        e1 = np.cross(n, ref)
        e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
        e2 = np.cross(n, e1)
        m.indicator = np.full(v.shape[0], math.sqrt(2.0))
        m.principal_dirs = np.concatenate([e1, e2], axis=1).astype(np.float32)
    return m


# --------------------------------------------------------------------------
# torus with normal bumps (configurations: ACVDQ and the adjoint workload)
# --------------------------------------------------------------------------

def _torus_bumps(seed: int, n_bumps: int = 8):
    rng = np.random.default_rng(seed)
    mk = rng.integers(2, 17, size=n_bumps)
    nk = rng.integers(2, 17, size=n_bumps)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=n_bumps)
    return mk.astype(np.float64), nk.astype(np.float64), ph


def _torus_point(u, v, R, r, amp, mk, nk, ph):
    cu, su, cv, sv = np.cos(u), np.sin(u), np.cos(v), np.sin(v)
    h = np.zeros_like(u)
    for m_, n_, p_ in zip(mk, nk, ph):
        h = h + amp * np.sin(m_ * u + n_ * v + p_)
    nrm = np.stack([cv * cu, cv * su, sv], axis=1)
    base = np.stack([(R + r * cv) * cu, (R + r * cv) * su, r * sv], axis=1)
    return base + h[:, None] * nrm


def torus(nu: int = 1024, nv: int = 512, R: float = 1.0, r: float = 0.3,
          amp: float = 0.01, n_bumps: int = 8, seed: int = 0, fp32: bool = True,
          with_curvature: bool = True) -> SynthMesh:
    mk, nk, ph = _torus_bumps(seed, n_bumps)
    i = np.repeat(np.arange(nu), nv)
    j = np.tile(np.arange(nv), nu)
    u = 2.0 * math.pi * i / nu
    v = 2.0 * math.pi * j / nv
    P = _torus_point(u, v, R, r, amp, mk, nk, ph)
    if fp32:
        P = P.astype(np.float32).astype(np.float64)
    ii = np.repeat(np.arange(nu), nv)
    jj = np.tile(np.arange(nv), nu)
    v00 = ii * nv + jj
    v10 = ((ii + 1) % nu) * nv + jj
    v01 = ii * nv + (jj + 1) % nv
    v11 = ((ii + 1) % nu) * nv + (jj + 1) % nv
    faces = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    m = SynthMesh(f"torus{nu}x{nv}", P, faces.astype(np.int32),
                  meta={"kind": "torus", "nu": nu, "nv": nv, "R": R, "r": r, "amp": amp,
                        "bumps_m": mk.tolist(), "bumps_n": nk.tolist(), "seed": seed})
    if with_curvature:
        h = 1e-4
        f = lambda uu, vv: _torus_point(uu, vv, R, r, amp, mk, nk, ph)
        Pu = (f(u + h, v) - f(u - h, v)) / (2 * h)
        Pv = (f(u, v + h) - f(u, v - h)) / (2 * h)
        P0 = f(u, v)
        Puu = (f(u + h, v) - 2 * P0 + f(u - h, v)) / (h * h)
        Pvv = (f(u, v + h) - 2 * P0 + f(u, v - h)) / (h * h)
        Puv = (f(u + h, v + h) - f(u + h, v - h) - f(u - h, v + h) + f(u - h, v - h)) / (4 * h * h)
        m.indicator, m.principal_dirs = _principal_from_forms(Pu, Pv, Puu, Puv, Pvv)
    return m


# --------------------------------------------------------------------------
# heightfield (configuration: quadric-anisotropic clustering)
# --------------------------------------------------------------------------

def _heightfield_octaves(seed: int, n_oct: int = 6):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, 2.0 * math.pi, size=n_oct)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=n_oct)
    return np.cos(ang), np.sin(ang), ph


def heightfield(n: int = 4096, n_oct: int = 6, amp0: float = 0.05, seed: int = 0,
                fp32: bool = True, with_curvature: bool = True, ny: int | None = None) -> SynthMesh:
    ny = n if ny is None else ny
    a, b, ph = _heightfield_octaves(seed, n_oct)
    ii = np.repeat(np.arange(n, dtype=np.int64), ny)
    jj = np.tile(np.arange(ny, dtype=np.int64), n)
    x = ii / (n - 1.0)
    y = jj / (ny - 1.0)
    z = np.zeros_like(x)
    zx = np.zeros_like(x); zy = np.zeros_like(x)
    zxx = np.zeros_like(x); zxy = np.zeros_like(x); zyy = np.zeros_like(x)
    for k in range(n_oct):
        A = amp0 / (2 ** k)
        w = 2.0 * math.pi * (2 ** k)
        arg = w * (a[k] * x + b[k] * y) + ph[k]
        s, c = np.sin(arg), np.cos(arg)
        z += A * s
        if with_curvature:
            zx += A * w * a[k] * c
            zy += A * w * b[k] * c
            zxx -= A * w * w * a[k] * a[k] * s
            zxy -= A * w * w * a[k] * b[k] * s
            zyy -= A * w * w * b[k] * b[k] * s
    P = np.stack([x, y, z], axis=1)
    if fp32:
        P = P.astype(np.float32).astype(np.float64)
    v00 = ii * ny + jj
    mask = (ii < n - 1) & (jj < ny - 1)
    v00 = v00[mask]
    v10 = v00 + ny
    v01 = v00 + 1
    v11 = v00 + ny + 1
    faces = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    m = SynthMesh(f"heightfield{n}x{ny}", P, faces.astype(np.int32),
                  meta={"kind": "heightfield", "n": n, "ny": ny, "seed": seed, "octaves": n_oct})
    if with_curvature:
        one = np.ones_like(x); zero = np.zeros_like(x)
        Pu = np.stack([one, zero, zx], 1)
        Pv = np.stack([zero, one, zy], 1)
        Puu = np.stack([zero, zero, zxx], 1)
        Puv = np.stack([zero, zero, zxy], 1)
        Pvv = np.stack([zero, zero, zyy], 1)
        m.indicator, m.principal_dirs = _principal_from_forms(Pu, Pv, Puu, Puv, Pvv)
    return m


# --------------------------------------------------------------------------
# small hand meshes for topology tests
# --------------------------------------------------------------------------

def tetrahedron() -> SynthMesh:
    p = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64)
    f = np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], dtype=np.int32)
    return SynthMesh("tetrahedron", p, f, meta={"kind": "tetrahedron"})


def octahedron() -> SynthMesh:
    p = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], dtype=np.float64)
    f = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4],
                  [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]], dtype=np.int32)
    return SynthMesh("octahedron", p, f, meta={"kind": "octahedron"})


def grid(n: int = 4, seed: int = 0) -> SynthMesh:
    """Flat n x n vertex grid with a boundary and a little in-plane jitter."""
    m = heightfield(n, n_oct=1, amp0=0.0, seed=seed, fp32=False, with_curvature=False)
    rng = np.random.default_rng(seed)
    m.points[:, :2] += rng.uniform(-0.1, 0.1, size=(m.n_points, 2)) / n
    m.name = f"grid{n}"
    m.meta = {"kind": "grid", "n": n, "seed": seed}
    return m


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------

def seed_labels(n_items: int, k: int, seed: int = 0) -> np.ndarray:
    """K single-item seeds (first K of a seeded shuffle); all other items null (=K)."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_items)[:k]
    lab = np.full(n_items, k, dtype=np.int32)
    lab[perm] = np.arange(k, dtype=np.int32)
    return lab


def batch_specs(n_meshes: int = 256, seed: int = 0, lo: int = 2000, hi: int = 500000):
    """(kind, size parameters) for the batched workload: type uniform over the three
    generators, vertex count log-uniform in [lo, hi] realised by grid dimensions or
    the nearest icosphere subdivision level."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_meshes):
        kind = ["icosphere", "torus", "heightfield"][int(rng.integers(0, 3))]
        target = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        if kind == "icosphere":
            # 10 * 4^L + 2 vertices
            lvl = int(round(math.log(max(target - 2, 12) / 10.0, 4)))
            lvl = max(2, min(lvl, 7))
            specs.append(("icosphere", {"level": lvl, "seed": seed + i}))
        elif kind == "torus":
            nv = max(8, int(round(math.sqrt(target / 2.0))))
            nu = max(8, int(round(target / nv)))
            specs.append(("torus", {"nu": nu, "nv": nv, "seed": seed + i}))
        else:
            s = max(8, int(round(math.sqrt(target))))
            specs.append(("heightfield", {"n": s, "seed": seed + i}))
    return specs


def make(kind: str, **kw) -> SynthMesh:
    return {"icosphere": icosphere, "torus": torus, "heightfield": heightfield,
            "tetrahedron": tetrahedron, "octahedron": octahedron, "grid": grid}[kind](**kw)


WORKLOADS = {
    # name: (mesh builder kwargs, metric, K, gradation)
    "icosphere_l5_iso": (("icosphere", {"level": 5, "seed": 0}), "iso", 1000, 0.0),
    "torus_1024x512_qem": (("torus", {"nu": 1024, "nv": 512, "seed": 0}), "qem", 20000, 1.5),
    "heightfield_4096_aniso": (("heightfield", {"n": 4096, "seed": 0}), "aniso", 200000, 1.5),
    "torus_512x512_qem": (("torus", {"nu": 512, "nv": 512, "seed": 0}), "qem", 10000, 1.0),
}
