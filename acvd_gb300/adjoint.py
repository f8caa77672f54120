"""Gradients of the clustering energy and of the placed cluster vertices for a
fixed clustering: a libtorch torch::autograd::Function (csrc/adjoint_torch.cpp) over
acvd_adjoint_on_stream (C ABI).

    E, C = ClusteringEnergy.apply(xyz, rho, engine, gradation)
    (E * 1.0 + (C * target).sum()).backward()   # -> xyz.grad, rho.grad

xyz: (N, 3) float32/float64 CUDA tensor of vertex positions; rho: (N,) densities
(the metric's per-vertex indicator; weight = dual area * rho^gradation) or None.
The clustering is the engine's current labels.  The backward recomputes the
cluster sums (no per-item intermediates are kept) and holds each cluster's
pseudo-inverse rank fixed.

`reference_energy` is an independent FP64 formulation of the same function in
plain torch (CPU autograd) used by the tests.
"""
from __future__ import annotations

import ctypes

import torch

from . import engine as _eng


def _ptr(t):
    return None if t is None else int(t.data_ptr())


_EXT = None


def _extension():
    """The libtorch extension (csrc/adjoint_torch.cpp), bound to the C ABI of the
    library instance this package loaded."""
    global _EXT
    if _EXT is None:
        from . import build as _build
        mod = _build.load_torch_extension()
        lib = _eng.load()
        mod.bind(ctypes.cast(lib.acvd_adjoint_on_stream, ctypes.c_void_p).value,
                 ctypes.cast(lib.acvd_last_error, ctypes.c_void_p).value)
        _EXT = mod
    return _EXT


class ClusteringEnergy:
    """E, C = ClusteringEnergy.apply(xyz, rho, engine, gradation): the libtorch
    torch::autograd::Function of csrc/adjoint_torch.cpp (forward and backward on
    torch's current stream through acvd_adjoint_on_stream, no host waits)."""

    @staticmethod
    def apply(xyz, rho, engine: "_eng.Engine", gradation: float):
        E, C = _extension().clustering_energy(xyz, rho, int(engine.ctx), float(gradation), int(engine.k))
        return E, C


def cluster_energies(engine: "_eng.Engine", xyz, rho, gradation: float):
    """Per-cluster energies E_k (FP64, device) of the fixed clustering at xyz / rho."""
    x64 = xyz.detach().to(torch.float64).contiguous()
    r64 = None if rho is None else rho.detach().to(torch.float64).contiguous()
    ek = torch.empty(engine.k, dtype=torch.float64, device=xyz.device)
    torch.cuda.current_stream(xyz.device).synchronize()
    engine.adjoint_raw(_ptr(x64), _ptr(r64), gradation, 0.0, None, None, None, None, _ptr(ek))
    return ek


def reference_energy(points, faces, labels, k: int, rho=None, gradation: float = 0.0, metric: str = "qem",
                     level: int = 3, thr: float = 1e-3, ratio: float | None = None):
    """FP64 torch formulation (CPU, autograd) of sum_k E_k and of the placed
    vertices c_k for a fixed clustering; the kept eigenvalues of every cluster's
    pseudo-inverse are decided without gradient, as in the forward pass."""
    dt = torch.float64
    N = points.shape[0]
    faces = torch.as_tensor(faces, dtype=torch.int64)
    labels = torch.as_tensor(labels, dtype=torch.int64)
    p0, p1, p2 = points[faces[:, 0]], points[faces[:, 1]], points[faces[:, 2]]
    cr = torch.cross(p1 - p0, p2 - p0, dim=1)
    L = cr.norm(dim=1)
    n = cr / L[:, None]
    area = 0.5 * L
    flat = faces.reshape(-1)
    a = torch.zeros(N, dtype=dt).index_add(0, flat, (area / 3.0).repeat_interleave(3))
    nnT = n[:, :, None] * n[:, None, :]
    Av = torch.zeros(N, 3, 3, dtype=dt).index_add(0, flat, nnT.repeat_interleave(3, dim=0))
    w = a * rho ** gradation if rho is not None else a
    if ratio is None:
        ratio = 10000.0 if metric == "qem" else 100000.0
    with torch.no_grad():
        mean = w.mean()
        clamped = (w > mean * ratio) | (w < mean / ratio)
        wc = torch.clamp(w, min=float(mean / ratio), max=float(mean * ratio))
    w = torch.where(clamped, wc, w)
    bv = (Av @ points[:, :, None])[:, :, 0]
    S = torch.zeros(k, 3, dtype=dt).index_add(0, labels, w[:, None] * points)
    W = torch.zeros(k, dtype=dt).index_add(0, labels, w)
    A = torch.zeros(k, 3, 3, dtype=dt).index_add(0, labels, Av)
    b = torch.zeros(k, 3, dtype=dt).index_add(0, labels, bv)
    m = S / W[:, None]
    if metric == "iso":
        c = m
    else:
        r = b - (A @ m[:, :, None])[:, :, 0]
        with torch.no_grad():
            lam = torch.linalg.eigvalsh(A)
            aw = lam.abs()
            order = torch.argsort(-aw, dim=1)
            mx = aw.max(dim=1).values
            keep_sorted = (torch.gather(aw, 1, order) > thr * mx[:, None]) & (torch.arange(3)[None, :] < level)
            nkeep = keep_sorted.sum(dim=1)
        full = nkeep == 3
        P = torch.zeros(k, 3, 3, dtype=dt)
        if bool(full.any()):
            P = P.index_put((full.nonzero()[:, 0],), torch.linalg.inv(A[full]))
        part = (~full) & (nkeep > 0)
        if bool(part.any()):
            lam_p, V = torch.linalg.eigh(A[part])
            with torch.no_grad():
                awp = lam_p.abs()
                mxp = awp.max(dim=1).values
                rank = torch.argsort(torch.argsort(-awp, dim=1), dim=1)
                keep = (awp > thr * mxp[:, None]) & (rank < level)
            inv = torch.where(keep, 1.0 / lam_p, torch.zeros_like(lam_p))
            Pp = V @ torch.diag_embed(inv) @ V.transpose(1, 2)
            P = P.index_put((part.nonzero()[:, 0],), Pp)
        c = m + (P @ r[:, :, None])[:, :, 0]
    E = W * (c * c).sum(dim=1) - 2.0 * (c * S).sum(dim=1)
    return E.sum(), c
