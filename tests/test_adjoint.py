"""GPU adjoint against the FP64 references (needs a GB300).

Fixed clustering of a bumped torus with densities U[0.5, 2] as the indicator
(gradation 1, weights = area * rho), at 128x64 with K = 600 and at the adjoint
workload's full size (512x512, 262,144 items, K = 10,000):
  * the energy equals the oracle's evaluation of the clustering (1e-10 relative);
  * gradients of  E + sum_k G_k . c_k  match the FP64 torch reference for every
    coordinate and density (1e-6 of the largest component);
  * energy gradients match FP64 central differences (step 1e-6) of the
    per-cluster energies on 64 random coordinates and 16 densities (1e-4 relative).
"""
import numpy as np
import pytest
import torch

import acvd_gb300
from acvd_gb300 import synth
from acvd_gb300.adjoint import ClusteringEnergy, cluster_energies, reference_energy

pytestmark = pytest.mark.gpu


SIZES = {"torus128x64_k600": (128, 64, 5, 600), "torus512x512_k10000": (512, 512, 0, 10000)}


@pytest.fixture(scope="module", params=sorted(SIZES))
def setup(oracle_lib, request):
    nu, nv, seed, k = SIZES[request.param]
    m = synth.torus(nu, nv, seed=seed)
    rho = np.random.default_rng(3).uniform(0.5, 2.0, m.n_points)
    p = oracle_lib.Port("qem", m.points, m.faces, k, 1.0, rho, unconstrained_init=1)
    p.init(None)
    p.run()
    lab = p.labels()
    row, col, ev = acvd_gb300.build_topology(m.n_points, m.faces)
    e = acvd_gb300.Engine()
    e.set_mesh(m.points, m.faces, row, col, ev)
    e.set_metric("qem", rho, None, 1.0)
    e.set_labels(k, lab)
    yield m, k, rho, lab, e
    e.close()


def test_energy_matches_oracle(setup, oracle_lib):
    m, k, rho, lab, e = setup
    x = torch.tensor(m.points, dtype=torch.float64, device="cuda")
    r = torch.tensor(rho, dtype=torch.float64, device="cuda")
    E, C = ClusteringEnergy.apply(x, r, e, 1.0)
    p = oracle_lib.Port("qem", m.points, m.faces, k, 1.0, rho)
    p.evaluate(lab, 1)
    e_ref = p.global_energy()
    assert abs(float(E) - e_ref) < 1e-10 * abs(e_ref)
    np.testing.assert_allclose(C.cpu().numpy(), p.clusters()["centroid"], rtol=0, atol=1e-9)


def test_gradients_match_fp64_reference(setup):
    m, k, rho, lab, e = setup
    G = torch.tensor(np.random.default_rng(7).normal(size=(k, 3)), dtype=torch.float64)
    x = torch.tensor(m.points, dtype=torch.float64, device="cuda", requires_grad=True)
    r = torch.tensor(rho, dtype=torch.float64, device="cuda", requires_grad=True)
    E, C = ClusteringEnergy.apply(x, r, e, 1.0)
    (E + (C * G.cuda()).sum()).backward()
    xr = torch.tensor(m.points, dtype=torch.float64, requires_grad=True)
    rr = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    Er, Cr = reference_energy(xr, m.faces, lab, k, rr, 1.0)
    (Er + (Cr * G).sum()).backward()
    gx, gxr = x.grad.cpu().numpy(), xr.grad.numpy()
    gr, grr = r.grad.cpu().numpy(), rr.grad.numpy()
    assert np.max(np.abs(gx - gxr)) <= 1e-6 * np.max(np.abs(gxr))
    assert np.max(np.abs(gr - grr)) <= 1e-6 * np.max(np.abs(grr))


def test_gradients_match_central_differences(setup):
    m, k, rho, lab, e = setup
    x = torch.tensor(m.points, dtype=torch.float64, device="cuda", requires_grad=True)
    r = torch.tensor(rho, dtype=torch.float64, device="cuda", requires_grad=True)
    E, _ = ClusteringEnergy.apply(x, r, e, 1.0)
    E.backward()
    gx, gr = x.grad.cpu().numpy(), r.grad.cpu().numpy()
    rng = np.random.default_rng(11)
    h = 1e-6
    xb = torch.tensor(m.points, dtype=torch.float64, device="cuda")
    rb = torch.tensor(rho, dtype=torch.float64, device="cuda")
    for _ in range(64):
        i, d = int(rng.integers(m.n_points)), int(rng.integers(3))
        xp, xm = xb.clone(), xb.clone()
        xp[i, d] += h
        xm[i, d] -= h
        fd = float((cluster_energies(e, xp, rb, 1.0) - cluster_energies(e, xm, rb, 1.0)).sum()) / (2 * h)
        assert abs(fd - gx[i, d]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(gx).max()), (i, d, fd, gx[i, d])
    for _ in range(16):
        i = int(rng.integers(m.n_points))
        rp, rm = rb.clone(), rb.clone()
        rp[i] += h
        rm[i] -= h
        fd = float((cluster_energies(e, xb, rp, 1.0) - cluster_energies(e, xb, rm, 1.0)).sum()) / (2 * h)
        assert abs(fd - gr[i]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(gr).max()), (i, fd, gr[i])
