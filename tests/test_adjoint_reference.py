"""The FP64 torch reference of the adjoint against the oracle (CPU only).

Its energy must equal the restatement's evaluation of the same clustering, and
its autograd gradient must match central differences of the restatement's own
per-cluster energies (step 1e-6) -- which pins the reference the GPU adjoint is
compared with.
"""
import numpy as np
import pytest
import torch

from acvd_gb300 import synth
from acvd_gb300.adjoint import reference_energy


def _setup(O):
    m = synth.torus(40, 24, seed=3)
    k = 48
    rho = np.random.default_rng(2).uniform(0.5, 2.0, m.n_points)
    p = O.Port("qem", m.points, m.faces, k, 1.0, rho, unconstrained_init=1)
    p.init(None)
    p.run()
    return m, k, rho, p.labels()


def _port_energies(O, points, faces, k, rho, lab):
    p = O.Port("qem", points, faces, k, 1.0, rho)
    p.evaluate(lab, 1)
    return p.clusters()["energy"]


def test_reference_energy_equals_oracle(oracle_lib):
    m, k, rho, lab = _setup(oracle_lib)
    x = torch.tensor(m.points, dtype=torch.float64)
    E, _ = reference_energy(x, m.faces, lab, k, torch.tensor(rho), 1.0)
    e_port = _port_energies(oracle_lib, m.points, m.faces, k, rho, lab).sum()
    assert abs(float(E) - e_port) < 1e-11 * abs(e_port)


def test_reference_gradient_matches_central_differences(oracle_lib):
    m, k, rho, lab = _setup(oracle_lib)
    x = torch.tensor(m.points, dtype=torch.float64, requires_grad=True)
    r = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    E, _ = reference_energy(x, m.faces, lab, k, r, 1.0)
    E.backward()
    gx, gr = x.grad.numpy(), r.grad.numpy()
    rng = np.random.default_rng(5)
    h = 1e-6
    for _ in range(16):
        i, d = int(rng.integers(m.n_points)), int(rng.integers(3))
        pp, pm = m.points.copy(), m.points.copy()
        pp[i, d] += h
        pm[i, d] -= h
        fd = np.sum(_port_energies(oracle_lib, pp, m.faces, k, rho, lab)
                    - _port_energies(oracle_lib, pm, m.faces, k, rho, lab)) / (2 * h)
        assert abs(fd - gx[i, d]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(gx).max()), (i, d, fd, gx[i, d])
    for _ in range(8):
        i = int(rng.integers(m.n_points))
        rp, rm = rho.copy(), rho.copy()
        rp[i] += h
        rm[i] -= h
        fd = np.sum(_port_energies(oracle_lib, m.points, m.faces, k, rp, lab)
                    - _port_energies(oracle_lib, m.points, m.faces, k, rm, lab)) / (2 * h)
        assert abs(fd - gr[i]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(gr).max()), (i, fd, gr[i])
