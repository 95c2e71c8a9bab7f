"""Analytic known answers of the reference's own checks, on the oracle and
the energy helpers (no GPU).

* The single-mode Stokes solution (core/rbc_galerkin.py:500-513): for
  theta = Theta cos(kx x) sin(kz z) with eta = 1, psi = -Ra kx/g^2 Theta
  sin(kx x) sin(kz z) and u_z = Ra kx^2/g^2 theta, g = kx^2 + kz^2.
* Its dissipation (physics/dissipation.py:495-517): <Phi> = Ra^2 kx^2 /
  (4 g^2) Theta^2, and <Phi> = Ra <theta u_z> for this state.
* The BDF2 coefficients at step ratios 1 and 2 and the backward-Euler
  restart (core/implicit_theta.py:706-719).
"""
import numpy as np

from oracle import specmc_oracle as O

RA, THETA = 1e4, 0.7


def _single_mode(model):
    kx, kz = np.pi, np.pi                      # m = n = 1 on the Lx = 2 carrier
    X, Z = np.meshgrid(model.x, model.z, indexing="ij")
    g = kx * kx + kz * kz
    th = THETA * np.cos(kx * X) * np.sin(kz * Z)
    psi = -RA * kx / g ** 2 * THETA * np.sin(kx * X) * np.sin(kz * Z)
    return model.coeffs(th), psi, RA * kx * kx / g ** 2 * th, RA ** 2 * kx ** 2 / (4.0 * g ** 2) * THETA ** 2


def test_single_mode_stokes_and_dissipation():
    from specmc_gb300 import energy
    m = O.ConstModel(Ra=RA, Nx=16, Nz=32)
    that, psi_ref, uz_ref, phi_ref = _single_mode(m)
    psi, _ = m.stokes(that)
    assert np.abs(m.grid(psi) - psi_ref).max() <= 1e-11 * np.abs(psi_ref).max()
    ux, uz = m.velocity(psi)
    assert np.abs(uz - uz_ref).max() <= 1e-11 * np.abs(uz_ref).max()
    phi = energy.phi_integral(m, psi)
    assert abs(phi - phi_ref) <= 1e-10 * phi_ref
    assert abs(energy.pi_theta(m, psi, that) - phi_ref) <= 1e-10 * phi_ref
    # the measured value the reference quotes for Ra = 1e4, kx = kz = pi, amp = 1
    assert abs(phi_ref / THETA ** 2 - 6.3325739776e5) <= 1e-10 * 6.3325739776e5


def test_bdf2_coefficients():
    m = O.DepthModel(Ra=RA, Nx=16, Nz=12, deta_T=10.0)
    dt = 3.0e-4
    m.set_step(dt, dt)
    assert np.allclose([m.a0 * dt, m.b0 * dt, m.b1 * dt], [1.5, 2.0, 0.5], rtol=0, atol=1e-14)
    m.set_step(dt, dt / 2.0)
    assert np.allclose([m.a0 * dt, m.b0 * dt, m.b1 * dt], [5.0 / 3.0, 3.0, 4.0 / 3.0], rtol=0,
                       atol=1e-14)
    n0 = m.n_be_fallback
    m.set_step(dt, None)
    assert (m.a0 * dt, m.b0 * dt, m.b1) == (1.0, 1.0, 0.0) and m.n_be_fallback == n0 + 1
