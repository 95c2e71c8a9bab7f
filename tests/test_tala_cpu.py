"""Host-side pieces of the TALA route, checked on the CPU.

* :mod:`specmc_gb300.compressibility` (the reference state the models expose)
  against the reference's own profiles (tests/golden/tala_ops_16x12.npz).
* The GPU assembles the TALA Schur blocks per operator word D^p M D^q
  (``tala_a12_words`` and ``smc_tala_block_kernel`` in csrc/smc_tala.cu) and
  applies the matrix-free operator per (D^b, k^p) field with the monomial
  coefficients split by the output derivative (``smc_tala_schur_combine_kernel``).
  Both regroupings of the reference's monomial table
  (stokes/stokes_tala.py:121-140) are restated here in NumPy and checked
  against the oracle, which the reference's fixtures pin.
"""
import os

import numpy as np
import pytest

from oracle import specmc_oracle as O

from conftest import GOLDEN


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def setup():
    from specmc_gb300.config import ConvectionConfig
    g = np.load(os.path.join(GOLDEN, "tala_ops_16x12.npz"))
    cfg = ConvectionConfig(Ra=1e4, Nx=16, Nz=12, viscosity_model="eta_T", compressibility="tala",
                           dissipation_number=0.7, precond="legacy")
    m = O.build(cfg)
    eta = m.eta_of(g["that"])
    return g, m, m.eta_mats(eta)


def test_reference_state_matches_reference(setup):
    from specmc_gb300 import compressibility as C
    from specmc_gb300.solver import basis_arrays
    g, _, _ = setup
    b = basis_arrays(16, 12, 2.0)
    assert C.a_coeff(0.7) == g["tala_a"].item()
    # exp of the host libm: within an ulp of the machine that wrote the fixture
    np.testing.assert_allclose(C.rho_bar_grid(b["z"], 0.7), g["rho_grid"], rtol=4.5e-16, atol=0.0)
    assert _rel(C.rho_bar_coeffs(b["Vi"], b["z"], 0.7), g["rho_c"]) < 1e-15
    assert _rel(C.rho_bar_coeffs(b["Vi"], b["z"], 1.4), g["rho2_c"]) < 1e-15
    # the Boussinesq limit is exact
    assert np.array_equal(C.rho_bar_grid(b["z"], 0.0), np.ones(12))
    assert np.array_equal(C.rho_bar_coeffs(b["Vi"], b["z"], 0.0), np.eye(12)[0])
    r = C.record(0.7)
    assert r["a"] == -0.7 and r["active"] and abs(r["rho_bottom"] - np.exp(0.7)) < 1e-15
    assert abs(r["T0"] - 0.091) < 1e-15 and not C.record(0.0)["active"]
    with pytest.raises(ValueError):
        C.a_coeff(-1.0)


def _words(a, ki, kj):
    """tala_a12_words: the A12 coefficient of W00 = M, W01 = M D, W02 = M D2,
    W10 = D M, W11 = D M D, W20 = D2 M at (ki, kj)."""
    return [((-2.0 * a) * a) * ki * kj + ((2.0 * a) * a) * (kj * kj),
            (-2.0 * a) * (ki * ki) + (4.0 * a) * ki * kj,
            2.0 * (ki * ki),
            (2.0 * a) * ki * kj + (-4.0 * a) * (kj * kj),
            -4.0 * ki * kj,
            2.0 * (kj * kj)]


def test_word_grouped_assembly_equals_reference_operator(setup):
    g, m, Ms = setup
    N, Nk, kx, a, D, D2 = m.Nz, m.Nk, m.kx, m.tala_a, m.D, m.D2
    W = {d: [M, M @ D, M @ D2, D @ M, D @ M @ D, D2 @ M] for d, M in Ms.items()}
    A = np.zeros((Nk * N, Nk * N), complex)
    for i in range(Nk):
        for j in range(Nk):
            ki, kj = kx[i], kx[j]
            T = sum(c * w for c, w in zip(_words(a, ki, kj), W[i - j]))
            A11 = W[i - j][5] + (-2.0 * a) * W[i - j][3] + (a * a - ki * ki) * W[i - j][0]
            if j >= 1 and i + j < Nk:                     # partner half, sign -1, at (ki, -kj)
                Wp = W[i + j]
                T = T - sum(c * w for c, w in zip(_words(a, ki, -kj), Wp))
                A11 = A11 - (Wp[5] + (-2.0 * a) * Wp[3] + (a * a - ki * ki) * Wp[0])
            B = A11 + T @ m.Gt[j]
            B[-2:] = 0.0
            if i == j:
                B[-2], B[-1] = m.V[0], m.V[-1]
            A[i * N:(i + 1) * N, j * N:(j + 1) * N] = B
    assert _rel(A, g["A"]) < 1e-13
    # at a = 0 the words reduce to the Boussinesq C = 2kj^2 D2M + 2ki^2 MD2 - 4 ki kj DMD
    c = _words(0.0, 1.5, 2.5)
    assert c[0] == 0.0 and c[1] == 0.0 and c[3] == 0.0
    assert (c[2], c[4], c[5]) == (2.0 * 1.5 ** 2, -4.0 * 1.5 * 2.5, 2.0 * 2.5 ** 2)


def test_field_grouped_matvec_equals_reference_operator(setup):
    """The six convolutions and the epilogue split by output derivative."""
    g, m, Ms = setup
    N, Nk, a, D, D2 = m.Nz, m.Nk, m.tala_a, m.D, m.D2
    K = m.kx[:, None]
    v = g["v"].reshape(Nk, N)
    gv = np.array([m.Gt[i] @ v[i] for i in range(Nk)])
    fields = [v, K * gv, K ** 2 * gv, (D @ gv.T).T, K * (D @ gv.T).T, (D2 @ gv.T).T]
    flips = [False, True, False, False, True, False]
    t, T01, T02, T10, T11, T20 = [m.mult_eta(Ms, f, flip=fl) for f, fl in zip(fields, flips)]
    P0 = (((-2.0 * a) * a) * (K * T01) + ((2.0 * a) * a) * T02 + (-2.0 * a) * (K ** 2 * T10)
          + (4.0 * a) * (K * T11) + 2.0 * (K ** 2 * T20))
    P1 = (2.0 * a) * (K * T01) + (-4.0 * a) * T02 + (-4.0) * (K * T11)
    P2 = 2.0 * T02
    out = ((D2 @ t.T).T - (2.0 * a) * (D @ t.T).T) + (a * a - K ** 2) * t \
        + (P0 + (D @ P1.T).T + (D2 @ P2.T).T)
    out[:, -2], out[:, -1] = v @ m.V[0], v @ m.V[-1]
    assert _rel(out.ravel(), g["Av"]) < 1e-13
