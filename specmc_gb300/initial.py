"""Initial temperature states of the benchmark runs.

The functions of ``specmc/core/bench_ic.py`` and
``specmc/physics/heating.py:168-171``, for any model with the reference's
contract (``x``, ``z``, ``coeffs``, ``seed``): every one returns the (Nk, Nz)
coefficients of the deviation theta = T - (1 - z) from the conductive profile.

* ``conductive_theta(model, amp, m, n)``: the conductive profile with the
  seed amp cos(m pi x) sin(n pi z) (``bench_ic.py:166-168``), i.e.
  ``model.seed``.
* ``heated_conductive_theta(z, H)``: the steady conductive deviation with
  constant internal heating H, theta = H z (1 - z) / 2 (``heating.py:168-171``),
  as a profile on the nodes ``z``.
* ``analytic_bl_theta(model, ...)``: the boundary-layer profile plus a cosine
  perturbation of the case-2a parameter file (``bench_ic.py:148-165``).
* ``aspect_theta(model, path)``: an ASPECT ascii-data temperature field
  (``# POINTS: nx ny`` header, rows ``x y T`` with x fastest, cell-centred
  samples (j + 1/2)/n) mapped onto the model grid as ``bench_ic.py:72-140``
  does: exact cosine interpolation in x (the field is mirror symmetric), an
  interpolant in z through the data and the two isothermal walls.  The
  benchmark's own data file is not shipped; ``find_aspect_ic`` looks for it
  at ``path``, ``$SPECMC_ASPECT_IC`` and beside this package.
"""
from __future__ import annotations

import os

import numpy as np

__all__ = ["ASPECT_IC_NAME", "IC_KINDS", "conductive_theta", "heated_conductive_theta",
           "analytic_bl_field", "analytic_bl_theta", "find_aspect_ic", "read_aspect_ic",
           "aspect_field", "aspect_theta", "ic_theta"]

ASPECT_IC_NAME = "initial_temperature_case2a.txt"
IC_KINDS = ("aspect_file", "analytic_bl", "conductive")
_KIND_ALIASES = {"aspect_file": "aspect_file", "aspect": "aspect_file", "file": "aspect_file",
                 "analytic_bl": "analytic_bl", "analytic": "analytic_bl", "bl": "analytic_bl",
                 "conductive": "conductive", "cond": "conductive", "old": "conductive"}


def conductive_theta(model, amp=1e-3, m=1, n=1):
    """The conductive state with the single-roll seed (model.seed)."""
    return model.seed(amp=amp, m=m, n=n)


def heated_conductive_theta(z, H):
    """theta(z) = H z (1 - z) / 2 of the motionless state with heating H."""
    z = np.asarray(z, dtype=float)
    return (0.5 * float(H)) * z * (1.0 - z)


def analytic_bl_field(model, z1=0.102367, z2=0.897633, amp=0.1, m=1, n=1):
    """theta on the model grid for T = BL(z) + amp cos(m pi x) sin(n pi z):
    BL rises linearly from 0.5 at z1 to 1 at the bottom, is 0.5 between z1 and
    z2 and falls linearly to 0 at the top; theta is zeroed on both walls."""
    x = np.asarray(model.x, dtype=float)[:, None]
    z = np.asarray(model.z, dtype=float)[None, :]
    bottom = 0.5 + 0.5 * (z1 - z) / z1
    top = 0.5 * (1.0 - z) / (1.0 - z2)
    bl = np.where(z < z1, bottom, np.where(z > z2, top, 0.5))
    theta = bl + amp * np.cos(m * np.pi * x) * np.sin(n * np.pi * z) - (1.0 - z)
    theta[:, 0] = 0.0
    theta[:, -1] = 0.0
    return theta


def analytic_bl_theta(model, **kw):
    return model.coeffs(analytic_bl_field(model, **kw))


def find_aspect_ic(path=None):
    """-> the first existing ASPECT data file among ``path``,
    ``$SPECMC_ASPECT_IC`` and this package's directory; FileNotFoundError."""
    here = os.path.dirname(os.path.abspath(__file__))
    tried = [p for p in (path, os.environ.get("SPECMC_ASPECT_IC"),
                         os.path.join(here, ASPECT_IC_NAME)) if p]
    for p in tried:
        if os.path.exists(p):
            return p
    raise FileNotFoundError("no ASPECT initial-temperature file %s among %r" % (ASPECT_IC_NAME, tried))


def read_aspect_ic(path=None):
    """-> (path, x (nx,), y (ny,), T (ny, nx)) of an ASPECT ascii data file.
    ValueError when the rows are not a structured grid with x fastest."""
    path = find_aspect_ic(path)
    shape = None
    rows = []
    with open(path) as f:
        for line in f:
            text = line.strip()
            if not text:
                continue
            if text.startswith("#"):
                if text[1:].strip().upper().startswith("POINTS"):
                    shape = tuple(int(v) for v in text.split(":", 1)[1].split()[:2])
                continue
            rows.append([float(v) for v in text.split()])
    if shape is None:
        raise ValueError("%s has no '# POINTS: nx ny' header" % (path,))
    nx, ny = shape
    data = np.asarray(rows, dtype=float)
    if data.ndim != 2 or data.shape[0] != nx * ny or data.shape[1] < 3:
        raise ValueError("%s: %r values do not form a %d x %d grid of (x, y, T) rows"
                         % (path, data.shape, nx, ny))
    grid = data[:, :3].reshape(ny, nx, 3)
    x, y, T = grid[..., 0], grid[..., 1], grid[..., 2]
    if not np.allclose(x, x[:1, :]) or not np.allclose(y, y[:, :1]):
        raise ValueError("%s: the rows are not ordered with x fastest" % (path,))
    return path, x[0].copy(), y[:, 0].copy(), T.copy()


def aspect_field(model, path=None, zinterp="pchip"):
    """theta of an ASPECT data file on the model's (Nx, Nz) grid.

    In x the n cell-centred samples per row are the exact values of a cosine
    series of n terms (the field is mirror symmetric on the 1 x 1 box); the
    series is evaluated at the model's x nodes, which gives the mirror copy
    on the doubled box.  In z the series coefficients are interpolated
    through the data nodes and the two walls (theta = 0 there; the model's
    CGL nodes lie outside the data's first and last nodes): ``zinterp`` is
    'pchip' (shape preserving) or 'spline' (not-a-knot cubic); 'poly' raises
    ValueError, as the reference's evaluation of it does."""
    path, xs, ys, T = read_aspect_ic(path)
    n = len(xs)
    theta = T - (1.0 - ys)[:, None]                            # (ny, nx)
    xc = (np.arange(n) + 0.5) / n
    cos_basis = np.cos(np.pi * np.outer(xc, np.arange(n)))   # samples <- coefficients
    coef = np.linalg.solve(cos_basis, theta.T)                # (n terms, ny)
    knots = np.concatenate(([0.0], ys, [1.0]))
    values = np.concatenate((np.zeros((n, 1)), coef, np.zeros((n, 1))), axis=1)
    z = np.asarray(model.z, dtype=float)
    if zinterp == "pchip":
        from scipy.interpolate import PchipInterpolator
        at_z = PchipInterpolator(knots, values, axis=1)(z)
    elif zinterp == "spline":
        from scipy.interpolate import CubicSpline
        at_z = CubicSpline(knots, values, axis=1, bc_type="not-a-knot")(z)
    elif zinterp == "poly":
        # one polynomial through all 18 knots oscillates between them (on a
        # 24-node grid it reaches 50x the field's own maximum); the reference's
        # evaluation of this option raises ValueError, and so does this one
        raise ValueError("zinterp='poly' is not usable: the single interpolating polynomial "
                         "oscillates between the knots; use 'pchip' or 'spline'")
    else:
        raise ValueError("zinterp=%r: use 'pchip', 'spline' or 'poly'" % (zinterp,))
    x = np.asarray(model.x, dtype=float)
    g = np.cos(np.pi * np.outer(x, np.arange(n))) @ np.asarray(at_z, dtype=float)
    g[:, 0] = 0.0
    g[:, -1] = 0.0
    return g


def aspect_theta(model, path=None, zinterp="pchip"):
    return model.coeffs(aspect_field(model, path, zinterp))


def ic_theta(model, kind, path=None, amp=1e-3, zinterp="pchip"):
    """The initial state named ``kind`` (an entry or alias of IC_KINDS)."""
    k = _KIND_ALIASES.get(str(kind).strip().lower())
    if k is None:
        raise ValueError("initial condition %r: use one of %s" % (kind, ", ".join(IC_KINDS)))
    if k == "aspect_file":
        return aspect_theta(model, path=path, zinterp=zinterp)
    if k == "analytic_bl":
        return analytic_bl_theta(model)
    return conductive_theta(model, amp=amp)
