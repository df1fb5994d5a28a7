"""Geometry-block maps for the geometry-dof projection tests (the role of the
reference's GMP block routines hexa(No, eta, x, dxdeta)): x(eta) and its
Jacobian for block coordinates eta in [0, 1]^3, vectorised over points."""
import numpy as np


def shell_map(eta, r0=1.0, r1=1.5, th=(0.1, 0.9), ph=(0.6, 1.4)):
    """A sector of a spherical shell: phi = ph0 + (ph1 - ph0) eta_1 (polar),
    theta = th0 + (th1 - th0) eta_2 (azimuth), r = r0 + (r1 - r0) eta_3 --
    an orientation-preserving map (e_phi, e_theta, e_r right-handed).
    eta: (..., 3).  Returns x (..., 3) and dx/deta (..., 3, 3)."""
    eta = np.asarray(eta, float)
    dr, dt, dp = r1 - r0, th[1] - th[0], ph[1] - ph[0]
    r = r0 + dr * eta[..., 2]
    t = th[0] + dt * eta[..., 1]
    p = ph[0] + dp * eta[..., 0]
    st, ct, sp, cp = np.sin(t), np.cos(t), np.sin(p), np.cos(p)
    x = np.stack([r * sp * ct, r * sp * st, r * cp], axis=-1)
    J = np.zeros(eta.shape[:-1] + (3, 3))
    # d/d eta_1 (phi), d/d eta_2 (theta), d/d eta_3 (r)
    J[..., 0, 1] = -r * sp * st * dt
    J[..., 1, 1] = r * sp * ct * dt
    J[..., 2, 1] = 0.0
    J[..., 0, 0] = r * cp * ct * dp
    J[..., 1, 0] = r * cp * st * dp
    J[..., 2, 0] = -r * sp * dp
    J[..., 0, 2] = sp * ct * dr
    J[..., 1, 2] = sp * st * dr
    J[..., 2, 2] = cp * dr
    return x, J


def shell_volume(r0=1.0, r1=1.5, th=(0.1, 0.9), ph=(0.6, 1.4)):
    return (r1 ** 3 - r0 ** 3) / 3 * (th[1] - th[0]) * (np.cos(ph[0]) - np.cos(ph[1]))


def poly_map(eta):
    """A polynomial block map of per-axis degree <= 2: reproduced exactly by
    geometry dof of order >= 2."""
    e = np.asarray(eta, float)
    x = np.stack([e[..., 0] + 0.1 * e[..., 1] ** 2,
                  e[..., 1] + 0.2 * e[..., 0] * e[..., 2],
                  e[..., 2] + 0.1 * e[..., 0] ** 2 * e[..., 1]], axis=-1)
    J = np.zeros(e.shape[:-1] + (3, 3))
    J[..., 0, 0] = 1.0
    J[..., 0, 1] = 0.2 * e[..., 1]
    J[..., 1, 0] = 0.2 * e[..., 2]
    J[..., 1, 1] = 1.0
    J[..., 1, 2] = 0.2 * e[..., 0]
    J[..., 2, 0] = 0.2 * e[..., 0] * e[..., 1]
    J[..., 2, 1] = 0.1 * e[..., 0] ** 2
    J[..., 2, 2] = 1.0
    return x, J


def eval_geometry(O, xnod, norder, nori_edge, nori_face, xi):
    """x(xi) = sum_k xnod_k phi_k(xi) with the element's oriented functions."""
    shap, _ = O.shape_hexa(xi, norder, nori_edge, nori_face)
    return shap @ xnod


def eta_of(etav, xi):
    """The trilinear block coordinates of reference point xi."""
    etav = np.asarray(etav, float)
    s = [(1 - xi[0], xi[0]), (1 - xi[1], xi[1]), (1 - xi[2], xi[2])]
    off = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    return sum(etav[v] * s[0][o[0]] * s[1][o[1]] * s[2][o[2]] for v, o in enumerate(off))
