"""Inflow-profile parameterisation of the adjoint extension.

The reference builds its inlet data from one analytic profile
(``inletProfile``, common.hpp:240-246): the boundary values u(0, j, k) =
ramp * Um * P(y, z) (main.cu:250-251) and the inlet column's divergence lift
``div_bc_unit`` = -Um P / (beta dx) (immersed_operators.hpp:223-228). The
adjoint differentiates with respect to the profile itself, g[j + ny k] at the
inlet face centres, entering both of those places:

    u(0, j, k) = ramp * g[j, k]          (every BC cleanup of the step)
    div_bc[(0, j, k)] = -g[j, k] / (beta dx)

The implicit-diffusion inlet lift ``rhs_u_bc`` stays the reference's
unit-amplitude base profile: the reference builds it with Um = 1 and no ramp
(immersed_operators.hpp:26, gpu_dense_ops.hpp:16), independent of the inflow,
and the parameterised forward keeps that.

Parameters of the C4 workload: g = Um P + sum_ab c_ab L_a(yh) L_b(zh), with
L_a the Legendre polynomials, yh = 2y/Ly - 1, zh = 2z/Lz - 1 at the inlet face
centres, a, b < 8 (64 coefficients), and nu.
"""
from __future__ import annotations

import numpy as np


class InflowCase:
    """A case whose inlet data follow the profile g (ny*nz, y fastest).

    Every other array is the base case's. With g equal to the base case's
    ``uin`` the arrays are bitwise the base case's own."""

    def __init__(self, case, g):
        self.base = case
        self.params = case.params
        self.counts = case.counts
        nx, ny, nz = case.shape
        g = np.ascontiguousarray(g, dtype=np.float64)
        if g.shape != (ny * nz,):
            raise ValueError(f"inflow profile needs {ny * nz} values")
        self.g = g
        div = np.array(case.array("div_bc_unit"), dtype=np.float64)
        beta = case.array("beta_p").reshape(nz, ny, nx)[:, :, 0].ravel()
        idp = case.array("id_p").reshape(nz, ny, nx)[:, :, 0].ravel()
        fluid = case.array("fluid_p").reshape(nz, ny, nx)[:, :, 0].ravel()
        dx = case.params.Lx / nx
        m = (fluid != 0) & (idp > 0)
        div[idp[m]] = 0.0 - g[m] / (beta[m] * dx)
        self._arrays = {"uin": g, "div_bc_unit": div}

    @property
    def shape(self):
        return self.base.shape

    def array(self, name: str) -> np.ndarray:
        a = self._arrays.get(name)
        return a if a is not None else self.base.array(name)

    def initial_fields(self):
        nx, ny, nz = self.shape
        u, v, w, p = self.base.initial_fields()
        u = u.reshape(nz, ny, nx + 1).copy()
        u[:, :, 0] = self.g.reshape(nz, ny)
        return u.ravel(), v, w, p


def inlet_weights(case) -> np.ndarray:
    """d(div_bc)/dg on the inlet column as 1 / (beta dx) per inlet cell
    (0 on non-fluid cells), y fastest; the library computes the same."""
    nx, ny, nz = case.shape
    beta = case.array("beta_p").reshape(nz, ny, nx)[:, :, 0].ravel()
    fluid = (case.array("fluid_p").reshape(nz, ny, nx)[:, :, 0].ravel() != 0) & \
        (case.array("id_p").reshape(nz, ny, nx)[:, :, 0].ravel() > 0)
    out = np.zeros(ny * nz)
    out[fluid] = 1.0 / (beta[fluid] * (case.params.Lx / nx))
    return out


def legendre(n: int, t: np.ndarray) -> np.ndarray:
    """L_0..L_{n-1} at t (Bonnet's recursion), shape (n, len(t))."""
    t = np.asarray(t, dtype=np.float64)
    out = np.zeros((n, t.size))
    out[0] = 1.0
    if n > 1:
        out[1] = t
    for a in range(1, n - 1):
        out[a + 1] = ((2 * a + 1) * t * out[a] - a * out[a - 1]) / (a + 1)
    return out


def legendre_basis(case, order: int = 8) -> np.ndarray:
    """B[j + ny k, a + order b] = L_a(yh_j) L_b(zh_k) at the inlet face centres."""
    _, ny, nz = case.shape
    cp = case.params
    yh = 2.0 * ((np.arange(ny) + 0.5) * (cp.Ly / ny)) / cp.Ly - 1.0
    zh = 2.0 * ((np.arange(nz) + 0.5) * (cp.Lz / nz)) / cp.Lz - 1.0
    Ly, Lz = legendre(order, yh), legendre(order, zh)
    B = np.einsum("aj,bk->kjba", Ly, Lz).reshape(ny * nz, order * order)
    return B


def inflow_from_coefficients(case, coeffs) -> np.ndarray:
    """g = the case's own profile (Um P) + B c."""
    c = np.asarray(coeffs, dtype=np.float64)
    order = int(round(np.sqrt(c.size)))
    return np.array(case.array("uin"), dtype=np.float64) + legendre_basis(case, order) @ c
