"""Per-node kinetic functions of the reference (L1), vectorised over numpy arrays.

Host-side helpers used to build inputs (initial conditions, analytic fields) and to
post-process downloaded populations; the per-step hot path runs in liblbm_gb300.so.

  hermite(n, ξ[, q])              src/hermite_polynomials.jl:1-82
  equilibrium_coefficient(n, ...) src/velocity_distribution_function/hermite.jl:37-77
  equilibrium(q, ρ, u, T)         hermite.jl:10-33 (Hermite expansion to order(q) ÷ 2)
  equilibrium_(q, ρ, u, T)        maxwell_boltzmann_equilibrium.jl:12-66 and the per-set
                                  forms of velocity_distribution_function/quadratures.jl
                                  (`equilibrium!`, the one the collision operators use)
  density, velocity, pressure, temperature, deviatoric_tensor, momentum_flux
                                  velocity_distribution_function/moments.jl

Arrays of populations have the population index FIRST: f[i, ...] (any trailing shape).
"""
from __future__ import annotations

import math

import numpy as np

from .quadratures import D2Q4, D2Q5, D2Q17, D2Q21, D2Q37, Quadrature, order


def _d(a, b):
    return 1.0 if a == b else 0.0


def hermite(n: int, xi, q: Quadrature | None = None):
    """Tensor Hermite polynomial H_n(ξ) as a numpy array of shape (2,)*n.  With a quadrature
    the isotropic terms are scaled by cs = 1 / q.speed_of_sound_squared (hermite_polynomials.jl:47-82)."""
    xi = np.asarray(xi, dtype=np.float64).ravel()
    D = len(xi)
    cs = 1.0 if q is None else 1.0 / q.speed_of_sound_squared
    if n == 0:
        return 1.0
    if n == 1:
        return xi * 1.0
    if n == 2:
        return np.array([[xi[b] * xi[a] - cs * _d(a, b) for b in range(D)] for a in range(D)])
    if n == 3:
        H = np.zeros((D, D, D))
        for a in range(D):
            for b in range(D):
                for c in range(D):
                    H[a, b, c] = xi[c] * xi[b] * xi[a] - cs * (xi[a] * _d(b, c) + xi[b] * _d(a, c) + xi[c] * _d(a, b))
        return H
    if n == 4:
        H = np.zeros((D, D, D, D))
        for a in range(D):
            for b in range(D):
                for c in range(D):
                    for e in range(D):
                        H[a, b, c, e] = (xi[e] * xi[c] * xi[b] * xi[a]
                                         - cs * (xi[a] * xi[b] * _d(c, e) + xi[a] * xi[c] * _d(b, e)
                                                 + xi[a] * xi[e] * _d(b, c) + xi[b] * xi[c] * _d(a, e)
                                                 + xi[b] * xi[e] * _d(a, c) + xi[c] * xi[e] * _d(a, b))
                                         + cs ** 2 * (_d(a, b) * _d(c, e) + _d(a, c) * _d(b, e) + _d(a, e) * _d(b, c)))
        return H
    raise ValueError("hermite polynomials are defined up to order 4")


def equilibrium_coefficient(n: int, q: Quadrature, rho, u, T):
    """a_eq^(n) as an array of shape (2,)*n + shape(ρ) (hermite.jl:37-77, including its
    repeated δ(b,d) / δ(a,d) terms at n = 4)."""
    cs = 1.0 / q.speed_of_sound_squared
    rho = np.asarray(rho, dtype=np.float64)
    u = [np.asarray(u[0], dtype=np.float64), np.asarray(u[1], dtype=np.float64)]
    T = np.asarray(T, dtype=np.float64)
    lam = cs * (T - 1)
    if n == 0:
        return rho
    if n == 1:
        return np.stack([rho * u[0], rho * u[1]])
    if n == 2:
        out = np.empty((2, 2) + rho.shape)
        for a in range(2):
            for b in range(2):
                m = u[a] * u[b]
                if a == b:
                    m = m + lam
                out[a, b] = rho * m
        return out
    if n == 3:
        out = np.empty((2, 2, 2) + rho.shape)
        for a in range(2):
            for b in range(2):
                for c in range(2):
                    out[a, b, c] = rho * (u[a] * u[b] * u[c]
                                          + lam * ((u[a] * _d(b, c) + u[b] * _d(a, c)) + u[c] * _d(a, b)))
        return out
    if n == 4:
        lam2 = (cs * cs) * ((T - 1) * (T - 1))
        out = np.empty((2, 2, 2, 2) + rho.shape)
        for a in range(2):
            for b in range(2):
                for c in range(2):
                    for d in range(2):
                        out[a, b, c, d] = rho * (
                            u[a] * u[b] * u[c] * u[d]
                            + lam * (u[a] * u[b] * _d(c, d) + u[a] * u[c] * _d(b, d) + u[a] * u[d] * _d(b, d)
                                     + u[b] * u[c] * _d(a, d) + u[b] * u[d] * _d(a, d) + u[c] * u[d] * _d(a, b))
                            + lam2 * (_d(a, b) * _d(c, d) + _d(a, c) * _d(b, d) + _d(a, d) * _d(b, c)))
        return out
    raise ValueError("equilibrium coefficients are defined up to order 4")


def _hermite_table(q: Quadrature, n: int):
    return [hermite(n, q.abscissae[:, i], q) for i in range(q.Q)]


def equilibrium(q: Quadrature, rho, u, T=1.0):
    """Hermite-expanded equilibrium to order N = order(q) ÷ 2 (hermite.jl:10-33), the one
    `equilibrium(q, ρ, u, T)` returns and the initial conditions use.  Shape (Q,) + shape(ρ)."""
    rho = np.asarray(rho, dtype=np.float64)
    N = order(q) // 2
    cs = 1.0 / q.speed_of_sound_squared
    aeq = [None] + [equilibrium_coefficient(n, q, rho, u, T) for n in range(1, N + 1)]
    f = np.empty((q.Q,) + rho.shape)
    for i in range(q.Q):
        s = None
        for n in range(1, N + 1):
            H = np.asarray(hermite(n, q.abscissae[:, i], q))
            # dot(a_eq[n], H_n(c_i)): column-major accumulation over the tensor entries
            acc = np.zeros(rho.shape)
            for idx in np.ndindex(*H.shape[::-1]):
                jdx = idx[::-1]
                acc = acc + aeq[n][jdx] * H[jdx]
            term = acc / (math.factorial(n) * cs ** n)
            s = term if s is None else s + term
        f[i] = q.weights[i] * (rho + s)
    return f


def equilibrium_(q: Quadrature, rho, u, T=1.0):
    """`equilibrium!` of the collision operators (maxwell_boltzmann_equilibrium.jl:12-66 and
    the per-set truncations of velocity_distribution_function/quadratures.jl)."""
    rho = np.asarray(rho, dtype=np.float64)
    ux = np.asarray(u[0], dtype=np.float64)
    uy = np.asarray(u[1], dtype=np.float64)
    usq = 0.0 + ux * ux + uy * uy
    cs = q.speed_of_sound_squared
    f = np.empty((q.Q,) + np.broadcast(rho, ux, uy).shape)
    for i in range(q.Q):
        cu = q.abscissae[0, i] * ux + q.abscissae[1, i] * uy
        rw = rho * q.weights[i]
        a1 = cs * cu
        if isinstance(q, (D2Q4, D2Q5)):
            f[i] = rw * (1.0 + a1)
            continue
        a2 = ((cs * cs) * (cu * cu) + 0.0) + (-cs * usq)
        if isinstance(q, (D2Q17, D2Q21, D2Q37)):
            a3 = (cs * cu) * (((cs * cs) * (cu * cu) - (3 * cs) * usq) + 0.0)
            if isinstance(q, D2Q37):
                cs2 = cs * cs
                a4 = ((cs2 * cs2) * (cu * cu * cu * cu) - ((6 * (cs2 * cs)) * usq) * (cu * cu)
                      + (3 * cs2) * (usq * usq))
                f[i] = rw * ((((1.0 + a1) + 0.5 * a2) + (1 / 6) * a3) + (1 / 24) * a4)
            else:
                f[i] = rw * (((1.0 + a1) + 0.5 * a2) + (1 / 6) * a3)
        else:
            f[i] = rw * ((1.0 + a1) + 0.5 * a2)
    return f


def density(q: Quadrature, f):
    """ρ = Σ_i f_i (moments.jl:1-3); f has the population index first."""
    f = np.asarray(f, dtype=np.float64)
    s = f[0].copy()
    for i in range(1, f.shape[0]):
        s = s + f[i]
    return s


def velocity(q: Quadrature, f, rho=None):
    """u = Σ_i f_i c_i / ρ (velocity!, moments.jl:5-19); returns (ux, uy)."""
    f = np.asarray(f, dtype=np.float64)
    if rho is None:
        rho = density(q, f)
    out = []
    for d in range(2):
        s = np.zeros(f.shape[1:])
        for i in range(f.shape[0]):
            s = s + f[i] * q.abscissae[d, i]
        out.append(s / rho)
    return out[0], out[1]


def second_moment(q: Quadrature, f):
    """a_bar_2 = Σ_i f_i H_2(c_i) as a (2, 2, ...) array."""
    f = np.asarray(f, dtype=np.float64)
    a2 = None
    for i in range(f.shape[0]):
        H = hermite(2, q.abscissae[:, i], q)
        term = f[i][None, None] * H.reshape((2, 2) + (1,) * (f.ndim - 1))
        a2 = term if a2 is None else a2 + term
    return a2


def pressure(q: Quadrature, f, rho=None, u=None):
    """p = (tr(a_2) - ρ(|u|² - D)) / D (moments.jl:21-33); 1 for D2Q4 / D2Q5."""
    f = np.asarray(f, dtype=np.float64)
    if isinstance(q, (D2Q4, D2Q5)):
        return np.ones(f.shape[1:])
    if rho is None:
        rho = density(q, f)
    if u is None:
        u = velocity(q, f, rho)
    a2 = second_moment(q, f)
    return ((a2[0, 0] + a2[1, 1]) - rho * ((u[0] ** 2 + u[1] ** 2) - 2)) / 2


def temperature(q: Quadrature, f, rho=None, u=None):
    if rho is None:
        rho = density(q, f)
    return pressure(q, f, rho, u) / rho


def deviatoric_tensor(q: Quadrature, tau, f, rho=None, u=None):
    """σ = s - I tr(s)/D with s = (a_bar_2 - a_eq_2) / (1 + 1/(2τ)) (moments.jl:81-96)."""
    f = np.asarray(f, dtype=np.float64)
    if rho is None:
        rho = density(q, f)
    if u is None:
        u = velocity(q, f, rho)
    a2 = second_moment(q, f)
    aeq = equilibrium_coefficient(2, q, rho, u, 1.0)
    s = (a2 - aeq) / (1 + 1 / (2 * tau))
    tr = (s[0, 0] + s[1, 1]) / 2
    out = s.copy()
    out[0, 0] = s[0, 0] - tr
    out[1, 1] = s[1, 1] - tr
    return out


def momentum_flux(q: Quadrature, f, rho=None, u=None):
    """P = (1/c_s²)·Σ_i f_i (c_i - u)(c_i - u) (moments.jl:35-55)."""
    f = np.asarray(f, dtype=np.float64)
    if rho is None:
        rho = density(q, f)
    if u is None:
        u = velocity(q, f, rho)
    P = np.zeros((2, 2) + f.shape[1:])
    for a in range(2):
        for b in range(2):
            for i in range(f.shape[0]):
                P[a, b] = P[a, b] + f[i] * (q.abscissae[a, i] - u[a]) * (q.abscissae[b, i] - u[b])
    return q.speed_of_sound_squared * P
