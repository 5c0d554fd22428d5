"""Vectorised float64 restatement of sph_forces (TEST INFRASTRUCTURE ONLY).

Follows galaxy_formation/sph.py:31-106 formula for formula, but over a chosen set of rows
(particles) at a time, with every other particle's density and smoothing length taken as
given. That is what a partial SPH evaluation of block time steps does: the gas due at a
sub-step gets a new density and new forces, while its neighbours that are not due enter
with their density and smoothing length from their own last evaluation.

    kernel_w / kernel_dw ...... sph.py:31-54 (M4 spline and (1/r) dW/dr), elementwise
    density ................... sph.py:63-71 for the given rows
    forces .................... sph.py:72-106 for the given rows; also returns, per row, the
                                sums of the absolute values of the pair terms of the
                                acceleration and of du/dt, the scales that bound the
                                rounding error of a sum whose terms cancel

Used by the block time-step oracle (force_ref.BlockOracle) and as the error scale of the
float32 SPH checks; nothing in the product imports it.
"""

import numpy as np


def kernel_w(r, h):
    """sph.py:31-40."""
    q = r / h
    s = 1.0 / (np.pi * h ** 3)
    t = 2.0 - q
    return np.where(q < 1.0, s * (1 - 1.5 * q * q + 0.75 * q ** 3),
                    np.where(q < 2.0, s * 0.25 * t ** 3, 0.0))


def kernel_dw(r, h):
    """sph.py:43-54: (1/r) dW/dr."""
    q = r / h
    s = 1.0 / (np.pi * h ** 4)
    t = 2.0 - q
    g = np.where(q < 1.0, s * (-3 * q + 2.25 * q * q), np.where(q < 2.0, -s * 0.75 * t * t, 0.0))
    return g / np.maximum(r, 1e-30)


def density(pos, mass, nb, h, rows):
    """rho of `rows` (sph.py:63-71): nb (n, k) local indices including the particle itself,
    h (n,) smoothing lengths; returns (len(rows),)."""
    rows = np.asarray(rows)
    j = nb[rows]
    d = pos[rows][:, None, :] - pos[j]
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    return np.sum(mass[j] * kernel_w(r, h[rows][:, None]), axis=1)


def forces(pos, vel, mass, nb, h, u, rho, rows, gamma, alpha, beta):
    """Acceleration (len(rows),3), du/dt, Courant step, and the per-row sums of |pair terms|
    of the acceleration and of du/dt (sph.py:72-106), with every particle's rho and h as
    given."""
    rows = np.asarray(rows)
    j = nb[rows]
    hi, rhoi, ui = h[rows][:, None], rho[rows][:, None], u[rows][:, None]
    Pi = (gamma - 1) * rhoi * ui
    ci = np.sqrt(gamma * (gamma - 1) * ui)
    d = pos[rows][:, None, :] - pos[j]
    r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    hj, rhoj, uj, mj = h[j], rho[j], u[j], mass[j]
    gi = kernel_dw(r, hi)
    gj = kernel_dw(r, hj)
    Pj = (gamma - 1) * rhoj * uj
    cj = np.sqrt(gamma * (gamma - 1) * uj)
    vr = np.einsum("ijk,ijk->ij", vel[rows][:, None, :] - vel[j], d)
    hb = 0.5 * (hi + hj)
    mu = np.where(vr < 0, hb * vr / (r * r + 0.01 * hb * hb), 0.0)
    visc = np.where(vr < 0, (-alpha * 0.5 * (ci + cj) * mu + beta * mu * mu) / (0.5 * (rhoi + rhoj)), 0.0)
    gb = 0.5 * (gi + gj)
    f = Pi / rhoi ** 2 * gi + Pj / rhoj ** 2 * gj + visc * gb
    other = j != rows[:, None]                       # sph.py:79: the particle itself is skipped
    w = np.where(other, mj * f, 0.0)
    acc = -np.einsum("ij,ijk->ik", w, d)
    scale = np.sum(np.abs(w) * r, axis=1)
    du_terms = np.where(other, mj * (Pi / rhoi ** 2 * gi + 0.5 * visc * gb) * vr, 0.0)
    dudt = np.sum(du_terms, axis=1)
    mu_max = np.max(np.where(other, -mu, 0.0), axis=1)
    ci = ci[:, 0]
    dt_i = 0.3 * h[rows] / (ci + 1.2 * (alpha * ci + beta * mu_max) + 1e-30)
    return acc, dudt, dt_i, scale, np.sum(np.abs(du_terms), axis=1)


def reselect(pos, cand, rows, k=32):
    """The k nearest of each row's cached candidates (sph.py:109-135 with ties in distance
    broken by candidate slot): returns (nb (len(rows), k), distance of the k-th) or None when a
    row has fewer than k candidates."""
    rows = np.asarray(rows)
    c = cand[rows]
    valid = c >= 0
    if (valid.sum(axis=1) < k).any():
        return None
    cj = np.where(valid, c, 0)
    d = pos[rows][:, None, :] - pos[cj]
    d2 = np.where(valid, np.einsum("ijk,ijk->ij", d, d), np.inf)
    order = np.argsort(d2, axis=1, kind="stable")[:, :k]
    nb = np.take_along_axis(c, order, axis=1)
    dk = np.sqrt(np.take_along_axis(d2, order[:, -1:], axis=1)[:, 0])
    return nb, dk
