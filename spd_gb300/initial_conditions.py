"""Initial conditions as pointwise callbacks ``f(xyz, case)``.

``xyz`` has shape (ndim, ...) and ``case`` selects the primitive variable:
0 = density, 1..ndim = velocity components, ndim+1 = pressure (the
convention of the reference's src/initial_conditions*.py).  The first
three mirror the reference's own cases; the others are the benchmark
problems (isentropic vortex, four-quadrant Riemann problem, Sedov blast,
Kelvin-Helmholtz shear layer).
"""
from __future__ import annotations

import numpy as np


def sine_wave(xyz, case, A=0.125, vx=1, vy=1, vz=1, P=1):
    """Advected density sine wave, uniform velocity and pressure
    (src/initial_conditions_3d.py:43-56 and its 1D/2D forms)."""
    d = xyz.shape[0]
    x = xyz[0]
    if case == 0:
        return 1.0 + A * np.sin(2 * np.pi * sum(xyz[i] for i in range(d)))
    vel = (vx, vy, vz)
    if 1 <= case <= d:
        return vel[case - 1] * np.ones(x.shape)
    if case == d + 1:
        return P * np.ones(x.shape)
    return np.ones(x.shape)


def step_function(xyz, case, vx=1, vy=1, vz=1, P=1):
    """Density 2 inside the centred box |x-0.5|<0.25 (per axis), else 1
    (src/initial_conditions_3d.py:5-41)."""
    d = xyz.shape[0]
    x = xyz[0]
    if case == 0:
        inside = np.ones(x.shape, dtype=bool)
        for i in range(d):
            inside &= np.fabs(xyz[i] - 0.5) < 0.25
        return np.where(inside, 2, 1)
    vel = (vx, vy, vz)
    if 1 <= case <= d:
        return vel[case - 1] * np.ones(x.shape)
    if case == d + 1:
        return P * np.ones(x.shape)
    return np.ones(x.shape)


def sod(xyz, case):
    """Sod shock tube along x (src/initial_conditions_1d.py:30-40)."""
    x = xyz[0]
    d = xyz.shape[0]
    if case == 0:
        return np.where(x < 0.5, 1.0, 0.125)
    if case == d + 1:
        return np.where(x < 0.5, 1.0, 0.1)
    return np.zeros(x.shape)


def isentropic_vortex(center=(5.0, 5.0), period=(10.0, 10.0), gamma=1.4, beta=5.0, background=(1.0, 1.0)):
    """2D isentropic vortex on a periodic box: rho = T^(1/(gamma-1)),
    P = rho*T, T = 1 - (gamma-1) beta^2/(8 gamma pi^2) exp(1-r^2), velocity
    background + beta/(2 pi) exp((1-r^2)/2) (-(y-yc), x-xc).  ``center`` may
    be moved to get the exact solution at a later time."""
    cx, cy = center
    Lx, Ly = period

    def f(xyz, case):
        x = (xyz[0] - cx + Lx / 2) % Lx - Lx / 2
        y = (xyz[1] - cy + Ly / 2) % Ly - Ly / 2
        r2 = x * x + y * y
        T = 1.0 - (gamma - 1) * beta ** 2 / (8 * gamma * np.pi ** 2) * np.exp(1 - r2)
        rho = T ** (1.0 / (gamma - 1))
        du = beta / (2 * np.pi) * np.exp((1 - r2) / 2)
        if case == 0:
            return rho
        if case == 1:
            return background[0] - du * y
        if case == 2:
            return background[1] + du * x
        if case == 3:
            return rho * T
        return np.ones_like(x)
    return f


def four_quadrant(xyz, case):
    """2D Riemann problem split at x = y = 0.5 (upper right rho=1.5, P=1.5;
    upper left rho=0.5323, u=1.206, P=0.3; lower left rho=0.138,
    u=v=1.206, P=0.029; lower right rho=0.5323, v=1.206, P=0.3)."""
    x, y = xyz[0], xyz[1]

    def q(ur, ul, ll, lr):
        return np.where(x >= 0.5, np.where(y >= 0.5, ur, lr), np.where(y >= 0.5, ul, ll))

    table = [q(1.5, 0.5323, 0.138, 0.5323), q(0.0, 1.206, 1.206, 0.0), q(0.0, 0.0, 1.206, 1.206),
             q(1.5, 0.3, 0.029, 0.3)]
    return table[case] * np.ones(x.shape)


def sedov(N, E=1.0, gamma=1.4, p_ambient=1e-5, rho=1.0):
    """3D Sedov-Taylor blast on [0,1]^3 with N^3 cells: energy E deposited
    as pressure in the 8 cells around the centre."""
    h = 1.0 / N
    p_blast = (gamma - 1) * E / (8 * h ** 3)

    def f(xyz, case):
        x = xyz[0]
        if case == 0:
            return rho * np.ones(x.shape)
        if case == 4:
            inside = np.ones(x.shape, dtype=bool)
            for i in range(3):
                inside &= np.fabs(xyz[i] - 0.5) < h
            return np.where(inside, p_blast, p_ambient)
        return np.zeros(x.shape)
    return f


def kelvin_helmholtz(N, seed=0, amp=0.01, noise=1e-3):
    """Periodic 2D shear layer on [0,1]^2: rho=2, u=0.5 for |y-0.5|<0.25,
    else rho=1, u=-0.5; P=2.5; v = amp sin(4 pi x) + a seeded N(0, noise)
    value per element (indexed by floor(x*N), floor(y*N))."""
    table = np.random.default_rng(seed).normal(0.0, noise, size=(N, N))

    def f(xyz, case):
        x, y = xyz[0], xyz[1]
        inner = np.fabs(y - 0.5) < 0.25
        if case == 0:
            return np.where(inner, 2.0, 1.0)
        if case == 1:
            return np.where(inner, 0.5, -0.5)
        if case == 2:
            ix = np.clip(np.floor(x * N).astype(np.int64), 0, N - 1)
            iy = np.clip(np.floor(y * N).astype(np.int64), 0, N - 1)
            return amp * np.sin(4 * np.pi * x) + table[iy, ix]
        if case == 3:
            return 2.5 * np.ones(x.shape)
        return np.ones(x.shape)
    return f


def gravity_column(g=1.0, amp=1e-2, step=False):
    """Isothermal atmosphere at rest in the gravity potential phi = g * x_last
    (case -1 returns phi, as the reference's init_potential samples it,
    src/sdader_simulator.py:425-434): P = exp(-g x_last) and rho = P (1 +
    amp sin(2 pi x_0)) for ndim > 1 (with ``step``, the sign of the sine: a
    density jump), so hydrostatic balance holds up to the perturbation."""
    def f(xyz, case):
        d = xyz.shape[0]
        z = xyz[d - 1]
        if case == -1:
            return g * z
        base = np.exp(-g * z)
        if case == 0:
            if d == 1:
                return base
            s = np.sin(2 * np.pi * xyz[0])
            return base * (1.0 + amp * (np.sign(s) if step else s))
        if 1 <= case <= d:
            return np.zeros(z.shape)
        return base
    return f
