"""Seeded synthetic initial conditions of the benchmark problems (host NumPy).

These stand in for the fields the example scripts build
(examples/taylor_green_vortex.py:22-29, examples/kelvin_helmholtz_instability.py:22-54,
examples/rayleigh_benard_convection.py:22-29); every field is drawn from
``numpy.random.default_rng(seed)`` so the GPU path and the CPU baseline get
identical inputs.
"""

import numpy as np


def grid_coords(nx, nz, lx, lz):
    x = np.linspace(0, lx, nx, endpoint=False)
    z = np.linspace(0, lz, nz, endpoint=False)
    return np.meshgrid(x, z, indexing="ij")


def taylor_green(nx, nz, eps=1e-3, seed=0):
    """``w = 2 sin x sin z + eps*(2U-1)`` on [0, 2pi]^2."""
    X, Z = grid_coords(nx, nz, 2 * np.pi, 2 * np.pi)
    rng = np.random.default_rng(seed)
    return 2 * np.sin(X) * np.sin(Z) + eps * (2 * rng.random((nx, nz)) - 1)


def decaying_turbulence(nx, nz, lx=2 * np.pi, lz=2 * np.pi, k0=10.0, seed=0):
    """Vorticity with energy spectrum ``E(k) ~ k^4 exp(-(k/k0)^2)``, uniform
    random phases, scaled so that ``sqrt(<ux^2 + uz^2>) = 1``."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, d=lx / (2 * np.pi * nx))
    kz = np.fft.rfftfreq(nz, d=lz / (2 * np.pi * nz))
    KX, KZ = np.meshgrid(kx, kz, indexing="ij")
    k = np.sqrt(KX ** 2 + KZ ** 2)
    spectrum = k ** 4 * np.exp(-((k / k0) ** 2))
    amp = np.sqrt(np.where(k > 0, k * spectrum / np.pi, 0.0))
    w_hat = amp * np.exp(1j * rng.uniform(0, 2 * np.pi, size=amp.shape))
    w = np.fft.irfft2(w_hat, s=(nx, nz))
    wh = np.fft.rfft2(w)
    psi = wh / np.where(k > 0, k ** 2, 1.0)
    ux = np.fft.irfft2(-1j * KZ * psi, s=(nx, nz))
    uz = np.fft.irfft2(1j * KX * psi, s=(nx, nz))
    return w / np.sqrt(np.mean(ux ** 2 + uz ** 2))


def kelvin_helmholtz(nx, nz, delta, seed=0, eps=1e-3):
    """Double shear layer ``u = tanh((z-pi)/d) - tanh((z-pi/2)/d)`` on
    [0, 2pi]^2: vorticity ``du/dz`` (ux = -dpsi/dz, lap psi = -w) plus
    ``eps * sum_{k=1..4} sin(k x + phi_k)``; passive scalar ``-u/2``."""
    X, Z = grid_coords(nx, nz, 2 * np.pi, 2 * np.pi)
    rng = np.random.default_rng(seed)
    d = delta
    dudz = (1 / np.cosh((Z - np.pi) / d)) ** 2 / d - (1 / np.cosh((Z - np.pi / 2) / d)) ** 2 / d
    u = np.tanh((Z - np.pi) / d) - np.tanh((Z - np.pi / 2) / d)
    phases = rng.uniform(0, 2 * np.pi, size=4)
    pert = sum(np.sin(k * X + phases[k - 1]) for k in range(1, 5))
    return dudz + eps * pert, -0.5 * u


def conductive(nx, nz, lx, lz, eps=1e-3, seed=0):
    """Linear profile ``1 - z + eps*(2U-1)`` on z = linspace(0, lz, nz, endpoint=False)."""
    _, Z = grid_coords(nx, nz, lx, lz)
    rng = np.random.default_rng(seed)
    return 1 - Z + eps * (2 * rng.random((nx, nz)) - 1)
