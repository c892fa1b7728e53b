"""Seeded initial conditions for the benchmark configurations, and the CLI's
softening and time-step rules.

The reference's own generators (galax-init/src/lib.rs) are unseeded and differ
from the benchmark presets; these follow the benchmark definitions:

* ``uniform``: positions U[0,100]^2, masses U[0.5,1.5], v = 0; tree box [0,100]^2.
* ``plummer``: total mass 1, a = 1, r = a/sqrt(u^(-2/3) - 1) truncated at r <= 10a
  (rejection, the rule of galax-init/src/lib.rs:19-24), uniform polar angle; speeds
  q*sqrt(2)*(1+r^2)^(-1/4) with q drawn by rejection from q^2 (1-q^2)^(7/2), random
  direction in the plane; equal masses 1/N; tree box [-50,50]^2 (the CLI box).
* ``disk``: surface density exp(-R/10) truncated at R = 60, uniform azimuth, equal
  masses summing to 1, circular speed from the enclosed mass plus 5% Gaussian
  velocity dispersion; tree box [-60,60]^2.
* ``galaxy``: one body of mass 1000 at the origin plus N-1 test particles of mass
  1e-6 with R ~ U[1,50] (surface density 1/R) on circular orbits v = sqrt(1000/R);
  tree box [-50,50]^2.
"""
from __future__ import annotations

import numpy as np

from . import Bodies

BOUNDS = {
    "uniform": (0.0, 100.0, 0.0, 100.0),
    "plummer": (-50.0, 50.0, -50.0, 50.0),
    "disk": (-60.0, 60.0, -60.0, 60.0),
    "galaxy": (-50.0, 50.0, -50.0, 50.0),
}


def uniform(n: int, seed: int = 0) -> Bodies:
    rng = np.random.default_rng(seed)
    return Bodies.from_arrays(rng.uniform(0.0, 100.0, n), rng.uniform(0.0, 100.0, n), rng.uniform(0.5, 1.5, n))


def plummer(n: int, seed: int = 0) -> Bodies:
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while r.size < n:
        u = rng.uniform(0.0, 1.0, 2 * (n - r.size) + 16)
        u = u[u > 0.0]
        rr = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= 10.0]])
    r = r[:n]
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    q = np.empty(0)
    while q.size < n:  # rejection from g(q) = q^2 (1-q^2)^(7/2); max g < 0.1
        qq = rng.uniform(0.0, 1.0, 4 * (n - q.size) + 16)
        g = rng.uniform(0.0, 0.1, qq.size)
        q = np.concatenate([q, qq[g < qq ** 2 * (1.0 - qq ** 2) ** 3.5]])
    q = q[:n]
    speed = q * np.sqrt(2.0) * (1.0 + r * r) ** (-0.25)
    psi = rng.uniform(0.0, 2.0 * np.pi, n)
    return Bodies.from_arrays(r * np.cos(phi), r * np.sin(phi), np.full(n, 1.0 / n), speed * np.cos(psi),
                              speed * np.sin(psi))


def disk(n: int, seed: int = 0, rd: float = 10.0, rmax: float = 60.0) -> Bodies:
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while r.size < n:  # radial pdf R exp(-R/Rd) is Gamma(2, Rd); truncate at rmax
        rr = rng.gamma(2.0, rd, 2 * (n - r.size) + 16)
        r = np.concatenate([r, rr[rr <= rmax]])
    r = r[:n]
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    enc = lambda R: 1.0 - (1.0 + R / rd) * np.exp(-R / rd)
    menc = enc(r) / enc(rmax)
    vc = np.sqrt(menc / np.maximum(r, 1e-12))
    vx = -vc * np.sin(phi) + 0.05 * vc * rng.standard_normal(n)
    vy = vc * np.cos(phi) + 0.05 * vc * rng.standard_normal(n)
    return Bodies.from_arrays(r * np.cos(phi), r * np.sin(phi), np.full(n, 1.0 / n), vx, vy)


def galaxy(n: int, seed: int = 0) -> Bodies:
    rng = np.random.default_rng(seed)
    m = n - 1
    r = rng.uniform(1.0, 50.0, m)
    phi = rng.uniform(0.0, 2.0 * np.pi, m)
    v = np.sqrt(1000.0 / r)
    x = np.concatenate([[0.0], r * np.cos(phi)])
    y = np.concatenate([[0.0], r * np.sin(phi)])
    vx = np.concatenate([[0.0], -v * np.sin(phi)])
    vy = np.concatenate([[0.0], v * np.cos(phi)])
    mass = np.concatenate([[1000.0], np.full(m, 1e-6)])
    return Bodies.from_arrays(x, y, mass, vx, vy)


PRESETS = {"uniform": uniform, "plummer": plummer, "disk": disk, "galaxy": galaxy}


def make(name: str, n: int, seed: int = 0) -> Bodies:
    return PRESETS[name](n, seed)


def cli_softening(x: np.ndarray, y: np.ndarray) -> float:
    """0.1 x mean |b_i - b_(i+1) mod n| over i < min(n, 1000), on Morton-sorted
    bodies (galax-cli/src/main.rs:182-190)."""
    n = x.size
    if n == 0:
        return 0.0
    k = min(n, 1000)
    s = 0.0
    for i in range(k):
        dx = float(x[i]) - float(x[(i + 1) % n])
        dy = float(y[i]) - float(y[(i + 1) % n])
        s += (dx * dx + dy * dy) ** 0.5
    return s / k * 0.1


def cli_dt(ax: np.ndarray, ay: np.ndarray) -> float:
    """dt = 0.5/sqrt(max |a|) if max |a| > 1e-30 else 0.01 (galax-cli/src/main.rs:232-244)."""
    if ax.size == 0:
        return 0.01
    a = np.sqrt(ax * ax + ay * ay)
    amax = float(np.nanmax(np.concatenate([a, [0.0]])))
    return 0.5 / amax ** 0.5 if amax > 1e-30 else 0.01
