"""Seeded initial conditions for the workloads (host side, numpy).

The reference generates its own initial conditions (src/initcond.c), but the
workloads run here need different ones, so the generators below write particle
arrays directly in the reference layout (positions, velocities as (N, 3)
float32, masses float32):

* ``uniform_ball``: positions uniform in the unit ball by rejection sampling
  from the counter-based pcg4d hash (src/rng.h:13-40), velocities v = 0.5 r
  (an expanding sphere), equal masses 1/N.
* ``plummer``: a Plummer sphere of scale a, total mass M (G = 1) sampled as
  described by Aarseth, Henon & Wielen (1974, A&A 37, 183): radii from the
  inverted cumulative mass profile, speeds by von Neumann rejection on
  g(q) = q^2 (1 - q^2)^(7/2), isotropic directions.

Both are deterministic functions of (N, seed).
"""
from __future__ import annotations

import numpy as np

_M32 = np.uint64(0xFFFFFFFF)


def pcg4d(a, b, c, d):
    """Vectorised pcg4d (rng.h:13-40) on uint32 arrays; returns four uint32 arrays."""
    a = np.asarray(a, np.uint32).astype(np.uint64)
    b = np.asarray(b, np.uint32).astype(np.uint64)
    c = np.asarray(c, np.uint32).astype(np.uint64)
    d = np.asarray(d, np.uint32).astype(np.uint64)
    mul, inc = np.uint64(1664525), np.uint64(1013904223)
    a = (a * mul + inc) & _M32
    b = (b * mul + inc) & _M32
    c = (c * mul + inc) & _M32
    d = (d * mul + inc) & _M32
    for _ in range(2):
        a = (a + b * d) & _M32
        b = (b + c * a) & _M32
        c = (c + a * b) & _M32
        d = (d + b * c) & _M32
        if _ == 0:
            a ^= a >> np.uint64(16)
            b ^= b >> np.uint64(16)
            c ^= c >> np.uint64(16)
            d ^= d >> np.uint64(16)
    return a.astype(np.uint32), b.astype(np.uint32), c.astype(np.uint32), d.astype(np.uint32)


def _uniforms(seed: int, index, draw: int):
    """Four uniforms in [0, 1) per index, for draw number ``draw``."""
    idx = np.asarray(index, np.uint32)
    s = np.full(idx.shape, seed & 0xFFFFFFFF, np.uint32)
    h = pcg4d(idx, s, np.full(idx.shape, draw, np.uint32), np.full(idx.shape, 0x5F3759DF, np.uint32))
    return [x.astype(np.float64) * (1.0 / 4294967296.0) for x in h]


def uniform_ball(n: int, seed: int = 1, radius: float = 1.0, vel_factor: float = 0.5):
    """(pos, vel, mas): uniform unit ball, v = vel_factor * r, m = 1/N."""
    pos = np.zeros((n, 3), np.float64)
    todo = np.arange(n, dtype=np.uint32)
    draw = 0
    while todo.size:
        u = _uniforms(seed, todo, draw)
        cand = np.stack([2.0 * u[0] - 1.0, 2.0 * u[1] - 1.0, 2.0 * u[2] - 1.0], axis=1)
        ok = np.einsum("ij,ij->i", cand, cand) <= 1.0
        pos[todo[ok]] = cand[ok]
        todo = todo[~ok]
        draw += 1
        if draw > 200:
            raise RuntimeError("rejection sampling did not converge")
    pos = (pos * radius).astype(np.float32)
    vel = (np.float32(vel_factor) * pos).astype(np.float32)
    mas = np.full(n, np.float32(1.0) / np.float32(n), np.float32)
    return pos, vel, mas


def _isotropic(u1, u2):
    z = 1.0 - 2.0 * u1
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * u2
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def plummer(n: int, seed: int = 1, a: float = 1.0, mass: float = 1.0, r_max: float = 10.0,
            G: float = 1.0, center: bool = True):
    """(pos, vel, mas): Plummer sphere (Aarseth, Henon & Wielen 1974)."""
    r = np.zeros(n)
    todo = np.arange(n, dtype=np.uint32)
    draw = 0
    while todo.size:
        u = _uniforms(seed, todo, draw)
        x = np.clip(u[0], 1e-12, 1.0 - 1e-12)
        rr = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
        ok = rr <= r_max * a
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
        draw += 1
    u = _uniforms(seed, np.arange(n, dtype=np.uint32), 1000)
    pos = r[:, None] * _isotropic(u[0], u[1])

    q = np.zeros(n)
    todo = np.arange(n, dtype=np.uint32)
    draw = 2000
    while todo.size:
        u = _uniforms(seed, todo, draw)
        g = u[0] ** 2 * (1.0 - u[0] ** 2) ** 3.5
        ok = 0.1 * u[1] < g
        q[todo[ok]] = u[0][ok]
        todo = todo[~ok]
        draw += 1
    v_esc = np.sqrt(2.0 * G * mass / a) * (1.0 + (r / a) ** 2) ** (-0.25)
    u = _uniforms(seed, np.arange(n, dtype=np.uint32), 3000)
    vel = (q * v_esc)[:, None] * _isotropic(u[0], u[1])
    if center:
        pos -= pos.mean(axis=0)
        vel -= vel.mean(axis=0)
    mas = np.full(n, np.float32(mass) / np.float32(n), np.float32)
    return pos.astype(np.float32), vel.astype(np.float32), mas


def log_uniform_sizes(count: int, lo: int, hi: int, seed: int = 7):
    """System sizes drawn log-uniform in [lo, hi] (the batched ensemble)."""
    u = _uniforms(seed, np.arange(count, dtype=np.uint32), 0)[0]
    return np.floor(np.exp(np.log(lo) + u * (np.log(hi + 1) - np.log(lo)))).astype(np.int64).clip(lo, hi)
