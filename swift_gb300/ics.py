"""Seeded synthetic initial conditions for the SPH boxes this library runs.

Every generator returns a dict of NumPy arrays in the layout the C-ABI takes:
``x`` float64 (N, 3) positions in the periodic box, ``v`` float32 (N, 3),
``m``, ``h``, ``u`` float32 (N,), ``time_bin`` int8 (N,), plus ``dim`` (box
size) and the generator's parameters.

The shapes follow the workloads the hot path is measured on:

* ``lattice``    - cubic lattice jittered by a uniform +/- fraction of the
  spacing, Gaussian velocities (the plain 32^3 box, and the uniform boxes of
  the serving stream);
* ``clustered``  - a lattice displaced by a Gaussian random field with a
  power-law spectrum P(k) ~ k^-2, normalised to a given rms displacement in
  units of the spacing (the 128^3 and 384^3 batched boxes);
* ``sedov``      - a jittered lattice with the blast energy deposited as
  internal energy in the particles nearest the centre, as the reference's
  Sedov example does (examples/HydroTests/SedovBlast_3D/makeIC.py), plus a
  synthetic time-bin hierarchy that activates a few per cent per step.

Smoothing lengths start at ``eta * spacing`` (the convention of the reference
test tests/test125cells.c:290); the ghost iterates them to convergence.
"""
from __future__ import annotations

import numpy as np

ETA = 1.2348


def _finish(x, v, u, n, eta, dim=1.0, time_bin=None, **meta):
    N = x.shape[0]
    spacing = dim / n
    out = {
        "x": np.ascontiguousarray(x, dtype=np.float64),
        "v": np.ascontiguousarray(v, dtype=np.float32),
        "m": np.full(N, 1.0 / N, dtype=np.float32),
        "h": np.full(N, eta * spacing, dtype=np.float32),
        "u": np.ascontiguousarray(u, dtype=np.float32),
        "time_bin": (np.zeros(N, dtype=np.int8) if time_bin is None
                     else np.ascontiguousarray(time_bin, dtype=np.int8)),
        "dim": float(dim),
        "eta": float(eta),
    }
    out.update(meta)
    return out


def _wrap(x, dim):
    x = np.mod(x, dim)
    x[x >= dim] = 0.0
    return x


def _grid(n):
    g = (np.arange(n, dtype=np.float64) + 0.5)
    gx, gy, gz = np.meshgrid(g, g, g, indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)


def lattice(n, seed=0, jitter=0.1, sigma_v=0.05, u=1.0, eta=ETA, dim=1.0):
    """n^3 particles on a jittered cubic lattice (uniform +/- jitter*spacing)."""
    rng = np.random.default_rng(seed)
    spacing = dim / n
    x = (_grid(n) + rng.uniform(-jitter, jitter, size=(n ** 3, 3))) * spacing
    v = rng.normal(0.0, sigma_v, size=(n ** 3, 3))
    uu = np.full(n ** 3, u)
    return _finish(_wrap(x, dim), v, uu, n, eta, dim, kind="lattice", seed=seed)


def grf_displacement(n, rms, seed, spectral_index=-2.0):
    """Displacement field (n^3, 3) in units of the spacing.

    A white-noise field is coloured to P(k) ~ k^spectral_index and turned into
    a curl-free displacement psi(k) = i k / k^2 delta(k); the result is scaled
    to the requested rms displacement per particle.
    """
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((n, n, n)).astype(np.float32)
    dk = np.fft.rfftn(noise)
    del noise
    kx = np.fft.fftfreq(n).astype(np.float32)
    kz = np.fft.rfftfreq(n).astype(np.float32)
    k2 = (kx[:, None, None] ** 2 + kx[None, :, None] ** 2
          + kz[None, None, :] ** 2)
    k2[0, 0, 0] = 1.0
    amp = k2 ** (spectral_index / 4.0)          # sqrt(P(k)), P ~ k^index
    dk *= amp
    dk[0, 0, 0] = 0.0
    psi = np.empty((n ** 3, 3), dtype=np.float64)
    kvecs = (kx[:, None, None], kx[None, :, None], kz[None, None, :])
    for a in range(3):
        comp = np.fft.irfftn(1j * kvecs[a] / k2 * dk, s=(n, n, n), axes=(0, 1, 2))
        psi[:, a] = comp.ravel()
        del comp
    cur = np.sqrt(np.mean(np.sum(psi ** 2, axis=1)))
    psi *= rms / max(cur, 1e-30)
    return psi


def clustered(n, seed=0, rms=0.3, u=1.0, sigma_v=0.05, eta=ETA, dim=1.0):
    """Lattice displaced by a P(k) ~ k^-2 Gaussian random field (rms in spacings)."""
    spacing = dim / n
    psi = grf_displacement(n, rms, seed)
    x = (_grid(n) + psi) * spacing
    rng = np.random.default_rng(seed + 7919)
    v = rng.normal(0.0, sigma_v, size=(n ** 3, 3))
    uu = np.full(n ** 3, u)
    return _finish(_wrap(x, dim), v, uu, n, eta, dim, kind="clustered",
                   seed=seed, rms=rms)


def sedov(n, seed=0, energy=1.0, n_hot=33, u_cold=1e-6, eta=ETA, dim=1.0,
          n_bins=8):
    """Jittered lattice with a Sedov blast and a synthetic time-bin hierarchy.

    The blast energy is spread as internal energy over the ``n_hot`` particles
    nearest the box centre.  Time bins are assigned by distance to the centre
    so that the hot core sits in the lowest bin and the cold outskirts in the
    highest: bin ``base + k`` holds the shell whose cumulative fraction reaches
    ``1% * 1.39^k`` (about 1%..10% over the first seven bins), the rest sits in
    the top bin.
    """
    d = lattice(n, seed=seed, sigma_v=0.0, u=u_cold, eta=eta, dim=dim)
    x = d["x"]
    c = np.full(3, 0.5 * dim)
    r = np.linalg.norm(x - c, axis=1)
    order = np.argsort(r, kind="stable")
    N = x.shape[0]
    u = d["u"]
    u[order[:n_hot]] = energy / (n_hot * d["m"][0])
    d["v"][:] = 0.0
    base = 20
    tb = np.full(N, base + n_bins - 1, dtype=np.int8)
    cum = 0
    for k in range(n_bins - 1):
        upto = int(round(N * 0.01 * (1.39 ** k)))
        tb[order[cum:upto]] = base + k
        cum = max(cum, upto)
    d["time_bin"] = tb
    d["kind"] = "sedov"
    d["bin_base"] = base
    return d


def max_active_bin_for_step(step, base=20, n_bins=8):
    """Largest active bin at integer step ``step`` (1-based) of the hierarchy.

    Bin ``base + k`` is active every 2^k steps, as in the reference's
    power-of-two time-line (src/timeline.h:59-130).
    """
    k = 0
    while k + 1 < n_bins and step % (1 << (k + 1)) == 0:
        k += 1
    return base + k


def make(config, seed=0):
    """Named workloads: 'plain32', 'clustered128', 'sedov256', 'large384',
    or '<kind>:<n>' for any lattice/clustered/sedov size."""
    if config == "plain32":
        return lattice(32, seed=seed)
    if config == "clustered128":
        return clustered(128, seed=seed, rms=0.3)
    if config == "sedov256":
        return sedov(256, seed=seed)
    if config == "large384":
        return clustered(384, seed=seed, rms=1.0)
    kind, _, n = config.partition(":")
    n = int(n)
    if kind == "lattice":
        return lattice(n, seed=seed)
    if kind == "clustered":
        return clustered(n, seed=seed)
    if kind == "sedov":
        return sedov(n, seed=seed)
    raise ValueError(f"unknown workload {config!r}")
