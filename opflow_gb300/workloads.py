"""Seeded synthetic inputs of the benchmark configurations (numpy only).

These are the inputs `bench.py` measures on and the configuration-size parity tests check, generated
from seeds so that both see the same problems:

- serving stream: 70% one-shot Poisson solves (2D side LogU[129,2049], 3D side LogU[64,256],
  Neumann or Dirichlet 50/50, f ~ N(0,1)) and 30% backward-Euler heat sessions of 10-100 steps
  (side LogU[129,1025], dt = 1/n);
- batched solves: (I - k Lap) u = f on corner-node Dirichlet grids, k ~ LogU[1e-4,1], side ~
  LogU[65,1025] rounded to 2^m + 1, f ~ N(0,1);
- the 3D variable coefficient exp(g), g a smooth seeded Fourier field of standard deviation 1;
- WENO5 initial lines: a square and a sine pulse per line.
"""
import numpy as np


def poisson_problem(api, n, ndim, bc):
    """-Lap(u) = f on n^ndim cells of the unit cube (alpha = 0, beta = 1)."""
    return api.Problem([n] * ndim, [1.0 / n] * ndim, alpha=0.0, beta=1.0, loc=api.LocOnMesh.Center, bc=bc)


def rhs_for(rng, p):
    """f ~ N(0,1) over the problem's unknowns, projected to zero mean where the operator is singular
    (pure Neumann Poisson)."""
    f = rng.standard_normal(int(np.prod(p.n)))
    if p.alpha == 0.0 and p.bc != 1:  # 1 = Dirichlet
        f -= f.mean()
    return f


def serve_mix(api, seed, count):
    """Requests of the serving configuration: a list of (problem, f, steps)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(count):
        u = rng.random()
        if u < 0.7:
            if rng.random() < 0.5:
                n = int(round(np.exp(rng.uniform(np.log(129), np.log(2049)))))
                ndim = 2
            else:
                n = int(round(np.exp(rng.uniform(np.log(64), np.log(256)))))
                ndim = 3
            bc = api.BCType.Neum if rng.random() < 0.5 else api.BCType.Dirc
            p = poisson_problem(api, n, ndim, bc)
            steps = 1
        else:
            n = int(round(np.exp(rng.uniform(np.log(129), np.log(1025)))))
            dt = 1.0 / n
            p = api.Problem([n, n], [1.0 / n] * 2, alpha=1.0, beta=dt, loc=api.LocOnMesh.Center, bc=api.BCType.Dirc)
            steps = int(rng.integers(10, 101))
        reqs.append((p, rhs_for(rng, p), steps))
    return reqs


def batched_problems(api, seed, count):
    """(I - k Lap) u = f on corner-loc Dirichlet grids: a list of (problem, f)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        k = float(np.exp(rng.uniform(np.log(1e-4), np.log(1.0))))
        side = float(np.exp(rng.uniform(np.log(65), np.log(1025))))
        n = (1 << int(round(np.log2(side - 1)))) + 1
        h = 1.0 / (n - 1)
        p = api.Problem([n, n], [h, h], alpha=1.0, beta=k, loc=api.LocOnMesh.Corner, bc=api.BCType.Dirc)
        out.append((p, rng.standard_normal((n - 2) * (n - 2))))
    return out


def smooth_field(rng, n, modes=6):
    """A smooth random field on n^3 cell centres (sum of low-wavenumber Fourier modes), std 1,
    indexed [z, y, x]."""
    x = (np.arange(n) + 0.5) / n
    g = np.zeros((n, n, n))
    for _ in range(modes):
        k = rng.integers(1, 4, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        a = rng.standard_normal()
        g += a * (np.cos(2 * np.pi * k[2] * x + ph[2])[:, None, None] * np.cos(2 * np.pi * k[1] * x + ph[1])[None, :, None]
                  * np.cos(2 * np.pi * k[0] * x + ph[0])[None, None, :])
    return (g - g.mean()) / g.std()


def weno_u0(seed, nx, ny):
    """Per line: a square pulse and a sine pulse with seeded positions, widths and amplitudes."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    c1, w1, a1 = rng.uniform(0.1, 0.4, ny), rng.uniform(0.05, 0.15, ny), rng.uniform(0.5, 1.0, ny)
    c2, w2, a2 = rng.uniform(0.55, 0.85, ny), rng.uniform(0.05, 0.12, ny), rng.uniform(0.3, 0.8, ny)
    u = np.where(np.abs(x[None, :] - c1[:, None]) < w1[:, None], a1[:, None], 0.0)
    d = (x[None, :] - c2[:, None]) / w2[:, None]
    u += np.where(np.abs(d) < 1.0, a2[:, None] * np.cos(0.5 * np.pi * d) ** 2, 0.0)
    return u
