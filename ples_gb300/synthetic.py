"""Seeded synthetic grids and right-hand sides for the pressure solve.

No public data set is involved: the workloads are the wavy-wall channel
family described below, generated deterministically from a seed.

Grid (node coordinates, the layout of PLES's ``gri3dp_in.dat``, read in
fsrc/stratiParticle.f03:365-423: i fastest, then j, then k):

* x_i = Lx * i / jx and z_k = Lz * k / jz, periodic in x and z;
* bottom wall y0(x, z) = A * sin(2x) * cos(2z);
* tanh stretching s(eta) = (1 + tanh(beta * (2 eta - 1)) / tanh(beta)) / 2,
  eta = j / jy, and y = y0 + (Ly - y0) * s(eta), which clusters cells at both
  walls and gives non-zero cross metric terms g12, g13 and g23.

Right-hand side: the discrete divergence (fsrc/diver.f03:25-27) of i.i.d.
N(0,1) face fluxes uc(0:jx,1:jy,1:jz), vc(1:jx,0:jy,1:jz), wc(1:jx,1:jy,0:jz),
drawn in that order in Fortran order from ``numpy.random.default_rng(seed)``;
uc and wc are made periodic (uc(0)=uc(jx), wc(0)=wc(jz)), vc vanishes on the
walls, and the mean is removed for compatibility with the Neumann problem.
"""

from __future__ import annotations

import math

import numpy as np

__all__ = [
    "wavy_channel_grid",
    "uniform_grid",
    "divergence_rhs",
    "read_gri3dp",
    "write_gri3dp",
    "Workload",
    "WORKLOADS",
    "BATCH_SIZES",
    "batch_instances",
    "SERVE_SIZES",
    "serve_members",
    "poisson_arrivals",
    "next_rhs",
    "sphere_mask",
]


def wavy_channel_grid(jx, jy, jz, amp, beta, lx=2.0 * math.pi, ly=2.0, lz=math.pi):
    """Node coordinates (jx+1, jy+1, jz+1), float64, Fortran order."""
    i = np.arange(jx + 1, dtype=np.float64)
    j = np.arange(jy + 1, dtype=np.float64)
    k = np.arange(jz + 1, dtype=np.float64)
    xs = lx * i / jx
    zs = lz * k / jz
    eta = j / jy
    if beta > 0.0:
        s = 0.5 * (1.0 + np.tanh(beta * (2.0 * eta - 1.0)) / math.tanh(beta))
    else:
        s = eta.copy()
    s[0], s[-1] = 0.0, 1.0
    X = np.broadcast_to(xs[:, None, None], (jx + 1, jy + 1, jz + 1))
    Z = np.broadcast_to(zs[None, None, :], (jx + 1, jy + 1, jz + 1))
    y0 = amp * np.sin(2.0 * X) * np.cos(2.0 * Z)
    Y = y0 + (ly - y0) * s[None, :, None]
    return (np.asfortranarray(X, dtype=np.float64),
            np.asfortranarray(Y, dtype=np.float64),
            np.asfortranarray(Z, dtype=np.float64))


def uniform_grid(jx, jy, jz, lx, ly, lz):
    """Uniform Cartesian nodes; the PLES sample deck is this with 32^3 cells,
    Lx = 2 pi, Ly = 2, Lz = 2 pi / 3 (gri3dp_in.dat:1-2)."""
    return wavy_channel_grid(jx, jy, jz, 0.0, 0.0, lx=lx, ly=ly, lz=lz)


def divergence_rhs(jx, jy, jz, seed, dt=1.0):
    """Mean-free RHS (jx, jy, jz), float64, Fortran order."""
    rng = np.random.default_rng(seed)
    uc = rng.standard_normal((jx + 1) * jy * jz).reshape((jx + 1, jy, jz), order="F")
    vc = rng.standard_normal(jx * (jy + 1) * jz).reshape((jx, jy + 1, jz), order="F")
    wc = rng.standard_normal(jx * jy * (jz + 1)).reshape((jx, jy, jz + 1), order="F")
    uc[0, :, :] = uc[jx, :, :]
    wc[:, :, 0] = wc[:, :, jz]
    vc[:, 0, :] = 0.0
    vc[:, jy, :] = 0.0
    rhs = (uc[1:, :, :] - uc[:-1, :, :] + vc[:, 1:, :] - vc[:, :-1, :]
           + wc[:, :, 1:] - wc[:, :, :-1]) / dt
    rhs -= rhs.mean()
    return np.asfortranarray(rhs)


def read_gri3dp(path):
    """Read a PLES grid file: lengths, cell counts, then one coordinate per
    line for every node, x, y, z interleaved, i fastest."""
    with open(path) as f:
        lx, ly, lz = (float(v) for v in f.readline().split())
        jx, jy, jz = (int(v) for v in f.readline().split())
        vals = np.array(f.read().split(), dtype=np.float64)
    n = (jx + 1) * (jy + 1) * (jz + 1)
    if vals.size != 3 * n:
        raise ValueError(f"{path}: expected {3 * n} coordinates, found {vals.size}")
    v = vals.reshape(n, 3)
    shape = (jx + 1, jy + 1, jz + 1)
    return ((lx, ly, lz), (jx, jy, jz),
            tuple(np.asfortranarray(v[:, c].reshape(shape, order="F")) for c in range(3)))


def write_gri3dp(path, lengths, x, y, z):
    jx, jy, jz = (s - 1 for s in x.shape)
    with open(path, "w") as f:
        f.write("%18.10E%18.10E%18.10E\n" % tuple(lengths))
        f.write("%12d%12d%12d\n" % (jx, jy, jz))
        xf, yf, zf = (a.ravel(order="F") for a in (x, y, z))
        for q in range(xf.size):
            f.write("%18.10E\n%18.10E\n%18.10E\n" % (xf[q], yf[q], zf[q]))


class Workload:
    """One named grid + RHS case."""

    def __init__(self, name, jx, jy, jz, amp, beta, seed):
        self.name, self.jx, self.jy, self.jz = name, jx, jy, jz
        self.amp, self.beta, self.seed = amp, beta, seed

    @property
    def cells(self):
        return self.jx * self.jy * self.jz

    def grid(self):
        return wavy_channel_grid(self.jx, self.jy, self.jz, self.amp, self.beta)

    def rhs(self, dt=1.0):
        return divergence_rhs(self.jx, self.jy, self.jz, self.seed, dt)


WORKLOADS = {
    "channel_64x32x64": Workload("channel_64x32x64", 64, 32, 64, 0.05, 2.0, 0),
    "channel_256x128x256": Workload("channel_256x128x256", 256, 128, 256, 0.1, 2.5, 1),
    "channel_512x256x512": Workload("channel_512x256x512", 512, 256, 512, 0.1, 3.0, 4),
}

# Many-grid workloads.  Batched solves: 64 independent instances, seeds
# 2..65; each seed draws its grid size uniformly from BATCH_SIZES, then the
# wall amplitude A ~ U(0, 0.15) and the stretch beta ~ U(1.5, 3.0), with
# numpy.random.default_rng(seed); the RHS is divergence_rhs(..., seed).
BATCH_SIZES = ((32, 32, 32), (48, 32, 48), (64, 64, 64), (96, 48, 96), (128, 64, 128))


def batch_instances(seeds=range(2, 66)):
    """Workloads of the batched-solve case, one per seed."""
    out = []
    for seed in seeds:
        rng = np.random.default_rng(seed)
        jx, jy, jz = BATCH_SIZES[int(rng.integers(len(BATCH_SIZES)))]
        amp, beta = float(rng.uniform(0.0, 0.15)), float(rng.uniform(1.5, 3.0))
        out.append(Workload(f"batch_{seed}", jx, jy, jz, amp, beta, seed))
    return out


# Served ensemble: 16 members, member m drawing its fixed grid from
# SERVE_SIZES and A, beta as above with default_rng(1000 + m); its first RHS
# uses seed 1000 + m, every later one is the previous plus 5% N(0,1) noise
# (re-mean-zeroed), and each solve warm-starts from the member's previous
# solution.
SERVE_SIZES = ((48, 48, 48), (96, 48, 96), (128, 64, 128), (192, 96, 192))


def serve_members(n=16):
    out = []
    for m in range(n):
        rng = np.random.default_rng(1000 + m)
        jx, jy, jz = SERVE_SIZES[int(rng.integers(len(SERVE_SIZES)))]
        amp, beta = float(rng.uniform(0.0, 0.15)), float(rng.uniform(1.5, 3.0))
        out.append(Workload(f"member_{m}", jx, jy, jz, amp, beta, 1000 + m))
    return out


def poisson_arrivals(rate, n, seed=7, members=16):
    """n arrival times (s, from 0) of a Poisson process with the given
    aggregate rate, each for a member drawn uniformly."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    return t - t[0], rng.integers(members, size=n)


def next_rhs(rhs, rng, frac=0.05):
    """The next time step's right-hand side of a member."""
    r = rhs + frac * rng.standard_normal(rhs.shape)
    return np.asfortranarray(r - r.mean())


def sphere_mask(x, y, z, n=32, rmin=0.05, rmax=0.2, seed=11, lx=2.0 * math.pi, lz=math.pi):
    """Immersed-boundary mask (jx, jy, jz), True = solid: n spheres with
    centres uniform in the box [0,lx] x [min y, max y] x [0,lz] and radius
    U(rmin, rmax), drawn with default_rng(seed) in the order (cx, cy, cz, r)
    per sphere; a cell is solid when its centroid (mean of its 8 nodes) lies
    inside a sphere, distances periodic in x and z."""
    rng = np.random.default_rng(seed)
    cx = 0.125 * sum(x[a:a + x.shape[0] - 1, b:b + x.shape[1] - 1, c:c + x.shape[2] - 1]
                     for a in (0, 1) for b in (0, 1) for c in (0, 1))
    cy = 0.125 * sum(y[a:a + y.shape[0] - 1, b:b + y.shape[1] - 1, c:c + y.shape[2] - 1]
                     for a in (0, 1) for b in (0, 1) for c in (0, 1))
    cz = 0.125 * sum(z[a:a + z.shape[0] - 1, b:b + z.shape[1] - 1, c:c + z.shape[2] - 1]
                     for a in (0, 1) for b in (0, 1) for c in (0, 1))
    y0, y1 = float(y.min()), float(y.max())
    solid = np.zeros(cx.shape, dtype=bool)
    for _ in range(n):
        sx, sy, sz, r = rng.uniform(0, lx), rng.uniform(y0, y1), rng.uniform(0, lz), rng.uniform(rmin, rmax)
        dx = np.abs(cx - sx)
        dx = np.minimum(dx, lx - dx)
        dz = np.abs(cz - sz)
        dz = np.minimum(dz, lz - dz)
        solid |= dx * dx + (cy - sy) ** 2 + dz * dz < r * r
    return np.asfortranarray(solid)
