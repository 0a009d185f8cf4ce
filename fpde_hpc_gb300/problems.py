"""Seeded synthetic inputs of the benchmark configurations (host side, numpy).

The reference ships no data; its problems are hard-coded analytic tests. These generators
give the line problems of the benchmark their coefficient fields and initial states:
  - lognormal conductivity: white noise N(0,1) on the grid, convolved with a Gaussian of
    correlation length ell (periodic FFT convolution), rescaled to unit variance,
    k = exp(mu + sigma g);
  - initial head: a sum of 8 Gaussians with centres U[0.1,0.9], widths U[0.01,0.1] and
    amplitudes U[0.5,1.0], times a taper that is zero at both ends (Dirichlet 0).
"""
import math
from dataclasses import dataclass

import numpy as np


def lognormal_field(n_nodes, mu, sigma, ell, seed, h):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(n_nodes)
    freqs = np.fft.rfftfreq(n_nodes, d=h)
    kern = np.exp(-0.5 * (2 * np.pi * freqs * ell) ** 2)       # Gaussian filter, length ell
    g = np.fft.irfft(np.fft.rfft(w) * kern, n=n_nodes)
    g = (g - g.mean()) / g.std()
    return np.exp(mu + sigma * g)


def gaussian_mixture(x, seed, n=8):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.1, 0.9, n)
    w = rng.uniform(0.01, 0.1, n)
    a = rng.uniform(0.5, 1.0, n)
    u = np.zeros_like(x)
    for ci, wi, ai in zip(c, w, a):
        u += ai * np.exp(-0.5 * ((x - ci) / wi) ** 2)
    return u * np.sin(np.pi * x)          # zero at x = 0 and x = 1


@dataclass
class LineProblem:
    name: str
    N: int            # intervals (nodes 0..N)
    alpha: float
    tau: float
    steps: int
    k: np.ndarray     # N+1 node conductivities
    u0: np.ndarray    # N+1 initial values
    left: tuple = (0, 0.0)
    right: tuple = (0, 0.0)

    @property
    def x(self):
        return np.arange(self.N + 1) / self.N

    @property
    def dL(self):
        return np.full(self.N + 1, 1.0 / self.N)

    @property
    def Da(self):
        return 1.0 / math.gamma(1.0 - self.alpha)

    def coefs(self):
        """A, B, Rlap of fpde_hpc_1d.cpp A_/B/R with gamma = 1, iw = 1 (numpy restatement of
        fpde_line_coefs; the library function gives identical values)."""
        N, k, dL = self.N, self.k, self.dL
        A, B, R = np.zeros(N + 1), np.zeros(N + 1), np.zeros(N + 1)
        i = np.arange(1, N)
        A[i] = k[i - 1] * 1.0 / (dL[i] * dL[i - 1])
        B[i] = k[i] * 1.0 / (dL[i] * dL[i])
        R[i] = 1.0 * ((k[i] / (dL[i] * dL[i])) + (k[i - 1] / (dL[i] * dL[i - 1])))
        return A, B, R

    @property
    def node_steps(self):
        return (self.N - 1) * self.steps


def config1(steps=1000):
    """1D, N=1000, alpha 0.8, tau 1e-3, k = 1 + 0.5 sin(2 pi x), H0 = exp(-50 (x-0.5)^2), Dirichlet 0."""
    N = 1000
    x = np.arange(N + 1) / N
    u0 = np.exp(-50.0 * (x - 0.5) ** 2)
    u0[0] = u0[-1] = 0.0
    return LineProblem("config1_N1000", N, 0.8, 1e-3, steps, 1.0 + 0.5 * np.sin(2 * np.pi * x), u0)


def config2(N=65536, steps=8192, tau=1e-4):
    """1D, N=65536, 8192 steps, alpha 0.7, lognormal k (mu 0, sigma 0.5, ell 0.01, seed 1),
    8-Gaussian H0 (seed 2), Dirichlet 0; tau = 1e-4 (T = 0.8192)."""
    x = np.arange(N + 1) / N
    k = lognormal_field(N + 1, 0.0, 0.5, 0.01, 1, 1.0 / N)
    u0 = gaussian_mixture(x, 2)
    u0[0] = u0[-1] = 0.0
    return LineProblem(f"config2_N{N}", N, 0.7, tau, steps, k, u0)


@dataclass
class DOProblem:
    """Distributed-order line problem in fr_do's Crank-Nicolson form (eq_solve, fr_do.cpp:733-775)
    with variable conductivity: int_0^1 w(a) D^a u da = d/dx(k du/dx), half the space operator
    implicit and half explicit (theta = 1 on the halved coefficients), Dirichlet 0 ends.
    The a-integral is a quadrature (orders, qw = quadrature weights x w(a)); the library fuses
    it into one lag-weight vector (fpde_do_weights)."""
    name: str
    N: int
    tau: float
    steps: int
    k: np.ndarray
    u0: np.ndarray
    orders: np.ndarray
    qw: np.ndarray

    @property
    def x(self):
        return np.arange(self.N + 1) / self.N

    def coefs(self):
        """Halved A, B, Rlap of the k-Laplacian (implicit half; theta = 1 adds the explicit half)."""
        A, B, R = LineProblem("", self.N, 0.5, self.tau, self.steps, self.k, self.u0).coefs()
        return 0.5 * A, 0.5 * B, 0.5 * R

    @property
    def gnorm(self):
        return np.array([math.gamma(2.0 - a) for a in self.orders])

    @property
    def node_steps(self):
        return (self.N - 1) * self.steps


def gauss_legendre_01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def config3(N=16384, steps=4096, tau=1e-4):
    """DO, N=16384, 4096 steps, w(a) = 6a(1-a), 16-node Gauss-Legendre on [0,1]; lognormal k
    (mu 0, sigma 0.5, ell 0.01, seed 3), 8-Gaussian initial state (seed 4), Dirichlet 0."""
    x = np.arange(N + 1) / N
    k = lognormal_field(N + 1, 0.0, 0.5, 0.01, 3, 1.0 / N)
    u0 = gaussian_mixture(x, 4)
    u0[0] = u0[-1] = 0.0
    a, w = gauss_legendre_01(16)
    return DOProblem(f"config3_DO_N{N}", N, tau, steps, k, u0, a, w * 6.0 * a * (1.0 - a))


def lognormal_field_3d(shape, mu, sigma, ell, seed, h):
    """3D version of lognormal_field on a (nz, ny, nx) grid with uniform spacing h."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    fz = np.fft.fftfreq(shape[0], d=h)[:, None, None]
    fy = np.fft.fftfreq(shape[1], d=h)[None, :, None]
    fx = np.fft.rfftfreq(shape[2], d=h)[None, None, :]
    kern = np.exp(-0.5 * (2 * np.pi * ell) ** 2 * (fz ** 2 + fy ** 2 + fx ** 2))
    g = np.fft.irfftn(np.fft.rfftn(w) * kern, s=shape, axes=(0, 1, 2))
    g = (g - g.mean()) / g.std()
    return np.exp(mu + sigma * g)


@dataclass
class LodProblem:
    """3D LOD problem on (sN+2)(M+2)(K+2) grid points, grids shaped (K+2, M+2, sN+2)."""
    name: str
    dims: tuple         # (sN, M, K) intervals
    alpha: float
    tau: float
    steps: int
    k: np.ndarray       # conductivity at every grid point
    u0: np.ndarray
    left_kind: tuple = (0, 0, 0)
    right_kind: tuple = (0, 0, 0)

    @property
    def h(self):
        return tuple(1.0 / n for n in self.dims)

    @property
    def dLN(self):
        return self.h

    @property
    def Da(self):
        return 1.0 / math.gamma(1.0 - self.alpha)

    def coefs(self):
        """Per-pass A, B, Rlap grids (pass 0 along i, 1 along j, 2 along k) from node-sampled k
        at p and p-1 along the pass axis (A_/B/R of fpde_hpc_1d.cpp with gamma = 1, iw = 1)."""
        shape = self.u0.shape
        cA, cB, cR = (np.zeros((3,) + shape) for _ in range(3))
        for pss, axis in ((0, 2), (1, 1), (2, 0)):
            hh = self.h[pss]
            km = np.roll(self.k, 1, axis=axis)          # k at p-1 (wraps only at p = 0, unused)
            cA[pss] = km / (hh * hh)
            cB[pss] = self.k / (hh * hh)
            cR[pss] = (self.k / (hh * hh)) + (km / (hh * hh))
        return cA, cB, cR

    @property
    def node_steps(self):
        sN, M, K = self.dims
        return (sN - 1) * (M - 1) * (K - 1) * self.steps


def config4(n=128, steps=1024, tau=1e-3):
    """3D n^3 (default 128^3), alpha 0.85, LOD x/y/z, lognormal k (mu 0, sigma 0.4, ell 0.05,
    seed 5), Gaussian blob initial state (centre (0.5, 0.5, 0.6), width 0.1), zero-flux sides
    (i and j passes), Dirichlet 0 top and bottom (k pass)."""
    shape = (n + 2, n + 2, n + 2)
    k = lognormal_field_3d(shape, 0.0, 0.4, 0.05, 5, 1.0 / n)
    z, y, x = np.meshgrid(*(np.arange(n + 2) / n for _ in range(3)), indexing="ij")
    u0 = np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.6) ** 2) / (2 * 0.1 ** 2))
    u0[0] = 0.0
    u0[n:] = 0.0
    return LodProblem(f"config4_{n}^3", (n, n, n), 0.85, tau, steps, k, u0, (1, 1, 0), (1, 1, 0))


def config5(n_cols=512, steps=2048, tau=1e-3, n_min=256, n_max=16384, seed=6):
    """Ensemble of n_cols 1D columns: N log-uniform in [n_min, n_max] (E[N] ~ 3878 for the
    defaults), alpha ~ U[0.5, 0.95] (both drawn with seed 6); column c has a lognormal k
    (mu 0, sigma 0.5, ell 0.01) and an 8-Gaussian initial state, both seeded seed + c;
    Dirichlet 0 ends, tau 1e-3."""
    rng = np.random.default_rng(seed)
    Ns = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_cols))).astype(int)
    alphas = rng.uniform(0.5, 0.95, n_cols)
    cols = []
    for c, (N, a) in enumerate(zip(Ns, alphas)):
        x = np.arange(N + 1) / N
        k = lognormal_field(N + 1, 0.0, 0.5, 0.01, seed + c, 1.0 / N)
        u0 = gaussian_mixture(x, seed + c)
        u0[0] = u0[-1] = 0.0
        cols.append(LineProblem(f"col{c}", int(N), float(a), tau, steps, k, u0))
    return cols


@dataclass
class SfLodProblem(LodProblem):
    """A 3D LOD problem with the implicit space-fractional line solves (the reference's impl 2,
    toeplitz_mult_alg 0) of order gamma: per pass the line coefficients of A_/B/R with the
    space-fractional local weight Dg kb(gamma) = h^(1-gamma) / Gamma(2-gamma) of a uniform axis
    (:3095-3142), Mcoefs of Om1T (:4362-4376, equation 0: k / h^2 stencils), inv_dw_dh
    iw = 1.5 + sin(z / 4) (the analytic problems' form, :2534-2545) and the Toeplitz rows of
    fpde_sf_toeplitz_row; Dirichlet line ends (bc 0), a Gaussian source in the K pass."""
    gamma: float = 0.7
    space_der: int = 0
    tol: float = 1e-9
    max_iter: int = 5000

    def iw(self):
        z = np.arange(self.u0.shape[0])[:, None, None] / self.dims[2]
        return np.broadcast_to(1.5 + np.sin(z / 4.0), self.u0.shape).copy()

    def coefs(self):
        shape = self.u0.shape
        iw = self.iw()
        cA, cB, cR = (np.zeros((3,) + shape) for _ in range(3))
        for pss, axis in ((0, 2), (1, 1), (2, 0)):
            hh = self.h[pss]
            w = hh ** (1.0 - self.gamma) / math.gamma(2.0 - self.gamma)
            km = np.roll(self.k, 1, axis=axis)
            cA[pss] = w * km * iw / (hh * hh)
            cB[pss] = w * self.k * iw / (hh * hh)
            cR[pss] = w * iw * ((self.k / (hh * hh)) + (km / (hh * hh)))
        return cA, cB, cR

    def sf_operands(self):
        """(Tm rows (3, max+2), mc (3 passes, 3, grid), iw (3, grid)) for fpde_lod3d_desc.space_frac."""
        from .api import sf_toeplitz_row
        shape = self.u0.shape
        mc = np.zeros((3, 3) + shape)
        iw = np.stack([self.iw()] * 3)
        Tm = np.zeros((3, max(self.dims) + 2))
        for pss, axis in ((0, 2), (1, 1), (2, 0)):
            hh = self.h[pss]
            km = np.roll(self.k, 1, axis=axis)
            mc[pss, 0] = km / (hh * hh)
            mc[pss, 1] = -((self.k / (hh * hh)) + (km / (hh * hh)))
            mc[pss, 2] = self.k / (hh * hh)
            nl = self.dims[pss]
            Tm[pss, :nl + 1] = sf_toeplitz_row(self.gamma, np.arange(nl + 2) * hh, nl)
        return Tm, mc, iw

    def source(self):
        z, y, x = np.meshgrid(*(np.arange(s) / (s - 2) for s in self.u0.shape), indexing="ij")
        return 5.0 * np.exp(-((x - 0.4) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2) / (2 * 0.15 ** 2))


def sf3d(n=64, steps=32, tau=1e-3, gamma=0.7, space_der=0):
    """The space-fractional LOD workload: n^3, alpha 0.8, lognormal k (mu 0, sigma 0.4, ell 0.05,
    seed 11), Gaussian blob initial state, Dirichlet 0 at every line end, space-fractional order
    gamma (one-sided for space_der 0), the reference's default solver threshold (1e-9) and
    iteration cap (5000)."""
    shape = (n + 2, n + 2, n + 2)
    k = lognormal_field_3d(shape, 0.0, 0.4, 0.05, 11, 1.0 / n)
    z, y, x = np.meshgrid(*(np.arange(n + 2) / n for _ in range(3)), indexing="ij")
    u0 = np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2) / (2 * 0.12 ** 2))
    for a in range(3):
        idx = [slice(None)] * 3
        idx[a] = 0
        u0[tuple(idx)] = 0.0
        idx[a] = slice(n, None)
        u0[tuple(idx)] = 0.0
    return SfLodProblem(f"sf3d_{n}^3", (n, n, n), 0.8, tau, steps, k, u0, (0, 0, 0), (0, 0, 0),
                        gamma=gamma, space_der=space_der)
