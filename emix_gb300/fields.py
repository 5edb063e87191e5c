"""Seeded synthetic inputs for the eMix3d hot path.

The reference ships no input data (its ``data.in``, grid, field and mask
files are absent), so every workload here is generated.  Random numbers come
from a counter-based SplitMix64 hash of ``(seed, field_id, linear index)``,
so any cell of any field can be regenerated independently and the CPU oracle
and the GPU library see bit-identical inputs.

Layout matches the reference: Fortran column-major, ``i`` fastest, linear
index ``i + nx*(j + ny*k)`` (src/Engine/cuArray.cu:123); a multi-component
field is a ``(ncomp, nz, ny, nx)`` C-ordered numpy array, i.e. components
stacked with stride ``nx*ny*nz`` (solver/cuDeriv.cu:588-590).

Grid convention: computational coordinate xi in [0, 1] with spacing
h = 1/(n-1) on wall-bounded axes and xi in [0, 1) with h = 1/n on periodic
axes; physical x = x0 + L*xi.  The metric array ``jbn`` follows
solver/jacob_malla.f90: components 1..9 (0-based 0..8) are d(xi)/d(x),
component 10 is det(dx/dxi) and 11 is its inverse.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_G = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# compact-scheme identifiers shared with the C-ABI (include/emix_gb300.h)
SCHEME_A, SCHEME_B, SCHEME_BPER, SCHEME_C = 0, 1, 2, 3


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser applied elementwise to uint64 counters."""
    with np.errstate(over="ignore"):
        z = (x + _G).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, field_id: int, shape) -> np.ndarray:
    """U[-1, 1) doubles, one hash per cell of ``shape`` (C order)."""
    n = int(np.prod(shape))
    with np.errstate(over="ignore"):
        key = splitmix64(np.array([np.uint64(seed) * np.uint64(1000003) + np.uint64(field_id)],
                                  dtype=np.uint64))[0]
        idx = np.arange(n, dtype=np.uint64) + key
    bits = splitmix64(idx) >> np.uint64(11)
    return (bits.astype(np.float64) * (2.0 ** -52) - 1.0).reshape(shape)


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    length: tuple = (1.0, 1.0, 1.0)
    origin: tuple = (0.0, 0.0, 0.0)
    periodic: tuple = (False, False, False)

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def ncell(self):
        return self.nx * self.ny * self.nz

    def n(self, axis):
        return (self.nx, self.ny, self.nz)[axis]

    def h(self, axis):
        """Computational spacing along ``axis``."""
        n = self.n(axis)
        return 1.0 / n if self.periodic[axis] else 1.0 / (n - 1)

    def coords1d(self, axis):
        n = self.n(axis)
        xi = np.arange(n, dtype=np.float64) * self.h(axis)
        return self.origin[axis] + self.length[axis] * xi

    def coords(self):
        """Physical coordinates x, y, z as (3, nz, ny, nx)."""
        x, y, z = (self.coords1d(a) for a in range(3))
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        return np.stack([X, Y, Z])

    def jbn(self):
        """Metric array of solver/jacob_malla.f90 for this Cartesian grid."""
        j = np.zeros((11,) + self.shape)
        lx, ly, lz = self.length
        j[0] = 1.0 / lx
        j[4] = 1.0 / ly
        j[8] = 1.0 / lz
        det = lx * ly * lz
        j[9] = det
        j[10] = 1.0 / det
        return j


@dataclass
class Impeller:
    """A rotating impeller applied as a volumetric forcing each substep: blade
    b at angle theta0 + omega*t + b*2*pi/nblades is the box r1 <= along <= r2,
    |across| <= half_thick, z1 <= z <= z2; plus a hub disc and a shaft.  Inside
    it the velocity is the rigid rotation (-omega*y, omega*x)."""
    nblades: int = 6
    omega: float = 1.0
    theta0: float = -math.pi / 6.0
    r1: float = 0.165
    r2: float = 0.33
    z1: float = 0.6167
    z2: float = 0.7167
    half_thick: float = 0.012
    hub_r: float = 0.2475
    hub_z1: float = 0.654
    hub_z2: float = 0.679
    shaft_r: float = 0.0264
    shaft_z0: float = 0.6667
    shaft_z1: float = 5.0
    interp: int = 0          # 1: the blade-edge interpolation of the velocity as well


def tank_impeller(grid: "Grid", radius=1.0, height=2.0, omega=1.0, nblades=6, z_frac=1.0 / 3.0,
                  blade_r=0.33, blade_h=0.05) -> Impeller:
    """Impeller of the tank workload in the proportions of the reference's
    rushton(sub_step) (rush_ruth_me.f90:52-95: blades from R2/2 to R2, hub
    disc of 0.75 R2, blade half-thickness 1.5 dmin, shaft of 0.08 R2 from the
    disc upward, initial angle -pi/6), with blade radius blade_r*R and blade
    height blade_h*H at z = z_frac*H."""
    dmin = min(grid.length[a] * grid.h(a) for a in range(3))
    r2 = blade_r * radius
    zc = z_frac * height
    th = 1.5 * dmin
    return Impeller(nblades=nblades, omega=omega, theta0=-math.pi / 6.0, r1=0.5 * r2, r2=r2,
                    z1=zc - 0.5 * blade_h * height, z2=zc + 0.5 * blade_h * height, half_thick=th,
                    hub_r=0.75 * r2, hub_z1=zc - th, hub_z2=zc + th, shaft_r=0.08 * r2,
                    shaft_z0=zc, shaft_z1=2.5 * height)


@dataclass
class Workload:
    grid: Grid
    schemes: tuple
    um: np.ndarray          # (5, nz, ny, nx): p*Mach^2, rho*u, rho*v, rho*w, T
    phi: np.ndarray         # (nz, ny, nx) level set
    jbn: np.ndarray         # (11, nz, ny, nx)
    mask: np.ndarray        # (nz, ny, nx)
    mach: float = 0.1
    reynolds: float = 1000.0
    cs: float = 0.1
    amu0: float = 0.1781
    sgs_model: int = 1
    dt: float = 0.0
    name: str = ""
    extra: dict = field(default_factory=dict)
    impeller: Impeller | None = None   # rotating impeller forcing (None: static mask only)
    t0: float = 0.0                    # time at the start of the first step


def cfl_dt(grid: Grid, u: np.ndarray, mach: float, cfl: float) -> float:
    """Time step from the CFL rule of TSTEP (src/MSVSingle/tstep_incomp.f90:99-153)
    for a first step: dt = cfl / max_d (|u_d| + sqrt(cs^2 + u_d^2)) / dx_d with
    cs = sqrt(1/Mach) (src/MSVSingle/source_incomp.f90:11)."""
    cs = math.sqrt(1.0 / mach)
    cfla = 0.0
    for a in range(3):
        dx = grid.length[a] * grid.h(a)
        ua = np.abs(u[a])
        cfla = max(cfla, float(np.max((ua + np.sqrt(cs * cs + ua * ua)) / dx)))
    return cfl / cfla


def _conserved(p_fluct, u, temp, mach):
    """um(1) = p*Mach^2 with p = 1/Mach^2 + p', um(2..4) = u*um(1), um(5) = T
    (src/MSVSingle/herramientas_incomp2.f90:44-52)."""
    r = 1.0 + mach * mach * p_fluct
    um = np.empty((5,) + r.shape)
    um[0] = r
    um[1] = u[0] * r
    um[2] = u[1] * r
    um[3] = u[2] * r
    um[4] = temp
    return um


def taylor_green(n=64, seed=1, noise=1e-3, scheme=SCHEME_BPER, mach=0.1, cfl=0.3,
                 reynolds=1000.0) -> Workload:
    """Periodic Taylor-Green box of side 2*pi with seeded noise and a sphere
    level set of radius L/4 (the 64^3 periodic configuration)."""
    L = 2.0 * math.pi
    g = Grid(n, n, n, (L, L, L), (0.0, 0.0, 0.0), (True, True, True))
    X, Y, Z = g.coords()
    u = np.stack([
        np.sin(X) * np.cos(Y) * np.cos(Z) + noise * uniform(seed, 1, g.shape),
        -np.cos(X) * np.sin(Y) * np.cos(Z) + noise * uniform(seed, 2, g.shape),
        noise * uniform(seed, 3, g.shape),
    ])
    p = (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    temp = 1.0 + 0.1 * np.sin(X) * np.sin(Y) * np.sin(Z)
    um = _conserved(p, u, temp, mach)
    c = L / 2.0
    phi = np.sqrt((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2) - 0.25 * L
    w = Workload(g, (scheme,) * 3, um, phi, g.jbn(), np.ones(g.shape), mach=mach,
                 reynolds=reynolds, name=f"taylor_green_{n}")
    w.dt = cfl_dt(g, u, mach, cfl)
    return w


def rushton_mask(grid: Grid, radius=1.0, height=2.0, nblades=6, z_frac=1.0 / 3.0,
                 blade_r=0.33, blade_h=0.05, blade_w=0.02, theta0=0.0) -> np.ndarray:
    """Static impeller mask: 0 inside the blades and hub disc, 1 elsewhere.
    Blades are radial plates reaching ``blade_r*R`` at ``z = z_frac*H``."""
    X, Y, Z = grid.coords()
    r = np.sqrt(X * X + Y * Y)
    th = np.arctan2(Y, X)
    zc = z_frac * height
    inz = np.abs(Z - zc) <= 0.5 * blade_h * height
    mask = np.ones(grid.shape)
    for b in range(nblades):
        a = theta0 + 2.0 * math.pi * b / nblades
        # distance from the blade's radial line
        d = np.abs(-np.sin(a) * X + np.cos(a) * Y)
        along = np.cos(a) * X + np.sin(a) * Y
        blade = inz & (d <= blade_w * radius) & (along >= 0.5 * blade_r * radius) & \
            (along <= blade_r * radius)
        mask[blade] = 0.0
    disc = (np.abs(Z - zc) <= 0.25 * blade_w * height) & (r <= 0.75 * blade_r * radius)
    mask[disc] = 0.0
    del th
    return mask


def stirred_tank(n=256, seed=2, nmodes=64, kmax=8, omega=1.0, radius=1.0, height=2.0,
                 scheme=SCHEME_B, mach=0.1, cfl=0.3, reynolds=1000.0, nz=None,
                 impeller=False, impeller_omega=None) -> Workload:
    """Wall-bounded tank [-R,R]^2 x [0,H]: solid-body rotation about z plus
    ``nmodes`` seeded Fourier modes with |k| <= kmax and Gaussian amplitudes
    rescaled to an RMS of 0.1*omega*R, a flat free surface at z = 0.8H and a
    6-blade impeller at z = H/3: a static mask, or with ``impeller`` a
    rotating impeller forcing (angular velocity ``impeller_omega``, default
    ``omega``) and no static mask."""
    nz = n if nz is None else nz
    g = Grid(n, n, nz, (2 * radius, 2 * radius, height), (-radius, -radius, 0.0),
             (False, False, False))
    X, Y, Z = g.coords()
    rng_k = uniform(seed, 10, (nmodes, 3))
    rng_a = uniform(seed, 11, (nmodes, 6))
    u = np.stack([-omega * Y, omega * X, np.zeros_like(X)])
    # mode m: amp_c * sin(kx*pi*x/R + ky*pi*y/R + kz*pi*z/H + 2*pi*u2_0), summed as
    # Im(sum_m [amp_c e^{i p} E_z E_y](z,y) [E_x](x)): one complex GEMM per component
    ks = np.zeros((nmodes, 3))
    amps = np.zeros((nmodes, 3))
    phase = np.zeros(nmodes)
    for m in range(nmodes):
        k = np.round(rng_k[m] * kmax)
        while np.sqrt(np.sum(k * k)) > kmax:
            k = np.trunc(k * 0.75)
        # Box-Muller from two uniforms per component -> Gaussian amplitude
        u1 = 0.5 * (rng_a[m, :3] + 1.0) + 1e-12
        u2 = 0.5 * (rng_a[m, 3:] + 1.0)
        ks[m] = k
        amps[m] = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
        phase[m] = 2.0 * math.pi * u2[0]
    x1, y1, z1 = (g.coords1d(a) for a in range(3))
    Ex = np.exp(1j * np.outer(ks[:, 0] * math.pi / radius, x1))          # (m, nx)
    Ey = np.exp(1j * np.outer(ks[:, 1] * math.pi / radius, y1))          # (m, ny)
    Ez = np.exp(1j * np.outer(ks[:, 2] * math.pi / height, z1))          # (m, nz)
    base = (Ez[:, :, None] * Ey[:, None, :]) * np.exp(1j * phase)[:, None, None]  # (m, nz, ny)
    base = base.reshape(nmodes, -1).T                                     # (nz*ny, m)
    pert = np.empty_like(u)
    for c in range(3):
        pert[c] = ((base * amps[:, c]) @ Ex).imag.reshape(g.shape)
    rms = math.sqrt(float(np.mean(np.sum(pert * pert, axis=0))))
    if rms > 0:
        pert *= 0.1 * omega * radius / rms
    u = u + pert
    p = 0.5 * omega * omega * (X * X + Y * Y)
    temp = np.ones(g.shape)
    um = _conserved(p, u, temp, mach)
    phi = Z - 0.8 * height
    mask = np.ones(g.shape) if impeller else rushton_mask(g, radius, height)
    w = Workload(g, (scheme,) * 3, um, phi, g.jbn(), mask, mach=mach, reynolds=reynolds,
                 name=f"stirred_tank_{n}x{n}x{nz}")
    if impeller:
        w.impeller = tank_impeller(g, radius, height,
                                   omega if impeller_omega is None else impeller_omega)
    w.dt = cfl_dt(g, u, mach, cfl)
    return w


def random_box(nx, ny, nz, seed=5, periodic=False, scheme=None, mach=0.1) -> Workload:
    """Smooth-plus-noise fields on a small box, for parity tests."""
    per = (periodic,) * 3
    g = Grid(nx, ny, nz, (1.3, 0.9, 1.1), (0.1, -0.2, 0.3), per)
    X, Y, Z = g.coords()
    u = np.stack([
        np.sin(3 * X) * np.cos(2 * Y) + 0.05 * uniform(seed, 1, g.shape),
        np.cos(2 * X + Z) + 0.05 * uniform(seed, 2, g.shape),
        np.sin(X + 2 * Y) * np.cos(Z) + 0.05 * uniform(seed, 3, g.shape),
    ])
    p = np.cos(X) * np.sin(Y + Z) + 0.1 * uniform(seed, 4, g.shape)
    temp = 1.0 + 0.1 * uniform(seed, 5, g.shape)
    um = _conserved(p, u, temp, mach)
    phi = np.sqrt((X - 0.7) ** 2 + (Y - 0.2) ** 2 + (Z - 0.8) ** 2) - 0.3
    if scheme is None:
        scheme = SCHEME_BPER if periodic else SCHEME_B
    w = Workload(g, (scheme,) * 3, um, phi, g.jbn(), np.ones(g.shape), mach=mach,
                 name=f"random_box_{nx}x{ny}x{nz}")
    w.dt = cfl_dt(g, u, mach, 0.3)
    return w


ENSEMBLE_SIZES = tuple(range(32, 161, 16))   # {32, 48, ..., 160}


def ensemble_shapes(ngrids=48, seed=7, sizes=ENSEMBLE_SIZES) -> list:
    """(nx, ny, nz) of every grid of ensemble(ngrids, seed, sizes=sizes)."""
    draws = uniform(seed, 100, (ngrids, 4))
    out = []
    for g in range(ngrids):
        idx = np.minimum(((draws[g, :3] + 1.0) * 0.5 * len(sizes)).astype(int), len(sizes) - 1)
        out.append(tuple(int(sizes[i]) for i in idx))
    return out


def ensemble(ngrids=48, seed=7, cfl=0.3, mach=0.1, scheme=SCHEME_BPER, sizes=ENSEMBLE_SIZES,
             noise=1e-3, only=None) -> list:
    """Uneven ensemble: grid g has nx, ny, nz drawn independently from
    ``sizes`` and its own rotation rate omega_g ~ U[0.5, 2.0] (seeded), with
    the periodic Taylor-Green fields of the 64^3 configuration scaled by
    omega_g.  ``only``: build just these grid indices (same grids as in the
    full ensemble)."""
    draws = uniform(seed, 100, (ngrids, 4))
    out = []
    L = 2.0 * math.pi
    for g in range(ngrids):
        if only is not None and g not in only:
            continue
        idx = np.minimum(((draws[g, :3] + 1.0) * 0.5 * len(sizes)).astype(int), len(sizes) - 1)
        nx, ny, nz = (sizes[i] for i in idx)
        omega = 0.5 + 1.5 * 0.5 * (draws[g, 3] + 1.0)
        grid = Grid(int(nx), int(ny), int(nz), (L, L, L), (0.0, 0.0, 0.0), (True, True, True))
        X, Y, Z = grid.coords()
        u = omega * np.stack([
            np.sin(X) * np.cos(Y) * np.cos(Z) + noise * uniform(seed + g, 1, grid.shape),
            -np.cos(X) * np.sin(Y) * np.cos(Z) + noise * uniform(seed + g, 2, grid.shape),
            noise * uniform(seed + g, 3, grid.shape),
        ])
        p = omega * omega * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
        temp = 1.0 + 0.1 * np.sin(X) * np.sin(Y) * np.sin(Z)
        um = _conserved(p, u, temp, mach)
        c = L / 2.0
        phi = np.sqrt((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2) - 0.25 * L
        w = Workload(grid, (scheme,) * 3, um, phi, grid.jbn(), np.ones(grid.shape), mach=mach,
                     name=f"ensemble_{g}_{nx}x{ny}x{nz}", extra={"omega": omega})
        w.dt = cfl_dt(grid, u, mach, cfl)
        out.append(w)
    return out


def sgs_geometry(grid: Grid):
    """Coordinates (3, nz, ny, nx) used by INISGDM (solver/sgdm_incomp.f90:2-114)."""
    return grid.coords()
