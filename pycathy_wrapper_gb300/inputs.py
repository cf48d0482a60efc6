"""CATHY input model: the content of a CATHY project's input files.

pyCATHY describes a simulation through text files that CATHY reads in
``datin.f``: ``input/parm`` (solver and time-stepping keys, written by
``CATHY.update_parm``, pyCATHY/cathy_tools.py:1515), ``input/soil`` (per
layer and zone soil table, ``CATHY.update_soil`` :2477), ``input/ic``
(``update_ic`` :1755), ``input/atmbc`` (``update_atmbc`` :1907),
``input/dem_parameters`` + ``prepro/dem`` (the DEM and its vertical
discretisation) and the non-atmospheric Dirichlet/Neumann lists
(``update_nansfdirbc`` / ``update_nansfneubc``).  The dataclasses below hold
exactly those contents in memory so that the GPU library can be called
without writing and re-reading files.  Field names follow the reference's
keys.

The module also generates the seeded synthetic workloads used for parity
tests and the benchmark (hillslope, fractal DEM with a lognormal Ks field,
uneven ensemble members, ponded clay loam).
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


@dataclass
class Dem:
    """DEM and vertical discretisation (``prepro/dem``, ``input/dem_parameters``).

    ``dem`` is (nrow, ncol) with row 1 to the north; a cell whose elevation
    is exactly 0 is inactive (triangoli.f:33).  ``zone`` holds 1-based zone
    ids per cell.  ``zratio`` are the layer thickness fractions (NSTR
    values), ``base`` the depth scale and ``ivert`` the GEN3D mode
    (gen3d.f:48-77).
    """

    dem: np.ndarray
    delta_x: float
    delta_y: float
    zratio: np.ndarray
    base: float
    ivert: int = 0
    zone: Optional[np.ndarray] = None
    west: float = 0.0
    south: float = 0.0
    factor: float = 1.0

    @property
    def nrow(self) -> int:
        return int(self.dem.shape[0])

    @property
    def ncol(self) -> int:
        return int(self.dem.shape[1])

    @property
    def nstr(self) -> int:
        return int(len(self.zratio))


@dataclass
class Soil:
    """Soil table (``input/soil``) for IVGHU=0 (van Genuchten).

    Each per-(layer, zone) table has shape (nzone, nstr): ``permx``,
    ``permy``, ``permz`` (saturated conductivity), ``elstor`` (specific
    storage), ``poros`` (porosity), ``vgn`` (VG n), ``vgrmc`` (residual
    moisture content) and ``vgpsat`` (VGPSATCELL = -1/alpha).

    ``feddes`` holds one row per vegetation type of the Feddes root-water
    uptake parameters PCANA, PCREF, PCWLT, ZROOT, PZ, OMGC (datin.f:424-428)
    and ``root_map`` the vegetation type of each DEM cell (``input/root_map``;
    None = type 1 everywhere).  ETRAN (etran.f) removes SCF times the
    potential evaporation through the root zone, so both are needed when
    ``scf`` > 0.
    """

    permx: np.ndarray
    permy: np.ndarray
    permz: np.ndarray
    elstor: np.ndarray
    poros: np.ndarray
    vgn: np.ndarray
    vgrmc: np.ndarray
    vgpsat: np.ndarray
    pmin: float = -5.0
    scf: float = 0.0
    kslope: int = 0
    tolksl: float = 0.01
    feddes: Optional[np.ndarray] = None
    root_map: Optional[np.ndarray] = None

    @property
    def nzone(self) -> int:
        return int(self.permx.shape[0])

    @staticmethod
    def homogeneous(nstr, nzone=1, ks=1e-5, alpha=2.0, n=1.8, theta_s=0.45,
                    theta_r=0.05, ss=1e-5, pmin=-5.0, scf=0.0):
        shp = (nzone, nstr)
        f = lambda v: np.full(shp, float(v))
        return Soil(permx=f(ks), permy=f(ks), permz=f(ks), elstor=f(ss),
                    poros=f(theta_s), vgn=f(n), vgrmc=f(theta_r),
                    vgpsat=f(-1.0 / alpha), pmin=pmin, scf=scf)


@dataclass
class Parm:
    """``input/parm`` keys used by the subsurface solver.

    Defaults are the values of the CATHY project template that pyCATHY
    clones (e.g. examples/SSHydro/weill_exemple/input/parm).
    ``precond`` selects the Picard linear solver: 0 = IC(0)-PCG (the
    reference's SYMSLV), 1 = Jacobi-PCG.  ``isfcvg`` = 1 makes nonlinear
    convergence also wait for the seepage-face exit points (ISFCVG).
    """

    iopt: int = 1
    lump: int = 1
    isolv: int = 0
    itmxcg: int = 500
    ituns: int = 10
    ituns1: int = 5
    ituns2: int = 7
    l2norm: int = 0
    nlrelx: int = 0
    isimgr: int = 1
    tetaf: float = 1.0
    toluns: float = 1e-4
    tolswi: float = 1e30
    ernlmx: float = 1e30
    tolcg: float = 1e-10
    omega: float = 0.8
    deltat: float = 5.0
    dtmin: float = 0.01
    dtmax: float = 100.0
    tmax: float = 7200.0
    dtmaga: float = 0.0
    dtmagm: float = 1.1
    dtreds: float = 0.0
    dtredm: float = 0.5
    pondh_min: float = 0.0
    precond: int = 0
    isfcvg: int = 0
    isfone: int = 0
    dupuit: int = 0
    kslope: int = 0
    tolksl: float = 0.01
    # output control (not used by the solver): IPRT1 = 3 asks for the mesh
    # files only; detailed output (psi, sw) at TIME=0 and at the first step
    # reaching each TIMPRT; the water table at the NODVP columns every step
    iprt1: int = 2
    iprt: int = 4
    timprt: List[float] = field(default_factory=list)
    nodvp: List[int] = field(default_factory=list)


@dataclass
class BC:
    """Boundary and initial conditions.

    Atmospheric forcing (``input/atmbc``): ``atmtim`` (natm times) and
    ``atminp`` rates [L/T], one value per time when ``hspatm`` != 0, else
    (natm, nnod).  ``ieto`` != 0 holds each rate constant until the next
    time (atmnxt.f:47).  ``contp``/``presc`` and ``contq``/``q`` are the
    non-atmospheric Dirichlet and Neumann node lists (1-based) with constant
    values.  ``indp`` selects the initial condition (0 uniform ``pinit[0]``,
    1 nodal ``pinit``, 2 water table at the surface, 3 water table at height
    ``wtposition`` above the bottom of each column, 4 water table at depth
    ``wtposition``).  ``sfnod`` lists the seepage faces (``input/sfbc``),
    one array of 1-based node numbers per face, ordered by descending
    elevation (sfvone.f).
    """

    atmtim: np.ndarray = field(default_factory=lambda: np.array([0.0, 1e30]))
    atminp: np.ndarray = field(default_factory=lambda: np.array([0.0, 0.0]))
    hspatm: int = 1
    ieto: int = 0
    contp: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    presc: np.ndarray = field(default_factory=lambda: np.zeros(0))
    contq: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    q: np.ndarray = field(default_factory=lambda: np.zeros(0))
    indp: int = 4
    wtposition: float = 1.0
    pinit: Optional[np.ndarray] = None
    sfnod: List[np.ndarray] = field(default_factory=list)


@dataclass
class Case:
    dem: Dem
    soil: Soil
    parm: Parm
    bc: BC
    name: str = "case"

    def replace(self, **kw) -> "Case":
        return dataclasses.replace(self, **kw)


# ---------------------------------------------------------------------------
# seeded synthetic workloads
# ---------------------------------------------------------------------------

def hillslope(nrow=20, ncol=20, cell=10.0, slope=0.05, z0=10.0, nstr=10,
              depth=2.0) -> Dem:
    """Planar hillslope DEM: elevation z0 + slope*x at cell centres."""
    xc = (np.arange(ncol) + 0.5) * cell
    dem = np.tile(z0 + slope * xc, (nrow, 1))
    return Dem(dem=dem, delta_x=cell, delta_y=cell,
               zratio=np.full(nstr, 1.0 / nstr), base=depth, ivert=0)


def config0(tmax=86400.0, precond=1) -> Case:
    """20x20 hillslope, 10 layers to 2 m, homogeneous VG soil, rain 1e-7 m/s,
    water table at 1 m depth, Picard + Jacobi-PCG, TOLUNS 1e-6, dt 1..600 s."""
    dem = hillslope()
    soil = Soil.homogeneous(dem.nstr)
    parm = Parm(toluns=1e-6, deltat=1.0, dtmin=1.0, dtmax=600.0, tmax=tmax,
                precond=precond)
    bc = BC(atmtim=np.array([0.0, 1e9]), atminp=np.array([1e-7, 1e-7]),
            indp=4, wtposition=1.0)
    return Case(dem, soil, parm, bc, name="hillslope20x20x10")


def perlin_dem(n, seed, octaves=3, relief=20.0, base_elev=100.0) -> np.ndarray:
    """Seeded gradient-noise (Perlin) DEM on an n x n cell grid."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, n))
    amp, freq, tot = 1.0, 4, 0.0
    for _ in range(octaves):
        g = rng.standard_normal((freq + 1, freq + 1, 2))
        g /= np.linalg.norm(g, axis=2, keepdims=True)
        u = (np.arange(n) + 0.5) / n * freq
        i0 = np.floor(u).astype(int)
        f = u - i0
        X0, Y0 = np.meshgrid(i0, i0, indexing="ij")
        FX, FY = np.meshgrid(f, f, indexing="ij")
        fade = lambda t: t * t * t * (t * (t * 6 - 15) + 10)

        def dot(ix, iy, dx, dy):
            gg = g[ix, iy]
            return gg[..., 0] * dx + gg[..., 1] * dy

        n00 = dot(X0, Y0, FX, FY)
        n10 = dot(X0 + 1, Y0, FX - 1, FY)
        n01 = dot(X0, Y0 + 1, FX, FY - 1)
        n11 = dot(X0 + 1, Y0 + 1, FX - 1, FY - 1)
        sx, sy = fade(FX), fade(FY)
        nx0 = n00 + sx * (n10 - n00)
        nx1 = n01 + sx * (n11 - n01)
        out += amp * (nx0 + sy * (nx1 - nx0))
        tot += amp
        amp *= 0.5
        freq *= 2
    out /= tot
    out = (out - out.min()) / max(out.max() - out.min(), 1e-12)
    return base_elev + relief * out


def lognormal_field(n, seed, mean=-11.5, sigma=1.0, corr=10.0) -> np.ndarray:
    """Seeded Gaussian field with exponential covariance (FFT circulant
    embedding on a doubled grid), exponentiated: ln Ks ~ N(mean, sigma^2)."""
    rng = np.random.default_rng(seed)
    m = 2 * n
    k = np.fft.fftfreq(m) * m
    dx = np.minimum(np.arange(m), m - np.arange(m)).astype(float)
    DX, DY = np.meshgrid(dx, dx, indexing="ij")
    cov = np.exp(-np.sqrt(DX ** 2 + DY ** 2) / corr)
    lam = np.real(np.fft.fft2(cov))
    lam = np.maximum(lam, 0.0)
    w = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    fld = np.real(np.fft.ifft2(np.sqrt(lam) * w)) * m
    fld = fld[:n, :n]
    fld = (fld - fld.mean()) / max(fld.std(), 1e-12)
    del k
    return np.exp(mean + sigma * fld)


def config1(ncell=200, nstr=30, tmax=172800.0, dem_seed=1, ks_seed=2,
            sigma=1.0) -> Case:
    """Fractal DEM (3-octave Perlin, 0-20 m relief), 30 layers to 5 m,
    per-cell lognormal Ks (zone = cell), rain 5e-7 m/s for 6 h then dry."""
    z = perlin_dem(ncell, dem_seed)
    ks = lognormal_field(ncell, ks_seed, sigma=sigma)
    zone = np.arange(1, ncell * ncell + 1, dtype=np.int32).reshape(ncell, ncell)
    dem = Dem(dem=z, delta_x=10.0, delta_y=10.0, zratio=np.full(nstr, 1.0 / nstr),
              base=5.0, ivert=0, zone=zone)
    nz = ncell * ncell
    soil = Soil.homogeneous(nstr, nzone=nz)
    kz = np.repeat(ks.reshape(-1, 1), nstr, axis=1)
    soil.permx, soil.permy, soil.permz = kz.copy(), kz.copy(), kz.copy()
    parm = Parm(toluns=1e-6, deltat=1.0, dtmin=0.1, dtmax=600.0, tmax=tmax)
    bc = BC(atmtim=np.array([0.0, 21600.0, 1e9]),
            atminp=np.array([5e-7, 0.0, 0.0]), ieto=1, indp=4, wtposition=1.0)
    return Case(dem, soil, parm, bc, name=f"fractal{ncell}x{ncell}x{nstr}")


def config2_members(nmembers=256, tmax=86400.0, base_seed=1000,
                    min_cells=30, max_cells=80) -> List[Case]:
    """Uneven ensemble: member m (seed 1000+m) draws a square DEM of 30..80
    cells per side, 10..20 layers, log-uniform Ks and alpha, uniform n and
    theta_s, theta_r = 0.05, water table uniform in 0.5..2 m depth."""
    cases = []
    for m in range(nmembers):
        rng = np.random.default_rng(base_seed + m)
        nc = int(rng.integers(min_cells, max_cells + 1))
        nstr = int(rng.integers(10, 21))
        ks = float(10 ** rng.uniform(-6, -4))
        alpha = float(10 ** rng.uniform(np.log10(0.5), np.log10(5.0)))
        nvg = float(rng.uniform(1.3, 2.5))
        ths = float(rng.uniform(0.35, 0.50))
        wt = float(rng.uniform(0.5, 2.0))
        z = perlin_dem(nc, base_seed + m, relief=5.0)
        dem = Dem(dem=z, delta_x=10.0, delta_y=10.0,
                  zratio=np.full(nstr, 1.0 / nstr), base=3.0, ivert=0)
        soil = Soil.homogeneous(nstr, ks=ks, alpha=alpha, n=nvg, theta_s=ths,
                                theta_r=0.05)
        # DTMIN is the CATHY template's default (0.01 s)
        parm = Parm(toluns=1e-6, deltat=1.0, dtmin=0.01, dtmax=600.0, tmax=tmax)
        bc = BC(atmtim=np.array([0.0, 1e9]), atminp=np.array([1e-7, 1e-7]),
                indp=4, wtposition=wt)
        cases.append(Case(dem, soil, parm, bc, name=f"member{m}"))
    return cases


# Feddes rows (PCANA PCREF PCWLT ZROOT PZ OMGC) of the two vegetation types
# of with_vegetation: shallow grass roots, deeper shrub roots
FEDDES_GRASS_SHRUB = np.array([[0.0, -4.0, -150.0, 0.6, 1.0, 1.0],
                               [-0.5, -3.0, -100.0, 1.2, 2.0, 0.5]])


def with_vegetation(case: Case) -> Case:
    """The same member with the Feddes root-water uptake switched on: SCF =
    1, shrubs on the upper half of the DEM's elevation range and grass on
    the rest, under a day of rain (6 h at 2e-7 m/s) then evaporation (up to
    2e-7 m/s), so that ETRAN takes the evaporation through the roots."""
    d, s = case.dem, case.soil
    soil = dataclasses.replace(s, scf=1.0, feddes=FEDDES_GRASS_SHRUB.copy(),
                               root_map=np.where(d.dem > np.median(d.dem), 2.0, 1.0))
    t = np.array([0.0, 21600.0, 43200.0, 64800.0, 86400.0, 1e9])
    rate = np.array([2e-7, 2e-7, -1e-7, -2e-7, -1e-7, -1e-7])
    bc = dataclasses.replace(case.bc, atmtim=t, atminp=rate)
    return case.replace(soil=soil, bc=bc, name=case.name + "_veg")


def config4_member(ncell=300, nstr=25, seed=0, tmax=43200.0) -> Case:
    """Dry clay loam under a 0.05 m ponded head on the top face (Newton +
    BiCGSTAB): fractal DEM, 25 layers to 10 m, IC -10 m."""
    z = perlin_dem(ncell, 4000 + seed)
    dem = Dem(dem=z, delta_x=10.0, delta_y=10.0, zratio=np.full(nstr, 1.0 / nstr),
              base=10.0, ivert=0)
    soil = Soil.homogeneous(nstr, ks=1e-7, alpha=1.0, n=1.25, theta_s=0.41,
                            theta_r=0.09)
    parm = Parm(iopt=2, isolv=0, toluns=1e-6, deltat=1.0, dtmin=0.1,
                dtmax=600.0, tmax=tmax)
    nnod = (ncell + 1) * (ncell + 1)
    bc = BC(contp=np.arange(1, nnod + 1, dtype=np.int32),
            presc=np.full(nnod, 0.05), indp=0, pinit=np.array([-10.0]))
    return Case(dem, soil, parm, bc, name=f"ponded{ncell}x{ncell}x{nstr}")
