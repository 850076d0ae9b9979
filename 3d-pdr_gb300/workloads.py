"""Seeded synthetic per-cell inputs for the five benchmark configurations.

The reference ships no timing workload (no public dataset exists for this
path); these generators restate the configurations' parameter distributions
with numpy Generator(PCG64(seed)), drawn in a fixed order so every run with the
same seed sees the same cells.  Grid shapes (4^3, 32^3, 64^3) only name the
cells: each cell is solved independently.

Unspecified inputs are seeded and stated here:
  * N(C) per ray ~ logU(1e10, 1e18); N(S) per ray ~ logU(1e10, 1e18) for
    networks that contain S; N(HD) = 0;
  * isotropic field: rad_surface_k = G0/12 for each of the 12 HEALPix level-0
    rays (3DPDR.F90:1674);
  * physics constants from params.dat: omega 0.42, grain radius 1e-7,
    gas-to-dust 100, metallicity 1, v_turb 1 km/s, H2FORM on.
"""
import numpy as np

NRAYS = 12
YEAR = 3.1556926e7


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


class ChemInputs:
    """Per-cell physical inputs of one chemistry workload (SoA, float64)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    @property
    def ncell(self):
        return self.n_H.shape[0]


def initial_abundances(species, layout_names=None, s_plus=True):
    """Atomic start: H 1, He 0.1, C+ 1.4e-4, O 3e-4, Mg+ 5e-6 (S+ 8e-8 when the
    network has S+), everything else 1e-20; the electron slot holds the charge
    balance of those ions.  Returned in species-file slot order."""
    init = {"H": 1.0, "He": 0.1, "C+": 1.4e-4, "O": 3e-4, "Mg+": 5e-6}
    if s_plus:
        init["S+"] = 8e-8
    x = np.full(len(species), 1e-20)
    names = list(layout_names) + [species[-1]] if layout_names is not None else list(species)
    for i, s in enumerate(names[:-1]):
        if s in init:
            x[i] = init[s]
    q = np.array([s.count("+") - s.count("-") for s in names[:-1]], dtype=np.float64)
    x[-1] = float(np.dot(q, x[:-1]))
    return x


def chemistry(config, ncell=None, seed=None):
    """Cell inputs for configs 'C1' (reduced 4^3), 'C2' (full 32^3),
    'C3' (reduced 64^3).  ncell overrides the grid size (same distributions)."""
    cfg = {
        "C1": dict(network="reduced", ncell=64, seed=1001, tlog=False, g0log=False),
        "C2": dict(network="full", ncell=32768, seed=1002, tlog=True, g0log=True),
        "C3": dict(network="reduced", ncell=262144, seed=1003, tlog=False, g0log=False),
    }[config]
    n = cfg["ncell"] if ncell is None else ncell
    rng = _rng(cfg["seed"] if seed is None else seed)
    n_H = 10.0 ** rng.uniform(2.0, 5.0, n)
    T = 10.0 ** rng.uniform(1.0, np.log10(2000.0), n) if cfg["tlog"] else rng.uniform(10.0, 300.0, n)
    Td = rng.uniform(10.0, 20.0, n)
    G0 = 10.0 ** rng.uniform(0.0, 5.0, n) if cfg["g0log"] else np.full(n, 10.0)
    AV = rng.uniform(0.0, 10.0, (n, NRAYS))
    N_H2 = 10.0 ** rng.uniform(14.0, 22.0, (n, NRAYS))
    N_CO = 10.0 ** rng.uniform(10.0, 18.0, (n, NRAYS))
    N_C = 10.0 ** rng.uniform(10.0, 18.0, (n, NRAYS))
    N_S = 10.0 ** rng.uniform(10.0, 18.0, (n, NRAYS))
    col5 = np.stack([N_H2, np.zeros_like(N_H2), N_CO, N_C, N_S], axis=-1)  # H2, HD, CO, C, S
    rad = np.repeat((G0 / NRAYS)[:, None], NRAYS, axis=1)
    return ChemInputs(network=cfg["network"], n_H=n_H, T=T, Td=Td, G0=G0, AV=AV,
                      rad_surface=rad, column5=col5, t_end_yr=1e7, rtol=1e-8, atol=1e-30,
                      zeta=5e-17, omega=0.42, grain_radius=1e-7, metallicity=1.0, g2d=100.0,
                      v_turb_kms=1.0)


# coolant abundances relative to n_H for the level-population workload (stated)
COOLANT_X = {"CII": 1.4e-4, "CI": 1e-5, "OI": 3e-4, "CO": 1e-4}


def levpop(ncell=262144, seed=1004):
    """Config C4: n_H logU(1e2,1e6), T U(10,2000), x(H2) U(0,0.5),
    x(e) logU(1e-8,1e-3); x(H) = max(0, 1-2x(H2)), x(He) = 0.1, x(H+) = x(e);
    T_dust U(10,20) (stated).  Optical depths per line and ray are drawn per
    coolant by levpop_tau()."""
    rng = _rng(seed)
    n_H = 10.0 ** rng.uniform(2.0, 6.0, ncell)
    T = rng.uniform(10.0, 2000.0, ncell)
    xH2 = rng.uniform(0.0, 0.5, ncell)
    xe = 10.0 ** rng.uniform(-8.0, -3.0, ncell)
    Td = rng.uniform(10.0, 20.0, ncell)
    xH = np.maximum(0.0, 1.0 - 2.0 * xH2)
    partner5 = np.stack([xH * n_H, xe * n_H, xe * n_H, 0.1 * n_H, xH2 * n_H], axis=-1)
    return dict(n_H=n_H, T=T, Td=Td, partner5=partner5, seed=seed)


def levpop_tau(ncell, nlines, seed, nrays=NRAYS):
    """Sobolev line-centre optical depths logU(1e-3, 1e3) per (cell, line, ray)."""
    rng = _rng(seed)
    return 10.0 ** rng.uniform(-3.0, 3.0, (ncell, nlines, nrays))


def serve_stream(nreq, seed=1005, rate_hz=200.0):
    """Config C5: Poisson arrivals (mean 200/s), blocks of logU(1, 50000) cells,
    80% reduced / 20% full, t_end logU(1e4, 1e7) yr."""
    rng = _rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, nreq)
    arrival = np.cumsum(gaps)
    size = np.maximum(1, np.floor(10.0 ** rng.uniform(0.0, np.log10(50000.0), nreq))).astype(np.int64)
    network = np.where(rng.uniform(0.0, 1.0, nreq) < 0.8, "reduced", "full")
    t_end = 10.0 ** rng.uniform(4.0, 7.0, nreq)
    seeds = rng.integers(0, 2**31 - 1, nreq)
    return [dict(arrival=float(a), ncell=int(s), network=str(nw), t_end_yr=float(t), seed=int(sd))
            for a, s, nw, t, sd in zip(arrival, size, network, t_end, seeds)]


def healpix_base_directions():
    """The 12 ray directions of a level-0 HEALPix sphere (nside 1, 3DPDR.F90:311-333):
    the base-pixel centres, nested order: z = 2/3 north ring, z = 0 equator,
    z = -2/3 south ring, four azimuths each."""
    v = []
    for ring, z in ((0, 2.0 / 3.0), (1, 0.0), (2, -2.0 / 3.0)):
        for k in range(4):
            phi = (k + (0.0 if ring == 1 else 0.5)) * np.pi / 2.0
            s = np.sqrt(1.0 - z * z)
            v.append((s * np.cos(phi), s * np.sin(phi), z))
    return np.array(v)


def rays(n=8, maxpoints=12, spacing_pc=0.05, step_pc=0.05, nspec=33, seed=1007):
    """Evaluation points of every cell of an n^3 lattice along the 12 HEALPix
    directions: points march from the cell in steps of step_pc until they leave
    the lattice or reach maxpoints, each projected to its nearest lattice point
    (3D-PDR's ray tracing records the same kind of lists).  Stored padded:
    ray (c, j) starts at point (c*12 + j)*(maxpoints + 1), point 0 is the cell.
    Grid densities n_H ~ logU(1e2, 1e5), abundances ~ logU(1e-12, 1e-2)
    (seeded, stated)."""
    rng = _rng(seed)
    d = healpix_base_directions()
    nrays = len(d)
    ii, jj, kk = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    lat = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=-1).astype(np.float64)   # lattice coords
    ncell = len(lat)
    steps = np.arange(maxpoints + 1, dtype=np.float64) * (step_pc / spacing_pc)
    # positions in lattice units: (ncell, nrays, maxpoints+1, 3)
    pos = lat[:, None, None, :] + steps[None, None, :, None] * d[None, :, None, :]
    inside = np.all((pos >= -0.5) & (pos <= n - 0.5), axis=-1)
    epray = (np.cumprod(inside, axis=-1).sum(axis=-1) - 1).astype(np.int32)   # points after the cell
    proj = np.clip(np.rint(pos), 0, n - 1).astype(np.int64)
    gp = (proj[..., 0] * n * n + proj[..., 1] * n + proj[..., 2]).astype(np.int32)
    xyz = pos * spacing_pc
    offset = (np.arange(ncell * nrays, dtype=np.int64) * (maxpoints + 1))
    rho = 10.0 ** rng.uniform(2.0, 5.0, ncell)
    ab = 10.0 ** rng.uniform(-12.0, -2.0, (ncell, nspec))
    return dict(ncell=ncell, nrays=nrays, ngrid=ncell, npoint=ncell * nrays * (maxpoints + 1),
                epray=epray.reshape(-1), offset=offset, xyz=xyz.reshape(-1, 3), gridpoint=gp.reshape(-1),
                rho=rho, abundance=ab, vectors=d)


def slab_rays(x, ray=6):
    """Evaluation points of a PSEUDO_1D slab (points at x[i] pc on the x axis,
    illuminated on the x = 0 face): HEALPix ray `ray` (6 = -x) of every cell
    runs from the cell through every point nearer the face, in order; the
    other rays carry no points.  Same dict layout as rays()."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    nrays = 12
    order = np.argsort(-x, kind="stable")
    epray = np.zeros((n, nrays), np.int32)
    offset = np.zeros((n, nrays), np.int64)
    gp = []
    for c in range(n):
        pts = [c] + [int(j) for j in order if x[j] < x[c]]
        offset[c, :] = len(gp)
        epray[c, ray] = len(pts) - 1
        gp += pts
    gp = np.array(gp, np.int32)
    xyz = np.zeros((len(gp), 3))
    xyz[:, 0] = x[gp]
    return dict(ncell=n, nrays=nrays, ngrid=n, npoint=len(gp), epray=epray.reshape(-1), offset=offset.reshape(-1),
                xyz=xyz, gridpoint=gp, vectors=healpix_base_directions())
