"""Seeded synthetic inputs for the benchmark configurations.

No dataset is involved: every domain is generated from its description and a
seed, with the shapes, sizes and value ranges of the workloads the project is
measured on.

* :func:`poiseuille_guo`   D2Q9 channel 256 x 64, halfway bounce-back walls,
  periodic in x, Guo body force g, tau 0.8 (plain FP64 method).
* :func:`sphere_channel`   D3Q19 512 x 256 x 256 flow past a sphere of radius
  24 voxelised on cell centres, equilibrium inlet u = 0.05, zero-gradient
  outlet, free-slip side walls, tau drawn from [0.52, 0.6].
* :func:`pb_spheres`       D3Q7 Poisson-Boltzmann on 256^3: 1-64 charged
  non-overlapping spheres of radius 4-16 with surface potential in [0.5, 4]
  (units of kT/e), Debye length in [4, 32] cells, phi = 0 on the box.
* :func:`cavities`         the batched lid-driven cavities: sides in
  [32, 512], Re log-uniform in [10, 1000], lid velocity 0.1.
"""
from __future__ import annotations

import math
from typing import Dict, List

import numpy as np

D2Q9, D3Q7, D3Q19 = 2, 3, 4
FLUID, SOLID, INLET, OUTLET, DIRICHLET = 0, 1, 2, 3, 4


def poiseuille_guo(nx: int = 256, ny: int = 64, tau: float = 0.8, g: float = 1e-6) -> Dict:
    """Body-force driven channel: walls (halfway bounce-back) at y = -1/2 and
    y = ny - 1/2 in cell-centre coordinates, so the exact steady profile is
    u(y) = g / (2 nu) s (ny - s) with s = y + 1/2 and nu = (tau - 1/2)/3."""
    return dict(lattice=D2Q9, shape=(nx, ny, 1), omega=1.0 / tau, faces=("periodic", "periodic", "wall", "wall", "wall", "wall"),
                body_force=(g, 0.0, 0.0), tau=tau, g=g)


def poiseuille_profile(ny: int, tau: float, g: float) -> np.ndarray:
    nu = (tau - 0.5) / 3.0
    s = np.arange(ny) + 0.5
    return g / (2.0 * nu) * s * (ny - s)


def sphere_channel(nx=512, ny=256, nz=256, radius=24.0, center=(128.0, 128.0, 128.0), seed=2026, u_in=0.05) -> Dict:
    rng = np.random.default_rng(seed)
    tau = float(rng.uniform(0.52, 0.6))
    flags = np.zeros((nz, ny, nx), dtype=np.uint8)
    lo = [max(0, int(math.floor(c - radius - 1))) for c in center]
    hi = [int(math.ceil(c + radius + 1)) for c in center]
    z, y, x = np.meshgrid(np.arange(lo[2], min(hi[2], nz)), np.arange(lo[1], min(hi[1], ny)), np.arange(lo[0], min(hi[0], nx)),
                          indexing="ij")
    inside = (x + 0.5 - center[0]) ** 2 + (y + 0.5 - center[1]) ** 2 + (z + 0.5 - center[2]) ** 2 < radius * radius
    flags[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]][inside] = SOLID
    flags[:, :, 0] = INLET
    flags[:, :, -1] = OUTLET
    return dict(lattice=D3Q19, shape=(nx, ny, nz), omega=1.0 / tau, tau=tau, flags=flags.reshape(-1),
                faces=("open", "open", "freeslip", "freeslip", "freeslip", "freeslip"), inlet_velocity=(u_in, 0.0, 0.0))


def pb_spheres(n: int = 256, seed: int = 7, count: int | None = None, tau: float = 1.0) -> Dict:
    """Charged spheres in an electrolyte: cells inside a sphere carry the
    sphere's potential, the outermost layer of the box carries 0, everything
    else relaxes to nabla^2 phi = kappa^2 sinh(phi)."""
    rng = np.random.default_rng(seed)
    count = int(rng.integers(1, 65)) if count is None else count
    debye = float(rng.uniform(4.0, 32.0))
    spheres: List = []
    tries = 0
    while len(spheres) < count and tries < 100000:
        tries += 1
        r = float(rng.uniform(4.0, min(16.0, (n - 6) / 2.0)))  # radius 4-16, smaller in a box below 38 cells
        c = rng.uniform(r + 2, n - r - 2, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 + 2 for c2, r2, _ in spheres):
            spheres.append((c, r, float(rng.uniform(0.5, 4.0))))
    flags = np.zeros((n, n, n), dtype=np.uint8)
    phi = np.zeros((n, n, n))
    for c, r, ps in spheres:
        lo = [max(0, int(math.floor(v - r - 1))) for v in c]
        hi = [min(n, int(math.ceil(v + r + 1))) for v in c]
        z, y, x = np.meshgrid(np.arange(lo[2], hi[2]), np.arange(lo[1], hi[1]), np.arange(lo[0], hi[0]), indexing="ij")
        m = (x + 0.5 - c[0]) ** 2 + (y + 0.5 - c[1]) ** 2 + (z + 0.5 - c[2]) ** 2 < r * r
        flags[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]][m] = DIRICHLET
        phi[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]][m] = ps
    for sl in (np.s_[0, :, :], np.s_[-1, :, :], np.s_[:, 0, :], np.s_[:, -1, :], np.s_[:, :, 0], np.s_[:, :, -1]):
        flags[sl] = DIRICHLET
        phi[sl] = 0.0
    return dict(lattice=D3Q7, shape=(n, n, n), omega=1.0 / tau, equation=1, kappa_sq=1.0 / debye ** 2, flags=flags.reshape(-1),
                dirichlet=phi.reshape(-1), faces=("wall",) * 6, spheres=spheres, debye=debye)


def cavities(count: int = 2048, seed: int = 11, lid: float = 0.1, nmin: int = 32, nmax: int = 512) -> Dict:
    rng = np.random.default_rng(seed)
    sides = rng.integers(nmin, nmax + 1, size=count)
    re = np.exp(rng.uniform(math.log(10.0), math.log(1000.0), size=count))
    tau = 3.0 * lid * sides / re + 0.5
    return dict(sides=sides.astype(np.int32), re=re, tau=tau, lid=lid)


def cylinder_channel(seed: int, nx: int = 512, ny: int = 128, u_in: float = 0.05, re: float | None = None) -> Dict:
    """D2Q9 channel for the learned warm start: 1-8 non-overlapping cylinders
    of radius 6-20 cells at ny = 128, scaled with ny (solid where the cell
    centre is inside), equilibrium
    inlet u_in at x = 0, zero-gradient outlet at x = nx-1, bounce-back walls
    at y = -1/2 and ny - 1/2.  Re = u_in * ny / nu is drawn uniformly from
    [20, 200] (channel-height Reynolds number: the cylinder Reynolds numbers
    then stay below the onset of shedding, so every case has a steady state);
    `re` overrides the drawn value (cases stacked in one box share it)."""
    rng = np.random.default_rng(seed)
    count = int(rng.integers(1, 9))
    re_drawn = float(rng.uniform(20.0, 200.0))
    re = re_drawn if re is None else float(re)
    cyl: List = []
    tries = 0
    while len(cyl) < count and tries < 10000:
        tries += 1
        r = float(rng.uniform(6.0, 20.0)) * ny / 128.0  # radii scale with the channel height
        cx = float(rng.uniform(r + 0.1875 * ny, nx - r - 0.75 * ny))
        cy = float(rng.uniform(r + 3.0, ny - r - 3.0))
        if all((cx - x2) ** 2 + (cy - y2) ** 2 > (r + r2 + 3.0) ** 2 for x2, y2, r2 in cyl):
            cyl.append((cx, cy, r))
    y, x = np.meshgrid(np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    flags = np.zeros((ny, nx), dtype=np.uint8)
    for cx, cy, r in cyl:
        flags[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = SOLID
    flags[:, 0] = INLET
    flags[:, -1] = OUTLET
    nu = u_in * ny / re
    return dict(flags=flags, re=re, tau=3.0 * nu + 0.5, cylinders=cyl, u_in=u_in, shape=(nx, ny))


def forced_channel(seed: int, nx: int = 512, ny: int = 128, u_ref: float = 0.08, re: float | None = None) -> Dict:
    """The warm-start channel in its closed form: the cylinders of
    cylinder_channel(seed), periodic in x, bounce-back walls at y = -1/2 and
    ny - 1/2, driven by a Guo body force g.  Re = u_ref ny / nu with u_ref =
    g ny^2 / (8 nu), the centre-line speed of the empty channel; Re is drawn
    uniformly from [20, 200] (or given).  Mass is conserved exactly, so the
    steady state is unique for the initial mass."""
    c = cylinder_channel(seed, nx, ny, re=re)
    flags = (c["flags"] == SOLID).astype(np.uint8) * SOLID
    nu = u_ref * ny / c["re"]
    return dict(flags=flags, re=c["re"], tau=3.0 * nu + 0.5, g=8.0 * nu * u_ref / (ny * ny), cylinders=c["cylinders"], u_ref=u_ref,
                shape=(nx, ny))


def stacked_forced(cases_: List[Dict]) -> Dict:
    """Several forced channels with one Re as the z-slices of one D2Q9 box."""
    nx, ny = cases_[0]["shape"]
    flags = np.stack([c["flags"] for c in cases_]).reshape(-1)
    return dict(lattice=D2Q9, shape=(nx, ny, len(cases_)), omega=1.0 / cases_[0]["tau"], flags=flags,
                faces=("periodic", "periodic", "wall", "wall", "periodic", "periodic"), body_force=(cases_[0]["g"], 0.0, 0.0))


def stacked_channels(cases_: List[Dict], tau: float) -> Dict:
    """Several 2D channels as the z-slices of one D2Q9 box (the lattice has no
    z links, so the slices evolve independently) sharing one relaxation time."""
    nx, ny = cases_[0]["shape"]
    flags = np.stack([c["flags"] for c in cases_]).reshape(-1)
    return dict(lattice=D2Q9, shape=(nx, ny, len(cases_)), omega=1.0 / tau, flags=flags,
                faces=("open", "open", "wall", "wall", "periodic", "periodic"), inlet_velocity=(cases_[0]["u_in"], 0.0, 0.0))


def stacked_sweep(cases_: List[Dict]) -> Dict:
    """Inlet-driven channels (cylinder_channel) of any Reynolds numbers as the
    z-slices of one D2Q9 box: a sweep over geometry and Re stepped together,
    each slice relaxing at its own rate (`slice_omega`, for
    BoxSolver.set_slice_omega).  All channels share the box shape and the
    inlet speed."""
    nx, ny = cases_[0]["shape"]
    u_in = cases_[0]["u_in"]
    if any(tuple(c["shape"]) != (nx, ny) or c["u_in"] != u_in for c in cases_):
        raise ValueError("the channels of a sweep share the shape and the inlet speed")
    flags = np.stack([c["flags"] for c in cases_]).reshape(-1)
    return dict(lattice=D2Q9, shape=(nx, ny, len(cases_)), omega=1.0 / cases_[0]["tau"], flags=flags,
                faces=("open", "open", "wall", "wall", "periodic", "periodic"), inlet_velocity=(u_in, 0.0, 0.0),
                slice_omega=[1.0 / c["tau"] for c in cases_])


def stacked_debye(cases_: List[Dict]) -> Dict:
    """Poisson-Boltzmann boxes (pb_spheres) of any Debye lengths and charge
    placements stacked along z into one D3Q7 box: a sweep over Debye length
    stepped together, each box's slices at its own kappa^2 (`slice_kappa_sq`,
    for BoxSolver.set_slice_kappa).  Each box keeps its outer layer of
    Dirichlet cells, so the boxes do not exchange populations.  All boxes
    share nx, ny and the relaxation rate."""
    nx, ny, _ = cases_[0]["shape"]
    omega = cases_[0]["omega"]
    if any(tuple(c["shape"][:2]) != (nx, ny) or c["omega"] != omega for c in cases_):
        raise ValueError("the boxes of a Debye sweep share nx, ny and the relaxation rate")
    for c in cases_:
        f = c["flags"].reshape(c["shape"][2], ny, nx)
        if not (np.all(f[0] == DIRICHLET) and np.all(f[-1] == DIRICHLET)):
            raise ValueError("each box of a Debye sweep must be closed by Dirichlet planes in z")
    flags = np.concatenate([c["flags"] for c in cases_])
    phi = np.concatenate([c["dirichlet"] for c in cases_])
    kz = np.concatenate([np.full(c["shape"][2], c["kappa_sq"]) for c in cases_])
    nz = int(sum(c["shape"][2] for c in cases_))
    return dict(lattice=D3Q7, shape=(nx, ny, nz), omega=omega, equation=1, kappa_sq=cases_[0]["kappa_sq"], flags=flags,
                dirichlet=phi, faces=("wall",) * 6, slice_kappa_sq=kz.tolist(),
                z0=np.cumsum([0] + [c["shape"][2] for c in cases_])[:-1].tolist())


def box_kwargs(case: Dict) -> Dict:
    """The BoxSolver / BoxOracle keyword arguments of a case."""
    keys = ("faces", "flags", "wall_velocity", "body_force", "inlet_velocity", "equation", "kappa_sq", "dirichlet")
    return {k: case[k] for k in keys if k in case}
