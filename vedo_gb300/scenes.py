"""Seeded synthetic scenes with the shapes of the DEM workloads this engine is measured on.

All scenes are built from numpy's PCG64 generator (bit-identical on x86_64 and
aarch64) and are plain :class:`~vedo_gb300.scene.Scene` objects, so the same
scene can be written as a reference ``.ido`` file and run by the reference CPU
code, the C oracle and the GPU engine.

* :func:`lsd_box` - 8,000 monodisperse spheres (r = 1 mm, 2500 kg/m^3) on a
  jittered 20x20x20 lattice (2.2 mm spacing, U(+-0.05 mm) jitter, N(0, 0.05 m/s)
  velocities) falling under g = 9.81 into an open box of 5 fixed plates 50 mm
  wide and 60 mm tall; linear spring-dashpot ``ISwBSDBF`` with kn = 1e4 N/m,
  ks = 0.8 kn, restitution 0.8, friction 0.5; dt = 1e-6 s.
* :func:`hertz_drum` - polydisperse Hertz spheres (lognormal radii binned into K
  classes, one DOModel per class) in a horizontal drum of R = 0.15 m, L = 0.3 m
  whose shell (one hollow cylinder, or a polygon of fixed plates) and two end plates
  turn at 30 rpm; filled by seeded random sequential placement.
* :func:`hopper` / :func:`hopper_batch` - flat-bottomed hoppers discharging through a
  rectangular orifice (a box of fixed plates whose floor is four plates around the
  orifice), monodisperse r = 1 mm Hertz spheres with friction (``ISwH``); the batch
  draws sphere counts log-uniform on [1e3, 5e4], friction U(0.2, 0.6), restitution
  U(0.5, 0.9) and orifice width U(6, 12) mm per scene.
* :func:`compressed_bed` - a large monodisperse Hertz bed (16,000,000 spheres of
  r = 0.5 mm by default, E = 10 GPa, friction 0.5) at solid fraction 0.55 in a
  0.4 x 0.4 m box of plates with 32 fixed vertical cylinders (r = 5 mm) on a jittered
  grid, compressed by an orbital top plate moving down at 0.05 m/s.
* :func:`dense_pack` - a contact-dense stress case: spheres on a face-centred cubic lattice
  whose neighbours overlap by a hair (12 contacts per sphere from the first step).
* :func:`serving_job` - the serving stream's jobs: a settling box or a projectile
  impact on a bed, lognormal radii (median 1 mm, sigma_log 0.15) in 8 classes, linear
  spring-dashpot or Hertz (``ISwH``, E = 0.5 GPa) contact.
* :func:`cluster` - small random clusters used by the parity tests (every
  solver, plates, cylinders, orbital walls).
"""
from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .scene import (CONSTRAINED, FIXED, GLOBAL, INNER_CYLINDER, LOCAL, MOBILE, ORBITAL, QUASI_CYLINDER, QUASI_PLATE,
                    QUASI_PLATE_WITH_CIRCULAR_HOLE, SPHERE,
                    Boundary, DOModel, IactModel, Scene, SystemParameter)


def damping_ratio(e: float) -> float:
    """Viscous damping ratio zeta of a linear spring-dashpot with restitution e."""
    le = math.log(e)
    return -le / math.sqrt(math.pi * math.pi + le * le)


def lsd_mechanisms(kn: float, ks: float, beta_n: float, beta_s: float, mu: float) -> List[Tuple[str, float]]:
    """Mechanism list read by ISwBSDBF's constructor (ISwBSDBF.cpp:10-18)."""
    return [("NormalStiffness", kn), ("ShearStiffness", ks), ("NormalDampingRatio", beta_n),
            ("ShearDampingRatio", beta_s), ("NormalBondStrength", 0.0), ("ShearBondStrength", 0.0),
            ("FrictionCoefficient", mu)]


def time_control(steps: int, dt: float) -> SystemParameter:
    """t_stop = (steps - 1/2) dt: the reference loop runs while t_current < t_stop after each
    step (SimMediator.cpp:839-841), so exactly `steps` steps run despite FP accumulation of t."""
    return SystemParameter(time_start=0.0, time_stop=(steps - 0.5) * dt, time_interval=dt, time_current=0.0)


def box_walls(width: float, height: float, thickness: float, depth_z0: float = 0.0):
    """Five fixed quasi-plates forming an open box: floor top surface at z = z0, inner side
    faces at x, y = +-width/2, walls `height` tall.  A plate's normal is OrientationZ, its
    width runs along OrientationX and its length along Oz x Ox (CDSphere2QuasiPlate.cpp:29-65)."""
    h = thickness
    L = width + 2 * h
    floor = DOModel("Floor", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (L, h, L))
    side = DOModel("Sides", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (height, h, L))
    pos = [(0.0, 0.0, depth_z0 - 0.5 * h)]
    ox = [(1.0, 0.0, 0.0)]
    oz = [(0.0, 0.0, 1.0)]
    zc = depth_z0 + 0.5 * height
    for sx, sy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        pos.append((sx * (0.5 * width + 0.5 * h), sy * (0.5 * width + 0.5 * h), zc))
        ox.append((0.0, 0.0, 1.0))
        oz.append((float(sx), float(sy), 0.0))
    return [floor, side], [0, 1, 1, 1, 1], np.array(pos), np.array(ox), np.array(oz)


def lsd_box(n_side: int = 20, seed: int = 12345, steps: int = 20000, dt: float = 1e-6, radius: float = 1e-3,
            density: float = 2500.0, spacing: float = 2.2e-3, jitter: float = 5e-5, vel_sigma: float = 0.05,
            kn: float = 1e4, ks_ratio: float = 0.8, restitution: float = 0.8, mu: float = 0.5,
            box_width: float = 0.05, box_height: float = 0.06, wall_thickness: float = 2e-3) -> Scene:
    """The plain FP64 linear spring-dashpot box (8,000 spheres at n_side = 20)."""
    rng = np.random.default_rng(seed)
    i, j, k = np.meshgrid(np.arange(n_side), np.arange(n_side), np.arange(n_side), indexing="ij")
    grid = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pos = np.empty_like(grid)
    pos[:, 0] = (grid[:, 0] - 0.5 * (n_side - 1)) * spacing
    pos[:, 1] = (grid[:, 1] - 0.5 * (n_side - 1)) * spacing
    pos[:, 2] = grid[:, 2] * spacing + 2.0 * radius
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    vel = rng.normal(0.0, vel_sigma, size=pos.shape)
    n = pos.shape[0]
    zeta = damping_ratio(restitution)
    # VEDO damps with the mean mass 1/2(ma+mb) (ISwModels.cpp:88-108): for equal spheres that is
    # m, twice the reduced mass, so beta = zeta/sqrt(2) gives the intended restitution; against a
    # wall (SudoMass 0) the sphere mass is the reduced mass and beta = zeta.
    ball = DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,))
    wmodels, widx, wpos, wox, woz = box_walls(box_width, box_height, wall_thickness)
    models = [ball] + wmodels
    iacts = [IactModel("Ball", "Ball", "ISwBSDBF", lsd_mechanisms(kn, ks_ratio * kn, zeta / math.sqrt(2.0),
                                                                  zeta / math.sqrt(2.0), mu)),
             IactModel("Wall", "Ball", "ISwBSDBF", lsd_mechanisms(kn, ks_ratio * kn, zeta, zeta, mu))]
    model_index = np.concatenate([np.zeros(n, np.uint32), 1 + np.array(widx, np.uint32)])
    P = np.concatenate([pos, wpos])
    V = np.concatenate([vel, np.zeros((len(widx), 3))])
    OX = np.concatenate([np.tile([1.0, 0.0, 0.0], (n, 1)), wox])
    OZ = np.concatenate([np.tile([0.0, 0.0, 1.0], (n, 1)), woz])
    return Scene(time_control(steps, dt), models, iacts, model_index, P, V, OX, OZ)


# ---------------------------------------------------------------------------------------------
def hertz_constants(E: float, nu: float, r_a: float, r_b: Optional[float], rho: float):
    """kn = 4/3 E* sqrt(R*) for the ISwHertz normal law (ISwModels.cpp:127-132); r_b None = wall."""
    Es = E / (2.0 * (1.0 - nu * nu)) if r_b is not None else E / (1.0 - nu * nu)
    Rs = r_a * r_b / (r_a + r_b) if r_b is not None else r_a
    return 4.0 / 3.0 * Es * math.sqrt(Rs)


def _sequential_placement(rng, radii: np.ndarray, inside, lo: np.ndarray, hi: np.ndarray, max_tries: int = 60):
    """Seeded random sequential placement: candidates drawn uniformly in [lo, hi]; a sphere is
    kept when `inside(p, r)` holds and it overlaps no sphere placed before (cell grid check)."""
    rmax = float(radii.max())
    cell = 2.0 * rmax
    dims = np.maximum(1, np.ceil((hi - lo) / cell).astype(np.int64))
    grid = {}
    out = np.full((radii.shape[0], 3), np.nan)
    placed = 0
    for idx in range(radii.shape[0]):
        r = radii[idx]
        for _ in range(max_tries):
            p = lo + rng.random(3) * (hi - lo)
            if not inside(p, r):
                continue
            c = np.floor((p - lo) / cell).astype(np.int64)
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for q in grid.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                            d = p - out[q]
                            if d @ d < (r + radii[q]) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                out[idx] = p
                grid.setdefault((c[0], c[1], c[2]), []).append(idx)
                placed += 1
                break
    keep = ~np.isnan(out[:, 0])
    return out[keep], keep


def place_spheres(radii: np.ndarray, lo, hi, cyl_radius: float = 0.0, seed: int = 0, max_tries: int = 2000):
    """Seeded random sequential placement through the engine library (vedo_place_spheres):
    sphere i, in the given order, is drawn uniformly in the box [lo, hi] (and, for
    cyl_radius > 0, inside that cylinder about the x axis), each wholly inside, and kept at
    its first draw that overlaps no sphere kept before.  Returns ([n][3] centres with NaN for
    spheres not placed, number placed)."""
    import ctypes as C
    from .engine import lib
    L = lib()
    dp = C.POINTER(C.c_double)
    L.vedo_place_spheres.argtypes = [C.c_uint32, dp, dp, dp, C.c_double, C.c_uint64, C.c_uint32, dp,
                                     C.POINTER(C.c_uint32)]
    radii = np.ascontiguousarray(radii, np.float64)
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    out = np.empty((radii.shape[0], 3))
    placed = C.c_uint32(0)
    rc = L.vedo_place_spheres(radii.shape[0], radii.ctypes.data_as(dp), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp),
                              float(cyl_radius), int(seed) & (2**64 - 1), int(max_tries), out.ctypes.data_as(dp),
                              C.byref(placed))
    if rc != 0:
        raise ValueError(f"vedo_place_spheres failed ({rc})")
    return out, int(placed.value)


def _circle_area_below(R: float, c: float) -> float:
    """Area of the disc of radius R about the origin below the line z = c."""
    c = min(max(c, -R), R)
    return R * R * math.acos(-c / R) + c * math.sqrt(max(R * R - c * c, 0.0))


def cluster(n: int = 64, seed: int = 7, solver: str = "ISwBSDBF", walls: str = "box", steps: int = 200,
            dt: float = 1e-6, radius: float = 1e-3, polydisperse: bool = False, density: float = 2500.0,
            vel_sigma: float = 0.2, orbital: bool = False, cylinders: int = 0, spacing: float = 2.05e-3,
            friction: float = 0.5) -> Scene:
    """Small jittered lattice of spheres close enough to collide within a few hundred steps,
    in a box of plates (optionally with orbital walls and vertical cylinders)."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(n ** (1.0 / 3.0)))
    g = np.stack(np.meshgrid(*(np.arange(side),) * 3, indexing="ij"), -1).reshape(-1, 3)[:n].astype(float)
    pos = (g - 0.5 * (side - 1)) * spacing
    pos[:, 2] += 0.5 * side * spacing + 1.5 * radius
    pos += rng.uniform(-0.02 * spacing, 0.02 * spacing, size=pos.shape)
    vel = rng.normal(0.0, vel_sigma, size=pos.shape)
    avel = rng.normal(0.0, 20.0, size=pos.shape)
    models: List[DOModel] = []
    if polydisperse:
        radii = np.array([0.8, 0.9, 1.0]) * radius
        for k, r in enumerate(radii):
            models.append(DOModel(f"Ball{k}", f"B{k}", MOBILE, LOCAL, density, 1.0, SPHERE, (float(r),)))
        midx = rng.integers(0, 3, size=n).astype(np.uint32)
    else:
        models.append(DOModel("Ball", "B0", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,)))
        midx = np.zeros(n, np.uint32)
    groups = sorted({m.group for m in models})
    extent = side * spacing + 4 * radius
    P, V, OX, OZ, AV = [pos], [vel], [np.tile([1.0, 0, 0], (n, 1))], [np.tile([0, 0, 1.0], (n, 1))], [avel]
    wall_groups = []
    if walls == "box":
        base = len(models)
        wm, widx, wp, wox, woz = box_walls(extent, extent + 4 * radius, 1e-3)
        if orbital:
            wm[1] = DOModel("Sides", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, QUASI_PLATE, wm[1].attrs)
        models += wm
        midx = np.concatenate([midx, base + np.array(widx, np.uint32)])
        P.append(wp); V.append(np.zeros_like(wp)); OX.append(wox); OZ.append(woz)
        wav = np.zeros_like(wp)
        if orbital:
            wav[1:, 2] = 3.0   # side plates spin slowly about the vertical axis through their own centres
        AV.append(wav)
        wall_groups.append("Wall")
    if cylinders:
        base = len(models)
        models.append(DOModel("Rod", "Rod", FIXED, GLOBAL, 0.0, 1.0, QUASI_CYLINDER, (0.6 * radius, extent)))
        cp = np.zeros((cylinders, 3))
        ang = np.arange(cylinders) * 2 * math.pi / cylinders
        cp[:, 0] = 0.3 * extent * np.cos(ang)
        cp[:, 1] = 0.3 * extent * np.sin(ang)
        cp[:, 2] = 0.5 * extent
        midx = np.concatenate([midx, np.full(cylinders, base, np.uint32)])
        P.append(cp); V.append(np.zeros_like(cp)); OX.append(np.tile([1.0, 0, 0], (cylinders, 1)))
        OZ.append(np.tile([0, 0, 1.0], (cylinders, 1))); AV.append(np.zeros_like(cp))
        wall_groups.append("Rod")
    iacts = []
    e = 0.7
    zeta = damping_ratio(e)
    for ga in groups + wall_groups:
        for gb in groups:
            if ga in wall_groups or ga <= gb:
                iacts.append(IactModel(ga, gb, solver, _mechanisms(solver, zeta, friction)))
    sc = Scene(time_control(steps, dt), models, iacts, midx, np.concatenate(P), np.concatenate(V),
               np.concatenate(OX), np.concatenate(OZ), np.concatenate(AV))
    return sc


def piston(n: int = 48, seed: int = 11, solver: str = "ISwBSDBF", behavior: str = "mobile", steps: int = 1000,
           dt: float = 1e-6, speed: float = 0.5, spin: float = 4.0, lid_density: float = 2500.0) -> Scene:
    """The colliding cluster of :func:`cluster` in its box of fixed plates, under a lid: a plate
    (2 mm thick) that is a mobile quasi-plate (`behavior` "mobile": DOQuasiPlate, moved by its
    impulses in translation and rotation) or a constrained one ("constrained":
    DOConstrainedQuasiPlate, moved only along its normal), starting 0.2 mm above the top layer at
    `speed` m/s downwards (and turning at `spin` rad/s about a horizontal axis when mobile), falling
    under gravity onto the spheres and pushed back by them."""
    sc = cluster(n=n, seed=seed, solver=solver, steps=steps, dt=dt)
    sph = np.array([sc.models[m].shape == SPHERE for m in sc.model_index])
    radius = sc.models[0].attrs[0]
    top = float(sc.position[sph, 2].max()) + radius
    side = int(math.ceil(n ** (1.0 / 3.0)))
    inner = side * 2.05e-3 + 4 * radius
    w = inner - 2.0 * radius                       # clear of the side plates
    beh = {"mobile": MOBILE, "constrained": CONSTRAINED}[behavior]
    models = list(sc.models) + [DOModel("Lid", "Lid", beh, GLOBAL, lid_density, 1.0, QUASI_PLATE, (w, 2e-3, w))]
    lid = len(models) - 1
    zeta = damping_ratio(0.7)
    iacts = list(sc.iact_models) + [IactModel("Lid", "B0", solver, _mechanisms(solver, zeta, 0.5))]
    app = lambda a, row: np.concatenate([a, np.asarray([row], dtype=np.float64)])   # noqa: E731
    return Scene(sc.sp, models, iacts, np.concatenate([sc.model_index, np.array([lid], np.uint32)]),
                 app(sc.position, [0.0, 0.0, top + 2e-4 + 1e-3]), app(sc.velocity, [0.0, 0.0, -speed]),
                 app(sc.orientation_x, [1.0, 0.0, 0.0]), app(sc.orientation_z, [0.0, 0.0, 1.0]),
                 app(sc.angular_velocity, [spin if behavior == "mobile" else 0.0, 0.0, 0.0]))


def _mechanisms(solver: str, zeta: float, mu: float):
    if solver in ("ISwBSDBF", "ISwBtSDBF", "ISwBSDB2F"):
        return lsd_mechanisms(1e4, 8e3, zeta, zeta, mu)
    if solver == "ISwHertz":
        return [("NormalStiffness", 5e7), ("NormalDampingCoefficient", 2e-2)]
    if solver == "ISwH":
        return [("HertzNormalStiffness", 5e7), ("EquivalentMass", 5e-6), ("ShearStiffnessCoefficient1", 2.0),
                ("ShearStiffnessCoefficient2", 3e3), ("DampingRatio", zeta), ("KineticFrictionCoefficient", mu)]
    raise ValueError(solver)


# ---------------------------------------------------------------------------------------------
def hertz_drum(n: int = 1_000_000, seed: int = 2024, steps: int = 10000, dt: float = 5e-7, K: int = 32,
               median_r: float = 1e-3, sigma_log: float = 0.2, r_lo: float = 0.5e-3, r_hi: float = 2e-3,
               E: float = 70e9, nu: float = 0.25, restitution: float = 0.7, mu: float = 0.4,
               density: float = 2500.0, R: float = 0.15, L: float = 0.3, rpm: float = 30.0,
               facets: int = 64, gap: float = 0.01, solver: str = "ISwH", vel_sigma: float = 0.0,
               fill: str = "rsa", rsa_fraction: float = 0.30, shell: str = "cylinder") -> Scene:
    """Polydisperse Hertz drum.

    Radii are lognormal(median_r, sigma_log) clipped to [r_lo, r_hi] and binned into K
    log-spaced classes; each class is one DOModel and one group, with K(K+1)/2 sphere-sphere
    and K sphere-wall interaction models (Hertz stiffness from E, nu and the class radii).
    shell="cylinder" (the default): the shell is one orbital hollow cylinder of radius R about
    the x axis turning at `rpm` with the end plates (the engine's inner-cylinder extension; the
    reference has no hollow cylinder, so such a scene runs on the engine and its oracle only).
    shell="polygon": `facets` fixed quasi-plates on a circle of radius R, which the reference
    can read.  The two end plates are orbital plates spinning at `rpm` about x.

    fill="rsa" (the default): random sequential placement, largest spheres first, in the part
    of the drum below the height at which the spheres make up `rsa_fraction` of its volume
    (0.30: the 1,000,000 default spheres, about 5.0e-3 m^3 of solid, occupy the lower ~75 % of
    the drum; settled under gravity they fill it to about 35-40 %).  fill="lattice": horizontal
    lattice layers from the bottom, largest first, each layer's spacing set by its largest
    sphere plus a `gap` fraction (no initial overlap, about 40 % of the drum volume).  Initial
    velocities are zero unless `vel_sigma` (m/s, per component) is given.

    Object order is a seeded permutation with one sphere of the largest class moved to the end
    of the sphere block.  The reference's NBS broad phase takes its cell size from the radius of
    the last local object, not the largest (NBSConsultant.cpp:140); with a small sphere last,
    contacts between large spheres are missed, they interpenetrate and the packing heats up.
    With the largest radius last that cell size is the correct one."""
    rng = np.random.default_rng(seed)
    edges = np.exp(np.linspace(math.log(r_lo), math.log(r_hi), K + 1))
    centres = np.sqrt(edges[:-1] * edges[1:])
    r = np.clip(median_r * np.exp(sigma_log * rng.standard_normal(n)), r_lo, r_hi)
    cls = np.clip(np.searchsorted(edges, r, side="right") - 1, 0, K - 1).astype(np.uint32)
    cls = np.sort(cls)[::-1].copy()            # largest classes first (bottom layers / placed first)
    radii = centres[cls]
    pos = np.zeros((n, 3))
    z = -R
    placed = 0
    if fill == "rsa":
        solid = float(np.sum(4.0 / 3.0 * math.pi * radii ** 3))
        lo_z, hi_z = -R, R                     # height below which the drum holds solid / rsa_fraction
        for _ in range(80):
            mid = 0.5 * (lo_z + hi_z)
            if _circle_area_below(R, mid) * L * rsa_fraction < solid:
                lo_z = mid
            else:
                hi_z = mid
        z_top = hi_z
        for attempt in range(40):
            top = min(z_top * 1.0 + attempt * 0.01 * R, R)
            pos, placed = place_spheres(radii, (-0.5 * L, -R, -R), (0.5 * L, R, top), cyl_radius=R,
                                        seed=seed * 1000003 + attempt)
            if placed == n:
                break
        if placed != n:
            raise ValueError(f"random sequential placement kept {placed} of {n} spheres")
    elif fill != "lattice":
        raise ValueError(f"unknown fill {fill!r}")
    while placed < n:
        rl = radii[placed]                       # largest radius of this layer (sorted descending)
        a = 2.0 * rl * (1.0 + gap)
        zc = z + a * 0.5 + 0.5 * gap * rl
        half = math.sqrt(max(0.0, (R - 0.5 * a) ** 2 - zc * zc)) if abs(zc) < R - 0.5 * a else 0.0
        if half < a:
            if zc > 0.0:
                raise ValueError(f"drum full after {placed} of {n} spheres")
            z += a
            continue
        ys = np.arange(-half + 0.5 * a, half - 0.5 * a + 1e-12, a)
        xs = np.arange(-0.5 * L + 0.5 * a, 0.5 * L - 0.5 * a + 1e-12, a)
        X, Y = np.meshgrid(xs, ys, indexing="ij")
        sites = np.stack([X.ravel(), Y.ravel(), np.full(X.size, zc)], 1)
        take = min(n - placed, sites.shape[0])
        pos[placed:placed + take] = sites[:take]
        placed += take
        z += a
    if fill == "lattice":
        pos += rng.uniform(-0.25 * gap, 0.25 * gap, size=pos.shape) * radii[:, None]
    perm = rng.permutation(n)                  # object order independent of the layer order
    last = int(np.flatnonzero(cls[perm] == cls.max())[-1])
    perm[[last, n - 1]] = perm[[n - 1, last]]  # a largest-class sphere last: see the docstring
    pos, cls = pos[perm], cls[perm]
    vel = rng.normal(0.0, vel_sigma, size=pos.shape) if vel_sigma > 0 else np.zeros_like(pos)
    models: List[DOModel] = []
    for k in range(K):
        models.append(DOModel(f"B{k:03d}", f"B{k:03d}", MOBILE, LOCAL, density, 1.0, SPHERE, (float(centres[k]),)))
    thick = 4e-3
    omega = rpm * 2.0 * math.pi / 60.0
    if shell == "cylinder":
        shell_m = DOModel("Shell", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, INNER_CYLINDER, (R, L + 2 * thick))
    elif shell == "polygon":
        fw = 2.0 * R * math.tan(math.pi / facets) * 1.02
        shell_m = DOModel("Shell", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (L + 2 * thick, thick, fw))
    else:
        raise ValueError(f"unknown shell {shell!r}")
    endp = DOModel("EndPl", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, QUASI_PLATE, (2.2 * R, thick, 2.2 * R))
    models += [shell_m, endp]
    wp, wox, woz, wav, widx = [], [], [], [], []
    if shell == "cylinder":                    # axis x through the centre, turning about it
        wp.append([0.0, 0.0, 0.0])
        woz.append([1.0, 0.0, 0.0])
        wox.append([0.0, 1.0, 0.0])
        wav.append([omega, 0.0, 0.0])
        widx.append(K)
    else:
        for f in range(facets):
            th = 2.0 * math.pi * (f + 0.5) / facets
            nrm = np.array([0.0, math.cos(th), math.sin(th)])
            wp.append(nrm * (R + 0.5 * thick))
            woz.append(-nrm)
            wox.append([1.0, 0.0, 0.0])
            wav.append([0.0, 0.0, 0.0])
            widx.append(K)
    for sx in (-1.0, 1.0):
        wp.append([sx * (0.5 * L + 0.5 * thick), 0.0, 0.0])
        woz.append([-sx, 0.0, 0.0])
        wox.append([0.0, 1.0, 0.0])
        wav.append([omega, 0.0, 0.0])
        widx.append(K + 1)
    iacts = []
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    for ka in range(K):
        for kb in range(ka, K):
            iacts.append(IactModel(models[ka].group, models[kb].group, solver,
                                   _hertz_mech(solver, E, nu, centres[ka], centres[kb], m_of, zeta, mu)))
    for ka in range(K):
        iacts.append(IactModel("Wall", models[ka].group, solver,
                               _hertz_mech(solver, E, nu, centres[ka], None, m_of, zeta, mu)))
    model_index = np.concatenate([cls, np.array(widx, np.uint32)])
    P = np.concatenate([pos, np.array(wp)])
    V = np.concatenate([vel, np.zeros((len(widx), 3))])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array(wox)])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array(woz)])
    AV = np.concatenate([np.zeros((n, 3)), np.array(wav)])
    return Scene(time_control(steps, dt), models, iacts, model_index, P, V, OX, OZ, AV)


def _hertz_mech(solver, E, nu, ra, rb, m_of, zeta, mu):
    kn = hertz_constants(E, nu, ra, rb, 0.0)
    meff = m_of(ra) if rb is None else m_of(ra) * m_of(rb) / (m_of(ra) + m_of(rb))
    if solver == "ISwHertz":
        cn = 2.0 * zeta * math.sqrt(meff * kn * math.sqrt(1e-6))   # damping at 1 um overlap
        return [("NormalStiffness", kn), ("NormalDampingCoefficient", cn)]
    # ISwH: ks = ksc1 (ksc2 |kn delta|)^(1/3) (ISwH.cpp:213) is Mindlin's kt = 8 G* a with the
    # Hertz contact radius a = (3 F R* / (4 E*))^(1/3): ksc1 = 8 G*, ksc2 = 3 R* / (4 E*).
    G = E / (2.0 * (1.0 + nu))
    Gs = G / (2.0 * (2.0 - nu)) if rb is not None else G / (2.0 - nu)
    Es = E / (2.0 * (1.0 - nu * nu)) if rb is not None else E / (1.0 - nu * nu)
    Rs = ra if rb is None else ra * rb / (ra + rb)
    return [("HertzNormalStiffness", kn), ("EquivalentMass", meff),
            ("ShearStiffnessCoefficient1", 8.0 * Gs), ("ShearStiffnessCoefficient2", 3.0 * Rs / (4.0 * Es)),
            ("DampingRatio", zeta), ("KineticFrictionCoefficient", mu)]


def hopper(n: int = 10000, seed: int = 0, friction: float = 0.4, restitution: float = 0.7, orifice: float = 8e-3,
           steps: int = 5000, dt: float = 5e-7, radius: float = 1e-3, density: float = 2500.0, E: float = 70e9,
           nu: float = 0.25, spacing_factor: float = 1.1, vel_sigma: float = 0.01, touching: bool = False) -> Scene:
    """Flat-bottomed hopper discharging through a square orifice of side `orifice`.

    The spheres start on a jittered square-prism lattice (spacing `spacing_factor` x 2r),
    about twice as tall as wide, resting 0.05 r above the floor; with `touching` on a simple
    cubic lattice whose neighbours and floor touch exactly (no jitter, at rest), so that the
    column carries its contacts from the first step while it drains.  Walls: four fixed side
    plates and a floor of four fixed plates that leave the orifice open in its centre (the
    reference's only holed plate has a circular hole, so the rectangular orifice is built from
    plain plates).  Contact: ``ISwH`` (Hertz normal stiffness with friction) from E, nu,
    restitution and friction, for sphere-sphere and sphere-wall."""
    rng = np.random.default_rng(seed)
    if touching:
        spacing_factor = 1.0
    a = 2.0 * radius * spacing_factor
    m = max(2, int(math.ceil((n / 2.0) ** (1.0 / 3.0))))
    nz = int(math.ceil(n / (m * m)))
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = np.empty((n, 3))
    pos[:, 0] = (g[:, 0] - 0.5 * (m - 1)) * a
    pos[:, 1] = (g[:, 1] - 0.5 * (m - 1)) * a
    pos[:, 2] = g[:, 2] * a + (1.0 if touching else 1.05) * radius
    jitter = rng.uniform(-0.02 * radius, 0.02 * radius, size=pos.shape)
    vel = rng.normal(0.0, vel_sigma, size=pos.shape)
    if touching:
        vel[:] = 0.0
    else:
        pos += jitter
    W = m * a if touching else m * a + 2.0 * radius    # inner width of the box
    H = nz * a + 4.0 * radius                      # side wall height
    t = 2e-3                                       # plate thickness
    w = min(orifice, W - 4.0 * radius)
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,)),
              DOModel("Side", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (H, t, W + 2 * t)),
              DOModel("FloorLR", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (0.5 * (W - w), t, W)),
              DOModel("FloorFB", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (w, t, 0.5 * (W - w)))]
    wp, wox, woz, widx = [], [], [], []
    for sx, sy in ((1, 0), (-1, 0), (0, 1), (0, -1)):   # sides: normal points inwards
        wp.append((sx * (0.5 * W + 0.5 * t), sy * (0.5 * W + 0.5 * t), 0.5 * H))
        wox.append((0.0, 0.0, 1.0))
        woz.append((-float(sx), -float(sy), 0.0))
        widx.append(1)
    q = 0.25 * (W + w)                             # centre of a floor strip beside the orifice
    for sx in (1, -1):                             # left/right strips, full depth
        wp.append((sx * q, 0.0, -0.5 * t)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, 1.0)); widx.append(2)
    for sy in (1, -1):                             # front/back strips between them
        wp.append((0.0, sy * q, -0.5 * t)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, 1.0)); widx.append(3)
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = [IactModel("Ball", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, radius, m_of, zeta, friction)),
             IactModel("Wall", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, None, m_of, zeta, friction))]
    k = len(widx)
    midx = np.concatenate([np.zeros(n, np.uint32), np.array(widx, np.uint32)])
    P = np.concatenate([pos, np.array(wp)])
    V = np.concatenate([vel, np.zeros((k, 3))])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array(wox)])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array(woz)])
    AV = np.zeros((n + k, 3))
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)


def spinning_plate(omega: float = 500.0, steps: int = 3000, dt: float = 2e-7, radius: float = 1e-3,
                   half: float = 10e-3, E: float = 70e9, nu: float = 0.25, restitution: float = 0.7,
                   friction: float = 0.4, density: float = 2500.0) -> Scene:
    """A square orbital plate (side 2 `half`, 2 mm thick, normal +z) spinning in its own plane at
    `omega` rad/s about its centre, with spheres at rest in that plane just outside it, no field:
    the turning corners sweep into the spheres (four spheres sit 15 degrees ahead of a corner,
    four 25 degrees, all within the rounded corners' reach by 5 % of r, and clear of the plate
    at the start).  A check of how the list handles
    a wall whose plane never moves while its edges do.  ISwH contact."""
    rho = half * math.sqrt(2.0) + 1e-3 + 0.95 * radius   # the rounded corners' reach + 0.95 r
    ang = [math.radians(45.0 + 15.0 + 90.0 * q) for q in range(4)] + \
          [math.radians(45.0 + 25.0 + 90.0 * q) for q in range(4)]
    pos = np.array([[rho * math.cos(a), rho * math.sin(a), 0.0] for a in ang])
    n = pos.shape[0]
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,)),
              DOModel("Plate", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, QUASI_PLATE, (2 * half, 2e-3, 2 * half))]
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = [IactModel("Ball", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, radius, m_of, zeta, friction)),
             IactModel("Wall", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, None, m_of, zeta, friction))]
    sp = time_control(steps, dt)
    sp.field_acceleration = (0.0, 0.0, 0.0)
    midx = np.concatenate([np.zeros(n, np.uint32), np.array([1], np.uint32)])
    P = np.concatenate([pos, np.zeros((1, 3))])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array([[1.0, 0.0, 0.0]])])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array([[0.0, 0.0, 1.0]])])
    AV = np.concatenate([np.zeros((n, 3)), np.array([[0.0, 0.0, omega]])])
    return Scene(sp, models, iacts, midx, P, np.zeros((n + 1, 3)), OX, OZ, AV)


def shell_drop(n: int = 150, seed: int = 6, steps: int = 600, dt: float = 1e-6, radius: float = 0.5e-3,
               R: float = 8e-3, length: float = 12e-3, solver: str = "ISwBSDBF", rpm: float = 0.0,
               speed: float = 3.0) -> Scene:
    """Spheres inside a horizontal hollow cylinder (the engine's inner-cylinder extension, axis
    x, radius R, closed by two fixed plates) placed by random sequential placement in its bottom
    band and thrown outwards at `speed` m/s, so that most reach the shell within a few hundred
    steps.  `rpm` turns the shell (orbital) about its axis.  LSD (ISwBSDBF) by default, for
    bit-exact comparisons."""
    rng = np.random.default_rng(seed)
    radii = np.full(n, radius)
    pos, placed = place_spheres(radii, (-0.5 * length, -R, -R), (0.5 * length, R, -0.55 * R), cyl_radius=R,
                                seed=seed)
    if placed != n:
        raise ValueError(f"shell_drop: placed {placed} of {n}")
    radial = pos.copy()
    radial[:, 0] = 0.0
    out = radial / np.maximum(np.linalg.norm(radial, axis=1), 1e-12)[:, None]
    vel = speed * out + rng.normal(0.0, 0.05, size=pos.shape)
    thick = 1e-3
    behavior = ORBITAL if rpm else FIXED
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (radius,)),
              DOModel("Shell", "Wall", behavior, GLOBAL, 0.0, 1.0, INNER_CYLINDER, (R, length + 2 * thick)),
              DOModel("End", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (2.2 * R, thick, 2.2 * R))]
    zeta = damping_ratio(0.6)
    if solver == "ISwBSDBF":
        mech = lambda b: lsd_mechanisms(2e4, 1.6e4, b, b, 0.4)
        iacts = [IactModel("Ball", "Ball", solver, mech(zeta / math.sqrt(2.0))),
                 IactModel("Wall", "Ball", solver, mech(zeta))]
    else:
        m_of = lambda rr: 2500.0 * 4.0 / 3.0 * math.pi * rr ** 3
        iacts = [IactModel("Ball", "Ball", solver, _hertz_mech(solver, 70e9, 0.25, radius, radius, m_of, zeta, 0.4)),
                 IactModel("Wall", "Ball", solver, _hertz_mech(solver, 70e9, 0.25, radius, None, m_of, zeta, 0.4))]
    omega = rpm * 2.0 * math.pi / 60.0
    wp = [[0.0, 0.0, 0.0], [-0.5 * length - 0.5 * thick, 0.0, 0.0], [0.5 * length + 0.5 * thick, 0.0, 0.0]]
    wox = [[0.0, 1.0, 0.0], [0.0, 1.0, 0.0], [0.0, 1.0, 0.0]]
    woz = [[1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [-1.0, 0.0, 0.0]]
    wav = [[omega, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]
    midx = np.concatenate([np.zeros(n, np.uint32), np.array([1, 2, 2], np.uint32)])
    P = np.concatenate([pos, np.array(wp)])
    V = np.concatenate([vel, np.zeros((3, 3))])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array(wox)])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array(woz)])
    AV = np.concatenate([np.zeros((n, 3)), np.array(wav)])
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)


def shell_rest(R: float = 8e-3, radius: float = 1e-3, kn: float = 1e4, length: float = 12e-3) -> Scene:
    """One sphere resting on the bottom of a fixed horizontal hollow cylinder at the linear
    law's equilibrium depth (kn delta = m g, ISwBSDBF), and a second sphere pressed 1 um into the
    shell's side with the field off along its normal: the analytic checks of the inner-cylinder
    detector (depth, outward radial normal, force balance)."""
    m = 2500.0 * 4.0 / 3.0 * math.pi * radius ** 3
    delta = m * 9.81 / kn
    pos = np.array([[0.0, 0.0, -(R - radius + delta)], [2e-3, R - radius + 1e-6, 0.0]])
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (radius,)),
              DOModel("Shell", "Wall", FIXED, GLOBAL, 0.0, 1.0, INNER_CYLINDER, (R, length))]
    iacts = [IactModel("Ball", "Ball", "ISwBSDBF", lsd_mechanisms(kn, 0.8 * kn, 0.1, 0.1, 0.5)),
             IactModel("Wall", "Ball", "ISwBSDBF", lsd_mechanisms(kn, 0.8 * kn, 0.1, 0.1, 0.5))]
    midx = np.array([0, 0, 1], np.uint32)
    P = np.concatenate([pos, [[0.0, 0.0, 0.0]]])
    OX = np.array([[1.0, 0, 0], [1.0, 0, 0], [0.0, 1.0, 0.0]])
    OZ = np.array([[0, 0, 1.0], [0, 0, 1.0], [1.0, 0.0, 0.0]])
    return Scene(time_control(10, 1e-6), models, iacts, midx, P, np.zeros((3, 3)), OX, OZ, np.zeros((3, 3)))


def holed_plate_drop(n_side: int = 6, seed: int = 4, steps: int = 600, dt: float = 1e-6, radius: float = 1e-3,
                     hole: float = 2.6e-3, hole_offset: Tuple[float, float] = (1.2e-3, -0.7e-3),
                     solver: str = "ISwBSDBF") -> Scene:
    """Spheres on a jittered square grid moving down onto a fixed square plate with a circular
    hole (the reference's QuasiPlateWithCircularHole, offset from the plate's centre): some
    fall through the hole, some land on its rim, one moves straight down the hole's axis (the
    detector's zero-offset branch), the rest land on the flat part.  LSD (ISwBSDBF) for
    bit-exact comparisons by default."""
    rng = np.random.default_rng(seed)
    sp = 2.3 * radius
    side = 14 * radius
    xs = (np.arange(n_side) - 0.5 * (n_side - 1)) * sp
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), np.full(X.size, radius + 0.5e-3 + 5e-6)], 1)   # just above the plate
    pos[:, :2] += rng.uniform(-0.2 * radius, 0.2 * radius, size=(pos.shape[0], 2))
    pos[:, 2] += rng.uniform(0.0, 0.02 * radius, size=pos.shape[0])
    pos[0, :2] = hole_offset                              # exactly over the hole's centre
    n = pos.shape[0]
    kn, ks = 2e4, 1.6e4
    zeta = damping_ratio(0.6)
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (radius,)),
              DOModel("Holed", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE_WITH_CIRCULAR_HOLE,
                      (side, 1e-3, side, hole, hole_offset[0], hole_offset[1]))]
    if solver == "ISwBSDBF":
        mech = lambda b: lsd_mechanisms(kn, ks, b, b, 0.4)
        iacts = [IactModel("Ball", "Ball", solver, mech(zeta / math.sqrt(2.0))),
                 IactModel("Wall", "Ball", solver, mech(zeta))]
    else:
        m_of = lambda rr: 2500.0 * 4.0 / 3.0 * math.pi * rr ** 3
        iacts = [IactModel("Ball", "Ball", solver, _hertz_mech(solver, 70e9, 0.25, radius, radius, m_of, zeta, 0.4)),
                 IactModel("Wall", "Ball", solver, _hertz_mech(solver, 70e9, 0.25, radius, None, m_of, zeta, 0.4))]
    midx = np.concatenate([np.zeros(n, np.uint32), np.array([1], np.uint32)])
    P = np.concatenate([pos, np.zeros((1, 3))])
    V = np.concatenate([rng.normal(0.0, 0.02, size=(n, 3)) * np.array([1.0, 1.0, 0.0]), np.zeros((1, 3))])
    V[:n, 2] = -0.2
    V[0, :2] = 0.0
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array([[1.0, 0.0, 0.0]])])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array([[0.0, 0.0, 1.0]])])
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, np.zeros((n + 1, 3)))


def periodic_layer(nx: int = 4, ny: int = 4, layers: int = 3, seed: int = 6, steps: int = 400, dt: float = 1e-6,
                   radius: float = 1e-3, solver: str = "ISwBSDBF", periodic_y: bool = True,
                   drift: Tuple[float, float] = (3.0, -2.0), floor_spin: float = 0.0,
                   side_walls: bool = False, outside: bool = False) -> Scene:
    """Spheres tiling a box that is periodic in x (and y) on a floor plate, drifting across the
    periodic faces.  The lattice is placed so that the spheres of one column start 0.1 mm short
    of the upper x face (and one row 0.1 mm above the lower y face), so they wrap within the
    first few dozen steps, while a pair in contact is still a candidate (with no drift the
    lattice sits 1 mm clear of the faces instead).  The floor's centre is
    off the box centre (lever arms to it cross half a period); `floor_spin` makes it an orbital
    plate turning about its normal.  `side_walls` (with y not periodic) adds two fixed plates
    normal to y whose centres lie outside the box in x: the periodic wrap moves them after the
    first step, as it moves every object.  `outside` adds two spheres above the lattice placed
    more than one range beyond the box in x (the wrap's fmod branch brings them back)."""
    rng = np.random.default_rng(seed)
    sp = 2.05 * radius
    Lx, Ly = nx * sp, ny * sp
    h = 1e-3
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(layers), indexing="ij")
    ox0, oy0 = (0.95, 0.05) if drift[0] or drift[1] else (0.5, 0.5)     # no drift: 1 mm clear of the faces
    pos = np.stack([-0.5 * Lx + (i.ravel() + ox0) * sp, -0.5 * Ly + (j.ravel() + oy0) * sp,
                    radius + 5e-6 + k.ravel() * sp], 1)
    pos += rng.uniform(-0.01 * sp, 0.01 * sp, size=pos.shape) * np.array([1.0, 1.0, 0.0])
    if outside:
        ztop = radius + 5e-6 + (layers + 1) * sp
        pos = np.concatenate([pos, [[0.5 * Lx + 2.2 * Lx, 0.1 * Ly, ztop], [-0.5 * Lx - 3.4 * Lx, -0.2 * Ly, ztop]]])
    n = pos.shape[0]
    vel = rng.normal(0.0, 0.3, size=pos.shape)
    vel[:, 0] += drift[0]
    vel[:, 1] += drift[1] if periodic_y else 0.0
    avel = rng.normal(0.0, 20.0, size=pos.shape)
    floor_beh = ORBITAL if floor_spin else FIXED
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (radius,)),
              DOModel("Floor", "Wall", floor_beh, GLOBAL, 0.0, 1.0, QUASI_PLATE, (4 * Lx, h, 4 * Ly))]
    midx = [np.zeros(n, np.uint32), np.array([1], np.uint32)]
    P = [pos, np.array([[-0.3 * Lx, -0.3 * Ly if periodic_y else 0.0, -0.5 * h]])]
    OX, OZ = [np.tile([1.0, 0, 0], (n, 1)), np.array([[1.0, 0.0, 0.0]])], [np.tile([0, 0, 1.0], (n, 1)),
                                                                          np.array([[0.0, 0.0, 1.0]])]
    AV = [avel, np.array([[0.0, 0.0, floor_spin]])]
    if side_walls and not periodic_y:
        models.append(DOModel("Side", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (4 * Lx, h, 4 * layers * sp)))
        midx.append(np.array([2, 2], np.uint32))
        P.append(np.array([[0.75 * Lx, 0.5 * Ly + 0.5 * h, 2 * layers * sp],
                           [0.8 * Lx, -0.5 * Ly - 0.5 * h, 2 * layers * sp]]))
        OX.append(np.tile([1.0, 0.0, 0.0], (2, 1)))
        OZ.append(np.array([[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]]))
        AV.append(np.zeros((2, 3)))
    zeta = damping_ratio(0.7)
    iacts = [IactModel("Ball", "Ball", solver, _mechanisms(solver, zeta / math.sqrt(2.0), 0.5)),
             IactModel("Wall", "Ball", solver, _mechanisms(solver, zeta, 0.5))]
    P = np.concatenate(P)
    sc = Scene(time_control(steps, dt), models, iacts, np.concatenate(midx), P,
               np.concatenate([vel, np.zeros((P.shape[0] - n, 3))]), np.concatenate(OX), np.concatenate(OZ),
               np.concatenate(AV))
    sc.sp.pbc = Boundary(switch=(True, periodic_y, False), lower=(-0.5 * Lx, -0.5 * Ly if periodic_y else 0.0, 0.0),
                         upper=(0.5 * Lx, 0.5 * Ly if periodic_y else 0.0, 0.0))
    return sc


def touching_lattice(seed: int = 13, nx: int = 5, ny: int = 5, nz: int = 3, loose: int = 40) -> Scene:
    """Spheres at exactly touching distances, for the coordination number: a simple cubic lattice
    of r = 2^-11 m spheres at spacing 2^-10 m (every axis neighbour at exactly the radius sum),
    a few of them moved by +-2^-40 m along x (just overlapping or just apart), r = 2^-12 m
    spheres at exactly the radius sum from a lattice sphere (and overlapping its next neighbour),
    seeded loose spheres near the lattice, then a floor plate and a rod (walls are not counted).
    Every lattice coordinate is exact in binary, so the tests meet exact ties."""
    rng = np.random.default_rng(seed)
    ra, rb = 2.0 ** -11, 2.0 ** -12
    sp = 2.0 ** -10
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    A = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(float) * sp
    move = rng.choice(len(A), size=len(A) // 5, replace=False)
    A[move, 0] += rng.choice([-1.0, 1.0], size=len(move)) * 2.0 ** -40
    host = rng.choice(len(A), size=6, replace=False)
    B = A[host] + np.array([3.0 * 2.0 ** -12, 0.0, 0.0])
    L = rng.uniform(-0.5 * sp, np.array([nx, ny, nz]) * sp, size=(loose, 3))
    pos = np.concatenate([A, B, L])
    midx = np.concatenate([np.zeros(len(A), np.uint32), np.ones(len(B), np.uint32), np.zeros(loose, np.uint32)])
    n = len(pos)
    models = [DOModel("BallA", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (ra,)),
              DOModel("BallB", "Ball", MOBILE, LOCAL, 2500.0, 1.0, SPHERE, (rb,)),
              DOModel("Floor", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (0.02, 1e-3, 0.02)),
              DOModel("Rod", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_CYLINDER, (1e-3, 0.01))]
    P = np.concatenate([pos, [[0.002, 0.002, -ra - 0.5e-3], [0.009, 0.002, 0.002]]])
    midx = np.concatenate([midx, np.array([2, 3], np.uint32)])
    V = np.concatenate([rng.normal(0.0, 0.1, size=(n, 3)), np.zeros((2, 3))])
    AV = np.concatenate([rng.normal(0.0, 5.0, size=(n, 3)), np.zeros((2, 3))])
    OX = np.tile([1.0, 0.0, 0.0], (n + 2, 1))
    OZ = np.tile([0.0, 0.0, 1.0], (n + 2, 1))
    zeta = damping_ratio(0.7)
    iacts = [IactModel("Ball", "Ball", "ISwBSDBF", lsd_mechanisms(1e4, 8e3, zeta, zeta, 0.5)),
             IactModel("Wall", "Ball", "ISwBSDBF", lsd_mechanisms(1e4, 8e3, zeta, zeta, 0.5))]
    return Scene(time_control(100, 1e-6), models, iacts, midx, P, V, OX, OZ, AV)


def hopper_params(num_scenes: int = 256, seed: int = 2025, n_lo: int = 1000, n_hi: int = 50000):
    """Per-scene draws of the hopper batch: (n, seed, friction, restitution, orifice)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), num_scenes)).astype(np.int64)
    mu = rng.uniform(0.2, 0.6, num_scenes)
    e = rng.uniform(0.5, 0.9, num_scenes)
    w = rng.uniform(6e-3, 12e-3, num_scenes)
    seeds = rng.integers(0, 2**31 - 1, num_scenes)
    return [(int(n[k]), int(seeds[k]), float(mu[k]), float(e[k]), float(w[k])) for k in range(num_scenes)]


def hopper_batch(num_scenes: int = 256, seed: int = 2025, steps: int = 5000, n_lo: int = 1000,
                 n_hi: int = 50000, touching: bool = True) -> List[Scene]:
    """The batched hopper workload: `num_scenes` independent hoppers of uneven sizes (touching
    fills by default: the column rests on the floor and drains through the orifice)."""
    return [hopper(n=n, seed=sd, friction=mu, restitution=e, orifice=w, steps=steps, touching=touching)
            for n, sd, mu, e, w in hopper_params(num_scenes, seed, n_lo, n_hi)]


def serving_job(kind: str, n: int, model: str, seed: int, steps: int = 1000, K: int = 8,
                median_r: float = 1e-3, sigma_log: float = 0.15, dt: float = 1e-6) -> Scene:
    """A job of the serving stream.

    kind 'settle': n spheres on a jittered lattice (spacing 2.2 r_max) fall into an open box
    of 5 fixed plates with velocities N(0, 0.05 m/s).  kind 'projectile': the same lattice
    rests just above the floor and one sphere of radius 3 mm, 1 m/s downwards, hits its
    centre.  Radii are lognormal(median_r, sigma_log) clipped to [0.6, 1.6] mm and binned
    into K classes, one DOModel per class.  model 'lsd': ``ISwBSDBF`` with kn = 1e4 N/m,
    ks = 0.8 kn, restitution 0.8, friction 0.5; 'hertz': ``ISwH`` with E = 0.5 GPa, nu = 0.3,
    restitution 0.7, friction 0.4 (a stiffness for which dt = 1e-6 s is about 0.13 of the
    smallest sphere's Rayleigh time)."""
    rng = np.random.default_rng(seed)
    edges = np.exp(np.linspace(math.log(0.6e-3), math.log(1.6e-3), K + 1))
    centres = np.sqrt(edges[:-1] * edges[1:])
    r = np.clip(median_r * np.exp(sigma_log * rng.standard_normal(n)), edges[0], edges[-1] * (1 - 1e-12))
    cls = np.clip(np.searchsorted(edges, r, side="right") - 1, 0, K - 1).astype(np.uint32)
    rmax = float(centres[cls].max())
    a = 2.2 * rmax
    m = max(2, int(math.ceil((n / 2.0) ** (1.0 / 3.0))))
    nz = int(math.ceil(n / (m * m)))
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = np.empty((n, 3))
    pos[:, 0] = (g[:, 0] - 0.5 * (m - 1)) * a
    pos[:, 1] = (g[:, 1] - 0.5 * (m - 1)) * a
    pos[:, 2] = g[:, 2] * a + 1.05 * rmax
    pos += rng.uniform(-0.02 * rmax, 0.02 * rmax, size=pos.shape)
    vel = rng.normal(0.0, 0.05, size=pos.shape) if kind == "settle" else np.zeros((n, 3))
    width = m * a + 4.0 * rmax
    density = 2500.0
    models = [DOModel(f"B{k}", f"B{k}", MOBILE, LOCAL, density, 1.0, SPHERE, (float(centres[k]),)) for k in range(K)]
    groups = [f"B{k}" for k in range(K)]
    P, V, midx = [pos], [vel], [cls]
    if kind == "projectile":
        rp = 3e-3
        models.append(DOModel("Proj", "Proj", MOBILE, LOCAL, density, 1.0, SPHERE, (rp,)))
        groups.append("Proj")
        P.append(np.array([[0.0, 0.0, nz * a + rmax + rp + 2e-4]]))
        V.append(np.array([[0.0, 0.0, -1.0]]))
        midx.append(np.array([K], np.uint32))
    base = len(models)
    wm, widx, wp, wox, woz = box_walls(width, nz * a + 12e-3, 1e-3)
    models += wm
    nball = sum(len(x) for x in P)
    midx = np.concatenate(midx + [base + np.array(widx, np.uint32)])
    P = np.concatenate(P + [wp])
    V = np.concatenate(V + [np.zeros_like(wp)])
    nt = len(midx)
    OX = np.concatenate([np.tile([1.0, 0, 0], (nball, 1)), wox])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (nball, 1)), woz])
    AV = np.zeros((nt, 3))
    radius_of = {gname: float(models[k].attrs[0]) for k, gname in enumerate(groups)}
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = []
    if model == "lsd":
        zeta = damping_ratio(0.8)
        mech = lambda wall: lsd_mechanisms(1e4, 8e3, zeta if wall else zeta / math.sqrt(2.0),
                                           zeta if wall else zeta / math.sqrt(2.0), 0.5)
        for i, ga in enumerate(groups):
            for gb in groups[i:]:
                iacts.append(IactModel(ga, gb, "ISwBSDBF", mech(False)))
        for gb in groups:
            iacts.append(IactModel("Wall", gb, "ISwBSDBF", mech(True)))
    else:
        zeta = damping_ratio(0.7)
        for i, ga in enumerate(groups):
            for gb in groups[i:]:
                iacts.append(IactModel(ga, gb, "ISwH", _hertz_mech("ISwH", 0.5e9, 0.3, radius_of[ga], radius_of[gb],
                                                                    m_of, zeta, 0.4)))
        for gb in groups:
            iacts.append(IactModel("Wall", gb, "ISwH", _hertz_mech("ISwH", 0.5e9, 0.3, radius_of[gb], None, m_of,
                                                                    zeta, 0.4)))
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)


def compressed_bed(n: int = 16_000_000, seed: int = 5, steps: int = 2000, dt: float = 2e-7, radius: float = 5e-4,
                   box: float = 0.4, E: float = 10e9, nu: float = 0.25, restitution: float = 0.7,
                   friction: float = 0.5, density: float = 2500.0, solid_fraction: float = 0.55,
                   cylinders: int = 32, cyl_radius: float = 5e-3, plate_speed: float = 0.05,
                   packing: str = "touching") -> Scene:
    """A bed of n spheres filling a `box` x `box` floor to the height that holds n, with
    `cylinders` fixed vertical rods on a jittered grid (spheres that would overlap a rod are not
    placed) and an orbital top plate moving at (0, 0, -plate_speed).  Walls: floor and four
    sides (fixed plates).  Contact ``ISwH`` (Hertz normal stiffness with friction) for
    sphere-sphere, sphere-plate and sphere-rod.

    packing="touching" (the default): a simple cubic lattice whose neighbours, floor, sides and
    top plate touch exactly (solid fraction pi/6 = 0.524), so the bed carries its contacts from
    the first step; it stands in for a random loose packing at 0.55, which only a long settle
    of all n spheres would give.  packing="fcc": a jittered face-centred cubic lattice at
    `solid_fraction` (at 0.55 the nearest-neighbour gap is 0.2 r: nothing touches) with the
    plate 10 um above it."""
    if packing == "touching":
        return _touching_bed(n, seed, steps, dt, radius, box, E, nu, restitution, friction, density, cylinders,
                             cyl_radius, plate_speed)
    rng = np.random.default_rng(seed)
    vs = 4.0 / 3.0 * math.pi * radius ** 3
    a = (4.0 * vs / solid_fraction) ** (1.0 / 3.0)          # FCC cell edge (4 spheres per cell)
    c = 1.1 * radius                                       # centre-to-wall distance of the outermost spheres
    m = int((box - 2.0 * c) / a + 0.5)                     # cells across the box
    inner = (m - 0.5) * a + 2.0 * c                        # lattice points span (m - 1/2) a
    # rods on a jittered grid
    g = int(math.ceil(math.sqrt(cylinders)))
    rods = []
    for k in range(cylinders):
        gx, gy = k % g, k // g
        cx = (gx + 0.5) / g * inner - 0.5 * inner + rng.uniform(-0.2, 0.2) * inner / g
        cy = (gy + 0.5) / g * inner - 0.5 * inner + rng.uniform(-0.2, 0.2) * inner / g
        rods.append((cx, cy))
    rods = np.array(rods)
    basis = np.array([[0.25, 0.25, 0.25], [0.75, 0.75, 0.25], [0.75, 0.25, 0.75], [0.25, 0.75, 0.75]]) * a
    layer = np.stack(np.meshgrid(np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 2) * a
    per_cell_layer = (layer[:, None, :] + basis[None, :, :2]).reshape(-1, 2) - 0.25 * a + c - 0.5 * inner
    zoff = np.tile(basis[:, 2], len(layer)) - 0.25 * a + c
    keep = np.ones(len(per_cell_layer), bool)
    for cx, cy in rods:
        d2 = (per_cell_layer[:, 0] - cx) ** 2 + (per_cell_layer[:, 1] - cy) ** 2
        keep &= d2 > (cyl_radius + radius * 1.2) ** 2
    xy = per_cell_layer[keep]
    zo = zoff[keep]
    per_layer = len(xy)
    nl = int(math.ceil(n / per_layer))
    pos = np.empty((nl * per_layer, 3))
    for L in range(nl):
        pos[L * per_layer:(L + 1) * per_layer, :2] = xy
        pos[L * per_layer:(L + 1) * per_layer, 2] = zo + L * a
    pos = pos[:n]
    pos += rng.uniform(-0.05 * radius, 0.05 * radius, size=pos.shape)
    top = float(pos[:, 2].max()) + radius
    height = top + 0.02
    t = 2e-3
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,)),
              DOModel("Floor", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (inner + 2 * t, t, inner + 2 * t)),
              DOModel("Side", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (height, t, inner + 2 * t)),
              DOModel("Rod", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_CYLINDER, (cyl_radius, height)),
              DOModel("Top", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, QUASI_PLATE, (inner, t, inner))]
    wp, wox, woz, wv, widx = [(0.0, 0.0, -0.5 * t)], [(1.0, 0.0, 0.0)], [(0.0, 0.0, 1.0)], [(0.0, 0.0, 0.0)], [1]
    for sx, sy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        wp.append((sx * (0.5 * inner + 0.5 * t), sy * (0.5 * inner + 0.5 * t), 0.5 * height))
        wox.append((0.0, 0.0, 1.0)); woz.append((-float(sx), -float(sy), 0.0)); wv.append((0.0, 0.0, 0.0)); widx.append(2)
    for cx, cy in rods:
        wp.append((cx, cy, 0.5 * height)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, 1.0))
        wv.append((0.0, 0.0, 0.0)); widx.append(3)
    wp.append((0.0, 0.0, top + 1e-5 + 0.5 * t)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, -1.0))
    wv.append((0.0, 0.0, -plate_speed)); widx.append(4)
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = [IactModel("Ball", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, radius, m_of, zeta, friction)),
             IactModel("Wall", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, None, m_of, zeta, friction))]
    k = len(widx)
    midx = np.concatenate([np.zeros(n, np.uint32), np.array(widx, np.uint32)])
    P = np.concatenate([pos, np.array(wp)])
    V = np.concatenate([np.zeros((n, 3)), np.array(wv)])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array(wox)])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array(woz)])
    AV = np.zeros((n + k, 3))
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)


def _touching_bed(n, seed, steps, dt, radius, box, E, nu, restitution, friction, density, cylinders, cyl_radius,
                  plate_speed) -> Scene:
    rng = np.random.default_rng(seed)
    a = 2.0 * radius
    m = int(box / a)                                       # spheres across
    inner = m * a                                          # the side walls touch the outer spheres
    g = int(math.ceil(math.sqrt(cylinders)))
    rods = []
    for k in range(cylinders):
        gx, gy = k % g, k // g
        cx = (gx + 0.5) / g * inner - 0.5 * inner + rng.uniform(-0.2, 0.2) * inner / g
        cy = (gy + 0.5) / g * inner - 0.5 * inner + rng.uniform(-0.2, 0.2) * inner / g
        rods.append((cx, cy))
    xs = (np.arange(m) + 0.5) * a - 0.5 * inner
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    xy = np.stack([X.ravel(), Y.ravel()], 1)
    keep = np.ones(len(xy), bool)
    for cx, cy in rods:
        keep &= (xy[:, 0] - cx) ** 2 + (xy[:, 1] - cy) ** 2 > (cyl_radius + radius * 1.001) ** 2
    xy = xy[keep]
    per_layer = len(xy)
    nl = int(math.ceil(n / per_layer))
    pos = np.empty((nl * per_layer, 3))
    for L in range(nl):
        pos[L * per_layer:(L + 1) * per_layer, :2] = xy
        pos[L * per_layer:(L + 1) * per_layer, 2] = radius + L * a
    pos = pos[:n]
    top = float(pos[:, 2].max()) + radius
    height = top + 0.02
    t = 2e-3
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,)),
              DOModel("Floor", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (inner + 2 * t, t, inner + 2 * t)),
              DOModel("Side", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_PLATE, (height, t, inner + 2 * t)),
              DOModel("Rod", "Wall", FIXED, GLOBAL, 0.0, 1.0, QUASI_CYLINDER, (cyl_radius, height)),
              DOModel("Top", "Wall", ORBITAL, GLOBAL, 0.0, 1.0, QUASI_PLATE, (inner, t, inner))]
    wp, wox, woz, wv, widx = [(0.0, 0.0, -0.5 * t)], [(1.0, 0.0, 0.0)], [(0.0, 0.0, 1.0)], [(0.0, 0.0, 0.0)], [1]
    for sx, sy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        wp.append((sx * (0.5 * inner + 0.5 * t), sy * (0.5 * inner + 0.5 * t), 0.5 * height))
        wox.append((0.0, 0.0, 1.0)); woz.append((-float(sx), -float(sy), 0.0)); wv.append((0.0, 0.0, 0.0)); widx.append(2)
    for cx, cy in rods:
        wp.append((cx, cy, 0.5 * height)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, 1.0))
        wv.append((0.0, 0.0, 0.0)); widx.append(3)
    wp.append((0.0, 0.0, top + 0.5 * t)); wox.append((1.0, 0.0, 0.0)); woz.append((0.0, 0.0, -1.0))
    wv.append((0.0, 0.0, -plate_speed)); widx.append(4)
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = [IactModel("Ball", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, radius, m_of, zeta, friction)),
             IactModel("Wall", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, None, m_of, zeta, friction))]
    k = len(widx)
    midx = np.concatenate([np.zeros(n, np.uint32), np.array(widx, np.uint32)])
    P = np.concatenate([pos, np.array(wp)])
    V = np.concatenate([np.zeros((n, 3)), np.array(wv)])
    OX = np.concatenate([np.tile([1.0, 0, 0], (n, 1)), np.array(wox)])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (n, 1)), np.array(woz)])
    AV = np.zeros((n + k, 3))
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)


def dense_pack(n: int = 1_000_000, seed: int = 9, steps: int = 1000, dt: float = 5e-7, radius: float = 1e-3,
               overlap: float = 1e-6, E: float = 70e9, nu: float = 0.25, restitution: float = 0.7,
               friction: float = 0.4, density: float = 2500.0) -> Scene:
    """n spheres on a face-centred cubic lattice (a cube of cells) whose nearest neighbours
    overlap by `overlap` x 2r, so every sphere has up to 12 contacts from the first step: the
    contact path of every kernel runs for every pair.  The lattice sits on the floor of an open
    box of fixed plates that touch its outer spheres; ISwH with Hertz stiffness from E and nu,
    restitution and friction; small seeded velocities N(0, 1 mm/s)."""
    rng = np.random.default_rng(seed)
    d = 2.0 * radius * (1.0 - overlap)              # nearest-neighbour distance
    a = d * math.sqrt(2.0)                          # FCC cell edge
    m = max(1, int(math.ceil((n / 4.0) ** (1.0 / 3.0))))
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]]) * a
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3) * a
    pos = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    pos = pos[np.lexsort((pos[:, 0], pos[:, 1], pos[:, 2]))][:n]   # fill from the bottom layer up
    lo = pos.min(0) - radius
    hi = pos.max(0) + radius
    ctr = 0.5 * (lo + hi)
    pos = pos - np.array([ctr[0], ctr[1], lo[2]])
    vel = rng.normal(0.0, 1e-3, size=pos.shape)
    half = 0.5 * (hi - lo)
    width = 2.0 * float(max(half[0], half[1]))
    height = float(hi[2] - lo[2]) + 4.0 * radius
    wm, widx, wp, wox, woz = box_walls(width, height, 1e-3)
    models = [DOModel("Ball", "Ball", MOBILE, LOCAL, density, 1.0, SPHERE, (radius,))] + wm
    zeta = damping_ratio(restitution)
    m_of = lambda rr: density * 4.0 / 3.0 * math.pi * rr ** 3
    iacts = [IactModel("Ball", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, radius, m_of, zeta, friction)),
             IactModel("Wall", "Ball", "ISwH", _hertz_mech("ISwH", E, nu, radius, None, m_of, zeta, friction))]
    k = len(widx)
    nn = len(pos)
    midx = np.concatenate([np.zeros(nn, np.uint32), 1 + np.array(widx, np.uint32)])
    P = np.concatenate([pos, wp])
    V = np.concatenate([vel, np.zeros((k, 3))])
    OX = np.concatenate([np.tile([1.0, 0, 0], (nn, 1)), wox])
    OZ = np.concatenate([np.tile([0, 0, 1.0], (nn, 1)), woz])
    AV = np.zeros((nn + k, 3))
    return Scene(time_control(steps, dt), models, iacts, midx, P, V, OX, OZ, AV)
