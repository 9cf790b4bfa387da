"""Seeded synthetic foams with the shapes of the benchmark configurations.

No public dataset is involved: every foam is generated from a seed with
numpy's PCG64 generator (`numpy.random.default_rng`), which is stable across
platforms. Positions are uniform in a box whose side makes the gas fraction
equal phi (2D: L = sqrt(pi sum r^2 / phi), 3D: L = cbrt(4/3 pi sum r^3 / phi)),
radii are Normal(mean, std) clipped to [lo, hi].

Derived constants follow the reference's init() (src/simulator.cu:538-575,
:713-717, :820-826):
    skin = 0.3 <r>,  f0/mu0 = sigma <r> / mu,  <A_in> = mean initial area,
    M = sqrt(phi V / pi) (2D) or cbrt(3/4 phi V / pi) (3D).
"""
import math

import numpy as np

from .foam import make_config


def foam(n, dim, phi, rmean=1.0, rstd=0.1, rclip=(0.3, 2.0), seed=1,
         kappa=0.01, k_param=0.1, mu=1.0, sigma=1.0, tol=1e-5,
         min_rad=None, wall=(0, 0, 0), time_step=1e-4, capacity=None,
         precision=0, use_graph=0, pair_capacity=0, **extra):
    """Returns (config, state) for one foam."""
    rng = np.random.default_rng(seed)
    r = np.clip(rng.normal(rmean, rstd, n), rclip[0], rclip[1])
    if dim == 3:
        side = (4.0 / 3.0 * math.pi * float(np.sum(r ** 3)) / phi) ** (1.0 / 3.0)
    else:
        side = math.sqrt(math.pi * float(np.sum(r ** 2)) / phi)
    x = rng.uniform(0.0, side, n)
    y = rng.uniform(0.0, side, n)
    z = rng.uniform(0.0, side, n) if dim == 3 else np.zeros(n)
    tfr = (side, side, side if dim == 3 else 0.0)
    volume = side ** dim
    if dim == 3:
        area = 4.0 * math.pi * r ** 2
        mult = (0.75 * phi * volume / math.pi) ** (1.0 / 3.0)
    else:
        area = 2.0 * math.pi * r
        mult = math.sqrt(phi * volume / math.pi)
    cfg = make_config(
        dimensionality=dim, wall=wall, lbb=(0.0, 0.0, 0.0), tfr=tfr,
        min_rad=(0.1 * rmean if min_rad is None else min_rad),
        f0_per_mu0=float(np.float32(sigma)) * rmean / mu,
        k_parameter=k_param, kappa=kappa, skin_radius=0.3 * rmean,
        bubble_volume_multiplier=mult,
        average_surface_area_in=float(np.mean(area)),
        error_tolerance=tol, time_step=time_step,
        capacity=capacity or n, pair_capacity=pair_capacity,
        precision=precision, use_graph=use_graph, **extra)
    state = {"x": x, "y": y, "z": z, "r": r,
             "index": np.arange(n, dtype=np.int32)}
    return cfg, state


def config_c1(seed=1, **kw):
    """2D periodic, N=10,000, phi=0.90, r~N(1,0.1) in [0.3,2.0],
    kappa=0.01, K=0.1, mu=1, no flow, tol 1e-5, min_rad 0.05."""
    return foam(10000, 2, 0.90, 1.0, 0.1, (0.3, 2.0), seed=seed,
                kappa=0.01, k_param=0.1, min_rad=0.05, **kw)


def config_c2(seed=2, n=1_000_000, **kw):
    """3D periodic, N=1e6, phi=0.80, r~N(1,0.15) in [0.3,2.5],
    kappa=0.01, K=0.1, tol 1e-5."""
    return foam(n, 3, 0.80, 1.0, 0.15, (0.3, 2.5), seed=seed,
                kappa=0.01, k_param=0.1, **kw)


def config_c5(seed=5, n=10_000_000, precision=1, **kw):
    """3D, walls in z (drag 0.1), periodic x / y, linear shear along x with
    maximum speed 0.05 at the walls, N=1e7, phi=0.80, r~N(1,0.15) in
    [0.3,2.5], kappa=0.01, K=0.1, tol 1e-5, mixed precision."""
    return foam(n, 3, 0.80, 1.0, 0.15, (0.3, 2.5), seed=seed, kappa=0.01, k_param=0.1,
                wall=(0, 0, 1), wall_drag=0.1, use_flow=1, shear_speed=0.05,
                precision=precision, **kw)


def prepare(sim):
    """Initial neighbour search and the Euler bootstrap of the AB2 history,
    the part of init() between the first search and stabilisation
    (src/simulator.cu:720-787)."""
    sim.search_neighbors()
    sim.bootstrap()


def sweep(count=256, seed=4, n_range=(1_000, 100_000), phi_range=(0.85, 0.95),
          kappa_range=(1e-3, 1e-1), **kw):
    """The batched parameter sweep: `count` independent 2D periodic foams,
    N log-uniform in n_range, phi uniform in phi_range, kappa log-uniform in
    kappa_range, r ~ N(1, 0.1) clipped to [0.3, 2.0], K=0.1, tol 1e-5,
    min_rad 0.05. Returns a list of (config, state), one per foam, each
    foam from its own seed."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    out = []
    for f in range(count):
        n = int(round(math.exp(rng.uniform(lo, hi))))
        phi = float(rng.uniform(*phi_range))
        kappa = float(math.exp(rng.uniform(math.log(kappa_range[0]),
                                           math.log(kappa_range[1]))))
        out.append(foam(n, 2, phi, 1.0, 0.1, (0.3, 2.0), seed=seed * 100003 + f,
                        kappa=kappa, k_param=0.1, min_rad=0.05, **kw))
    return out


def sweep_config_as(cfg, **changes):
    """A copy of a config with some fields changed (e.g. the precision)."""
    import copy
    c = copy.copy(cfg)
    for k, v in changes.items():
        setattr(c, k, v)
    return c
