"""Seeded synthetic initial conditions (the benchmark configurations).

The reference reads initial data from its plugin's QInit2D/QInit3D
(CH/problem.f90:45-146); the benchmark configurations instead draw
U(-1,1) per cell from splitmix64 on the cell's global index, so a field does
not depend on how the mesh is cut into patches:

    u   = splitmix64(seed ^ (gidx * 0x9E3779B97F4A7C15))
    U   = 2 * ((u >> 11) * 2**-53) - 1
    gidx = ((k-1)*M2 + (j-1))*M1 + (i-1)   on the level's global frame.

The chemical potential is mu0 = phi0^3 - phi0 - eps^2 * Lap_h(phi0), the
value that makes the initial state consistent with the CH operator
(Operator2D/3D, CH/problem.f90:393-422).
"""
import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)


def splitmix_pm1(seed, gidx):
    """U(-1,1) from splitmix64(seed ^ gidx * golden); vectorised over gidx."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) ^ (np.asarray(gidx).astype(np.uint64) * _GOLD)
        z = z + _GOLD
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return 2.0 * ((z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)) - 1.0


def global_index(shape):
    """gidx of every cell of a full level (Fortran index order i fastest)."""
    if len(shape) == 2:
        i, j = np.meshgrid(np.arange(shape[0], dtype=np.uint64), np.arange(shape[1], dtype=np.uint64),
                           indexing="ij")
        return j * np.uint64(shape[0]) + i
    i, j, k = np.meshgrid(*[np.arange(n, dtype=np.uint64) for n in shape], indexing="ij")
    return (k * np.uint64(shape[1]) + j) * np.uint64(shape[0]) + i


def periodic_lap(a, h):
    out = -2.0 * a.ndim * a
    for ax in range(a.ndim):
        out = out + np.roll(a, 1, ax) + np.roll(a, -1, ax)
    return out / (h * h)


def ch_spinodal(shape, eps, h, seed, mean=0.0, amp=0.05):
    """phi0 = mean + amp*U(-1,1), mu0 from phi0 (the Laplacian wrapped over
    the array; products in the order written, as the device generator
    bsamg_seed_spinodal forms them); returns the ghosted q array (Fortran
    order, shape (mx+2, ..., 2)) with zero ghosts."""
    phi = mean + amp * splitmix_pm1(seed, global_index(shape))
    mu = phi * phi * phi - phi - eps * eps * periodic_lap(phi, h)
    q = np.zeros(tuple(n + 2 for n in shape) + (2,), order="F")
    sl = tuple(slice(1, -1) for _ in shape)
    q[sl + (0,)] = phi
    q[sl + (1,)] = mu
    return q


def ch_circle(shape, eps, h, seed, radius=0.25, noise=0.01, center=None):
    """phi0 = tanh((r - radius)/(sqrt(2) eps)) + noise*U(-1,1) around the
    domain centre, mu0 from phi0 (non-periodic Laplacian with reflected
    edges); ghosted q array as in ch_spinodal."""
    nd = len(shape)
    center = center if center is not None else [0.5 * n * h for n in shape]
    coords = np.meshgrid(*[(np.arange(n) + 0.5) * h for n in shape], indexing="ij")
    r = np.sqrt(sum((c - c0) ** 2 for c, c0 in zip(coords, center)))
    phi = np.tanh((r - radius) / (np.sqrt(2.0) * eps)) + noise * splitmix_pm1(seed, global_index(shape))
    pad = np.pad(phi, 1, mode="edge")
    lap = -2.0 * nd * phi
    for ax in range(nd):
        sl_p = [slice(1, -1)] * nd
        sl_m = [slice(1, -1)] * nd
        sl_p[ax] = slice(2, None)
        sl_m[ax] = slice(0, -2)
        lap = lap + pad[tuple(sl_p)] + pad[tuple(sl_m)]
    mu = phi ** 3 - phi - eps * eps * lap / (h * h)
    q = np.zeros(tuple(n + 2 for n in shape) + (2,), order="F")
    sl = tuple(slice(1, -1) for _ in shape)
    q[sl + (0,)] = phi
    q[sl + (1,)] = mu
    return q


def ch_circle_patch(eps, seed, radius=0.25, noise=0.01, center=(0.5, 0.5, 0.5), length=1.0):
    """Initial condition of a patch of any level (a QInit for the regrid):
    phi0 = tanh((r - radius)/(sqrt(2) eps)) + noise*U(-1,1), U from splitmix64
    on the cell's global index on its level (so every level sees the same
    field whatever the patching), mu0 = 0 as the CH plugin's QInit2D/3D
    (CH/problem.f90:60-61).  Returns fn(level, mx, dx, xlower) -> ghosted
    Fortran-layout array."""
    def fn(level, mx, dx, xl):
        nd = len(mx)
        nglob = [int(round(length / dx[d])) for d in range(nd)]
        i0 = [int(round(xl[d] / dx[d])) for d in range(nd)]
        ax = [(np.arange(mx[d]) + 0.5) * dx[d] + xl[d] for d in range(nd)]
        coords = np.meshgrid(*ax, indexing="ij")
        r = np.sqrt(sum((c - center[d]) ** 2 for d, c in enumerate(coords)))
        idx = np.meshgrid(*[np.arange(mx[d], dtype=np.uint64) + np.uint64(i0[d]) for d in range(nd)], indexing="ij")
        g = idx[0]
        stride = np.uint64(1)
        for d in range(1, nd):
            stride = stride * np.uint64(nglob[d - 1])
            g = g + idx[d] * stride
        phi = np.tanh((r - radius) / (np.sqrt(2.0) * eps)) + noise * splitmix_pm1(seed, g)
        q = np.zeros(tuple(m + 2 for m in mx) + (2,), order="F")
        q[tuple(slice(1, -1) for _ in mx) + (0,)] = phi
        return q
    return fn


def growth_sphere(eps, seed, radius=0.1, noise=0.02, center=(0.5, 0.5, 0.5), length=1.0):
    """Initial condition of the three-variable growth plugin on a patch of
    any level: phi = tanh((r0 - r)/(sqrt(2) eps)) with r0 = radius +
    noise*U(-1,1) per cell (U from splitmix64 on the cell's global index on
    its level), nutrient n = 1, pressure p = 0.  Returns fn(level, mx, dx,
    xlower) -> ghosted Fortran-layout array with three variables."""
    def fn(level, mx, dx, xl):
        nd = len(mx)
        nglob = [int(round(length / dx[d])) for d in range(nd)]
        i0 = [int(round(xl[d] / dx[d])) for d in range(nd)]
        ax = [(np.arange(mx[d]) + 0.5) * dx[d] + xl[d] for d in range(nd)]
        coords = np.meshgrid(*ax, indexing="ij")
        r = np.sqrt(sum((c - center[d]) ** 2 for d, c in enumerate(coords)))
        idx = np.meshgrid(*[np.arange(mx[d], dtype=np.uint64) + np.uint64(i0[d]) for d in range(nd)], indexing="ij")
        g = idx[0]
        stride = np.uint64(1)
        for d in range(1, nd):
            stride = stride * np.uint64(nglob[d - 1])
            g = g + idx[d] * stride
        r0 = radius + noise * splitmix_pm1(seed, g)
        q = np.zeros(tuple(m + 2 for m in mx) + (3,), order="F")
        inner = tuple(slice(1, -1) for _ in mx)
        q[inner + (0,)] = np.tanh((r0 - r) / (np.sqrt(2.0) * eps))
        q[inner + (1,)] = 1.0
        return q
    return fn
