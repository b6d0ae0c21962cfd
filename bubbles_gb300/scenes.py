"""Synthetic dam-break scenes of the benchmark configurations.

There is no public dataset for this path: every configuration is a seeded cubic
lattice of fluid in the (-x, -y, -z) corner of a container box centred at the origin
(the reference builds containers with MakeBox(Transform(), size, true) and the grid
with UtilBuildGridForDomain(container bounds, spacing, 2.0)).  Each particle gets a
uniform jitter of +-0.1 spacing per axis from numpy's PCG64 with the given seed and
zero initial velocity.

Mass follows the reference recipe m = rho0 / max_i sum_j W_std(|x_i - x_j|)
(SphParticleSet3::ComputeMass, src/core/particle.h:557-582) evaluated on the simple
cubic lattice that is actually seeded; the reference's BCC-calibrated mass would
start a cubic lattice at about 57 % of the rest density.
"""
import math

import numpy as np

PI = 3.14159265358979323846


def cubic_mass(density, spacing, kernel_radius):
    """rho0 / (number density of an interior point of a simple cubic lattice), FP64."""
    h = kernel_radius
    c = 315.0 / (64.0 * PI * h ** 3)
    m = int(math.ceil(h / spacing)) + 1
    total = 0.0
    for i in range(-m, m + 1):
        for j in range(-m, m + 1):
            for k in range(-m, m + 1):
                r2 = (i * i + j * j + k * k) * spacing * spacing
                if r2 < h * h:
                    x = 1.0 - r2 / (h * h)
                    total += c * x * x * x
    return density / total


def base_scene(solver, spacing, box, gravity=-9.81):
    box = np.asarray(box, np.float64)
    return {
        "solver": solver,
        "spacing": float(spacing),
        "target_density": 1000.0,
        "relative_kernel_radius": 2.0,
        "grid_spacing_scale": 2.0,
        "gravity": (0.0, float(gravity), 0.0),
        "eos_exponent": 7.0,
        "negative_pressure_scale": 0.0,
        "viscosity": 0.04,
        "pseudo_viscosity": 10.0,
        "sound_speed": 100.0,
        "drag_coefficient": 1e-4,
        "time_step_limit_scale": 5.0 if solver == "pcisph" else 1.0,
        "domain_min": tuple(-box / 2),
        "domain_max": tuple(box / 2),
        "colliders": [{"type": "box", "size": tuple(box), "center": (0.0, 0.0, 0.0),
                       "reverse": True}],
        "mass": cubic_mass(1000.0, spacing, 2.0 * spacing),
    }


def dam_block(scene, counts, seed, jitter=0.1):
    """Cubic lattice block of counts=(nx, ny, nz) particles at the container's min corner."""
    s = scene["spacing"]
    lo = np.asarray(scene["domain_min"], np.float64) + s
    nx, ny, nz = counts
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # x fastest, then y, then z (the order ParticleSetBuilder3 receives particles in)
    grid = np.stack([ix.transpose(2, 1, 0).ravel(), iy.transpose(2, 1, 0).ravel(),
                     iz.transpose(2, 1, 0).ravel()], axis=1).astype(np.float64)
    pos = lo + grid * s
    rng = np.random.default_rng(seed)
    pos += rng.uniform(-jitter * s, jitter * s, size=pos.shape)
    return pos


def place_spheres(rng, count, rmin, rmax, box, block_hi, margin):
    """Non-overlapping static spheres inside the box, clear of the fluid block."""
    half = np.asarray(box, np.float64) / 2
    out = []
    tries = 0
    while len(out) < count and tries < 100000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(-half + r + margin, half - r - margin)
        if np.all(c - r < block_hi + margin):
            continue   # overlaps the fluid block's bounding box
        if any(np.linalg.norm(c - o["center"]) < r + o["radius"] + margin for o in out):
            continue
        out.append({"type": "sphere", "center": c, "radius": float(r)})
    for o in out:
        o["center"] = tuple(float(x) for x in o["center"])
    return out


# name -> builder(seed) returning (scene, positions)
def sph_16k(seed=0, positions=True):
    """Plain 3D SPH dam break: 32 x 16 x 32 particles at h0 = 0.02 in a unit box, dt 1e-3."""
    sc = base_scene("sph", 0.02, (1.0, 1.0, 1.0))
    sc.update(dt=1e-3, steps=200, workload="SPH dam break 16,384 particles (32x16x32 @ 0.02, 1x1x1 box)")
    sc["block"] = (32, 16, 32)
    return sc, (dam_block(sc, (32, 16, 32), seed) if positions else None)


def pcisph_262k(seed=0, positions=True):
    """Plain PCISPH dam break: 64^3 at 0.01 in a 2 x 1.5 x 1 box, sphere r 0.15 at the centre."""
    sc = base_scene("pcisph", 0.01, (2.0, 1.5, 1.0))
    sc["colliders"].append({"type": "sphere", "center": (0.0, 0.0, 0.0), "radius": 0.15})
    # Advance(5e-4) splits into 2 CFL substeps (speed limit 4e-4 at scale 5)
    sc.update(dt=2.5e-4, advance_dt=5e-4, steps=500, max_iterations=20, max_density_error_ratio=0.01,
              workload="PCISPH dam break 262,144 particles (64^3 @ 0.01, 2x1.5x1 box, sphere r0.15)")
    sc["block"] = (64, 64, 64)
    return sc, (dam_block(sc, (64, 64, 64), seed) if positions else None)


def pcisph_1m(seed=0, positions=True):
    """PCISPH dam break: 128 x 64 x 128 at 0.008; the 1.024-deep block needs box z = 1.2."""
    sc = base_scene("pcisph", 0.008, (2.0, 1.0, 1.2))
    dt = 0.4 * (2 * 0.008) / 100.0 * 5.0   # CFL speed limit at scale 5 (particle.h:598)
    # the configuration sets no iteration cap: the corrector runs to the 1 % tolerance,
    # capped at 64 so that every substep of both the plain and the learned arm meets it
    sc.update(dt=dt, steps=1000, max_iterations=64, max_density_error_ratio=0.01,
              workload="PCISPH dam break 1,048,576 particles (128x64x128 @ 0.008, 2x1x1.2 box)")
    sc["block"] = (128, 64, 128)
    return sc, (dam_block(sc, (128, 64, 128), seed) if positions else None)


def pcisph_4m(seed=0, positions=True):
    """Large PCISPH: 256 x 64 x 256 at 0.005 in a 4 x 1 x 2 box with 8 seeded spheres."""
    sc = base_scene("pcisph", 0.005, (4.0, 1.0, 2.0))
    rng = np.random.default_rng(seed + 1)
    lo = np.asarray(sc["domain_min"]) + 0.005
    block_hi = lo + np.array([256, 64, 256]) * 0.005
    sc["colliders"] += place_spheres(rng, 8, 0.1, 0.3, (4.0, 1.0, 2.0), block_hi, 0.02)
    # Advance(2.5e-4) splits into 2 CFL substeps (speed limit 2e-4 at scale 5)
    sc.update(dt=1.25e-4, advance_dt=2.5e-4, steps=2000, max_iterations=20, max_density_error_ratio=0.01,
              workload="PCISPH dam break 4,194,304 particles (256x64x256 @ 0.005, 4x1x2 box, 8 spheres)")
    sc["block"] = (256, 64, 256)
    return sc, (dam_block(sc, (256, 64, 256), seed) if positions else None)


def small_pcisph(n_side=(12, 10, 12), spacing=0.02, box=(0.6, 0.5, 0.6), seed=0, sphere=True):
    """Small PCISPH dam break for parity tests (seconds on the CPU oracle)."""
    sc = base_scene("pcisph", spacing, box)
    if sphere:
        sc["colliders"].append({"type": "sphere", "center": (0.05, -0.05, 0.05), "radius": 0.08})
    sc.update(dt=4e-4, max_iterations=20, max_density_error_ratio=0.01)
    return sc, dam_block(sc, n_side, seed)


def batch_scenes(count, spacing, nmin, nmax, seed=0, positions=True):
    """Independent dam breaks for a batch: particle counts log-uniform in [nmin, nmax],
    block aspect ratios uniform in [0.3, 1] per axis; each container is centred at the
    origin and holds its block in the (-x, -y, -z) corner with room to collapse (twice
    the block along x, 1.5 times along y, plus one spacing of margin on every side)."""
    rng = np.random.default_rng(seed)
    boxes, pos = [], []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        a = rng.uniform(0.3, 1.0, 3)
        k = (n / float(np.prod(a))) ** (1.0 / 3.0)
        dims = np.maximum(2, np.round(a * k)).astype(int)
        block = dims * spacing
        ext = np.array([2.0 * block[0], 1.5 * block[1], block[2]]) + 2.0 * spacing
        lo, hi = -ext / 2, ext / 2
        boxes.append((tuple(lo), tuple(hi)))
        if positions:
            sc = {"spacing": spacing, "domain_min": tuple(lo)}
            pos.append(dam_block(sc, tuple(int(d) for d in dims), int(rng.integers(1 << 31))))
        else:
            rng.integers(1 << 31)
            pos.append(np.zeros((int(np.prod(dims)), 3)))
    return boxes, pos


def batched_64(seed=0, positions=True):
    """64 independent PCISPH dam breaks at spacing 0.01 in one solver: counts
    log-uniform in [8,192, 131,072], aspect ratios uniform in [0.3, 1]."""
    sc = base_scene("pcisph", 0.01, (1.0, 1.0, 1.0))
    dt = 0.4 * (2 * 0.01) / 100.0 * 5.0   # CFL speed limit at scale 5 (particle.h:598)
    boxes, pos = batch_scenes(64, 0.01, 8192, 131072, seed=seed, positions=positions)
    total = sum(len(p) for p in pos)
    # config 4 states no corrector cap: 64 (the device limit), so that both arms reach 1 %
    sc.update(dt=dt, steps=500, max_iterations=64, max_density_error_ratio=0.01, batch=True,
              boxes=boxes,
              workload="Batched PCISPH: 64 dam breaks, %d particles (counts log-uniform in "
                       "[8192, 131072], spacing 0.01)" % total)
    return sc, pos


CONFIGS = {
    "sph_16k": sph_16k,
    "pcisph_262k": pcisph_262k,
    "pcisph_1m": pcisph_1m,
    "pcisph_4m": pcisph_4m,
    "batched_64": batched_64,
}


def config(name, seed=0, positions=True):
    return CONFIGS[name](seed, positions)
