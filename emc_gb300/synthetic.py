"""Seeded synthetic EMC problems with the shapes of the benchmark configurations.

The reference reads HDF5 diffraction patterns through libspimage
(emc_helper.cpp:198-248); that input path has no data here, so problems are
generated: a particle of isotropic Gaussian atoms inside a sphere, its
diffraction intensity |F(q)|^2 sampled at the model's voxel centres
q = idx - side/2 + 0.5 (the grid convention of the slicing kernels), patterns
that are slices of that intensity at uniform random orientations times a
per-pattern scale, Poisson-sampled to a target mean photon count, a detector
mask (circle of radius side/2 as in read_mask, emc_helper.cpp:358-366, minus a
central beamstop, optionally with panel gaps), and a uniform [0, 1) random
initial model (model_input = 0, emc_helper.cpp:449-456; numpy PCG64 instead of
GSL taus).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# emc.conf:3-6 detector geometry
WAVELENGTH = 1.03e-9
PIXEL_SIZE = 75.0e-6
DISTANCE = 740.0e-3
# emc.conf:8-10 annealing
SIGMA_START, SIGMA_FINAL, SIGMA_HALF_LIFE = 0.4, 0.12, 25


@dataclass
class Config:
    name: str
    side: int
    n_atoms: int
    atom_sigma: float
    radius: float
    n_images: int
    photons: float
    scale: tuple
    beamstop: float
    rot_n: int
    iterations: int
    seed: int = 0
    blur: float = 0.0
    masked_fraction: float = 0.0  # extra panel-gap masking (low-count config)
    extra: dict = field(default_factory=dict)


CONFIGS = {
    "small": Config("small", 64, 400, 1.5, 12, 2000, 1000, (0.5, 1.5), 4, 4, 20, blur=1.0),
    "mid": Config("mid", 128, 3000, 1.5, 28, 20000, 5000, (0.5, 1.5), 6, 8, 30),
    "lowcount": Config("lowcount", 128, 3000, 1.5, 28, 50000, 80, (0.2, 2.0), 6, 6, 30,
                       masked_fraction=0.5),
    "large": Config("large", 256, 20000, 1.5, 56, 100000, 10000, (0.5, 1.5), 12, 12, 5),
    # the mid geometry with a fifth of the patterns: kernel profiles of a few GB
    "mid_small": Config("mid_small", 128, 3000, 1.5, 28, 4000, 5000, (0.5, 1.5), 6, 8, 1),
    # the mid geometry and patterns with the 6,300 rotations of level 5: profiles of the
    # per-row kernels (expand, mprep) on a few GB
    "mid_r5": Config("mid_r5", 128, 3000, 1.5, 28, 20000, 5000, (0.5, 1.5), 6, 5, 1),
}


def tiny(side=24, n_images=48, rot_n=2, photons=400, seed=0, n_atoms=60, radius=5.0):
    """A problem small enough for the direct-loop oracle (tests)."""
    return Config(f"tiny{side}", side, n_atoms, 1.2, radius, n_images, photons, (0.5, 1.5), 2,
                  rot_n, 1, seed=seed)


def random_quaternions(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniform random unit quaternions (Shoemake; cf. rotations.c:30-41)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], 1)
    return q


def quat_matrices(q: np.ndarray) -> np.ndarray:
    """Rotation matrices of quaternions (w, x, y, z), the convention of
    emc_cuda.cu:113-121, in float64."""
    a, b, c, d = (q[:, k].astype(np.float64) for k in range(4))
    m = np.empty((q.shape[0], 3, 3))
    m[:, 0, 0] = a * a + b * b - c * c - d * d
    m[:, 0, 1] = 2 * b * c - 2 * a * d
    m[:, 0, 2] = 2 * b * d + 2 * a * c
    m[:, 1, 0] = 2 * b * c + 2 * a * d
    m[:, 1, 1] = a * a - b * b + c * c - d * d
    m[:, 1, 2] = 2 * c * d - 2 * a * b
    m[:, 2, 0] = 2 * b * d - 2 * a * c
    m[:, 2, 1] = 2 * c * d + 2 * a * b
    m[:, 2, 2] = a * a - b * b - c * c + d * d
    return m


def particle_intensity(side: int, n_atoms: int, atom_sigma: float, radius: float,
                       rng: np.random.Generator) -> np.ndarray:
    """|F(q)|^2 at q = idx - side/2 + 0.5 of Gaussian atoms uniform in a sphere,
    normalised to mean 1, float32 [z][y][x]."""
    s = side
    # atom centres uniform in a ball (voxels, relative to the box centre)
    pos = rng.normal(size=(n_atoms, 3))
    pos *= (radius * rng.random(n_atoms) ** (1 / 3) / np.linalg.norm(pos, axis=1))[:, None]
    # structure factor on the half-integer grid via FFT of a phase-ramped
    # point lattice: F(q) = G(q) sum_j exp(-2 pi i q . r_j / s)
    q1 = np.arange(s) - s / 2 + 0.5
    F = np.empty((s, s, s), np.complex128)
    # exact separable sum over atoms (no gridding error), one GEMM per z-plane
    ex = np.exp(-2j * np.pi * np.outer(pos[:, 0], q1) / s)
    ey = np.exp(-2j * np.pi * np.outer(pos[:, 1], q1) / s)
    ez = np.exp(-2j * np.pi * np.outer(pos[:, 2], q1) / s)
    for iz in range(s):
        F[iz] = (ey * ez[:, iz][:, None]).T @ ex
    qq = q1[:, None, None] ** 2 + q1[None, :, None] ** 2 + q1[None, None, :] ** 2
    G = np.exp(-2 * np.pi ** 2 * atom_sigma ** 2 * qq / s ** 2)
    I = np.abs(F * G) ** 2
    return (I / I.mean()).astype(np.float32)


def detector_mask(side: int, beamstop: float, masked_fraction: float,
                  rng: np.random.Generator) -> np.ndarray:
    """int32 [side*side] mask, index y*side + x."""
    c = np.arange(side) - side / 2.0 + 0.5
    r = np.sqrt(c[None, :] ** 2 + c[:, None] ** 2)  # [y][x]
    m = (r <= side / 2.0) & (r >= beamstop)
    if masked_fraction > 0:
        # rectangular panel gaps until the requested fraction is masked
        target = (1 - masked_fraction) * m.sum()
        while m.sum() > target:
            if rng.random() < 0.5:
                x0 = rng.integers(0, side)
                w = rng.integers(1, max(2, side // 24))
                m[:, x0:x0 + w] = False
            else:
                y0 = rng.integers(0, side)
                w = rng.integers(1, max(2, side // 24))
                m[y0:y0 + w, :] = False
    return m.astype(np.int32).reshape(-1)


def trilinear(model: np.ndarray, coords: np.ndarray) -> np.ndarray:
    """Trilinear samples of model [z][y][x] at fractional voxel coords [..., 3]
    (x, y, z); outside points read 0."""
    s = model.shape[0]
    out = np.zeros(coords.shape[:-1])
    x, y, z = coords[..., 0], coords[..., 1], coords[..., 2]
    x0, y0, z0 = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64), np.floor(z).astype(np.int64)
    tx, ty, tz = x - x0, y - y0, z - z0
    for c in range(8):
        xi, yi, zi = x0 + (c & 1), y0 + ((c >> 1) & 1), z0 + (c >> 2)
        w = np.where(c & 1, tx, 1 - tx) * np.where((c >> 1) & 1, ty, 1 - ty) * np.where(c >> 2, tz, 1 - tz)
        ok = (xi >= 0) & (xi < s) & (yi >= 0) & (yi < s) & (zi >= 0) & (zi < s)
        v = model[np.clip(zi, 0, s - 1), np.clip(yi, 0, s - 1), np.clip(xi, 0, s - 1)]
        out += np.where(ok, w * v, 0.0)
    return out


@dataclass
class Problem:
    cfg: Config
    true_model: np.ndarray   # float32 [s^3]
    init_model: np.ndarray   # float32 [s^3]
    images: np.ndarray       # float32 [N][s*s] photon counts
    mask: np.ndarray         # int32 [s*s]
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    quats: np.ndarray        # float32 [R][4]
    weights: np.ndarray      # float32 [R]
    true_quats: np.ndarray   # float64 [N][4]
    scales: np.ndarray       # float64 [N]


def make_problem(cfg: Config, device: str | None = None, coords=None, rotations=None,
                 pattern_seed: int | None = None) -> Problem:
    """Builds the problem.  `coords` = (x, y, z) and `rotations` = (quats,
    weights) come from the library's host functions (emc_calculate_coordinates,
    emc_generate_rotations) unless given.  `device` = "cuda" renders the
    patterns with torch on the GPU (same numbers up to float rounding).
    `pattern_seed` draws new orientations, scales, counts and initial model
    for the same particle and detector (a held-out set)."""
    rng = np.random.default_rng(cfg.seed)
    s = cfg.side
    true = particle_intensity(s, cfg.n_atoms, cfg.atom_sigma, cfg.radius, rng)
    if coords is None or rotations is None:
        import emc_gb300 as E
        if coords is None:
            coords = E.calculate_coordinates(s, PIXEL_SIZE, DISTANCE, WAVELENGTH)
        if rotations is None:
            rotations = E.generate_rotations(cfg.rot_n)
    x, y, z = coords
    quats, weights = rotations
    mask = detector_mask(s, cfg.beamstop, cfg.masked_fraction, rng)
    if pattern_seed is not None:
        rng = np.random.default_rng([cfg.seed, 7919, pattern_seed])
    N = cfg.n_images
    tq = random_quaternions(N, rng)
    scales = rng.uniform(cfg.scale[0], cfg.scale[1], N)
    pts = np.stack([x, y, z], 1).astype(np.float64)  # [P][3]
    # expected intensity of every pattern, then Poisson counts
    if device is None:
        lam = np.zeros((N, s * s), np.float32)
        for i0 in range(0, N, 256):
            i1 = min(N, i0 + 256)
            rc = np.einsum("nij,pj->npi", quat_matrices(tq[i0:i1]), pts) + (s / 2 - 0.5)
            lam[i0:i1] = trilinear(true.reshape(s, s, s), rc) * mask[None, :]
        lam *= (cfg.photons / lam.sum(1, dtype=np.float64).mean()) * scales[:, None]
        images = rng.poisson(lam).astype(np.float32)
    else:
        images = _render_torch(true.reshape(s, s, s), tq, pts, mask, scales, cfg, device,
                               0 if pattern_seed is None else 1000003 * (pattern_seed + 1))
    init = rng.random(s ** 3).astype(np.float32)
    return Problem(cfg, true.reshape(-1), init, images, mask, x, y, z, quats, weights, tq, scales)


def write_problem(prob: Problem, directory, iterations=1, extra="", model_input=2,
                  normalize_images=False, raw=None, read_stride=1):
    """Writes the `emc` driver's inputs: images.bin (float32 [N][s*s]),
    mask.bin (int32 [s*s]), model.bin (float32 [s^3], read with model_input 2)
    and an emc.conf that points at them.  With raw = (frames [N][D][D],
    masks [N][D][D]) it writes raw.bin / raw_mask.bin instead of images.bin,
    for binning by read_stride.  Returns the config path."""
    import os
    d = os.path.abspath(str(directory))
    os.makedirs(d, exist_ok=True)
    c = prob.cfg
    detector = c.side
    if raw is None:
        np.ascontiguousarray(prob.images, np.float32).tofile(os.path.join(d, "images.bin"))
    else:
        frames, fmasks = raw
        detector = frames.shape[-1]
        np.ascontiguousarray(frames, np.float32).tofile(os.path.join(d, "raw.bin"))
        np.ascontiguousarray(fmasks, np.int32).tofile(os.path.join(d, "raw_mask.bin"))
    np.ascontiguousarray(prob.mask, np.int32).tofile(os.path.join(d, "mask.bin"))
    np.ascontiguousarray(prob.init_model, np.float32).tofile(os.path.join(d, "model.bin"))
    conf = os.path.join(d, "emc.conf")
    with open(conf, "w") as f:
        f.write(f"""# synthetic problem {c.name}
model_side = {c.side};
read_stride = {read_stride};
wavelength = {WAVELENGTH!r};
pixel_size = {PIXEL_SIZE!r};
detector_size = {detector};
detector_distance = {DISTANCE!r};
rotations_n = {c.rot_n};
sigma_start = {SIGMA_START};
sigma_final = {SIGMA_FINAL};
sigma_half_life = {SIGMA_HALF_LIFE};
diff_type = "poisson";
slice_chunk = 5000;
N_images = {c.n_images};
max_iterations = {iterations};
image_prefix = "{d}/";
mask_file = "{d}/mask.bin";
normalize_images = {"true" if normalize_images else "false"};
known_intensity = false;
model_input = {model_input};
model_file = "{d}/model.bin";
isOutput = 1;
output_loop = 0;
output_period = 1;
isDebug = 1;
{extra}
""")
    return conf


def _render_torch(model, tq, pts, mask, scales, cfg, device, seed_offset=0):
    """GPU rendering of the Poisson patterns (torch; the generator is seeded)."""
    import torch
    s = model.shape[0]
    m = torch.as_tensor(model, device=device, dtype=torch.float32)[None, None]
    P = torch.as_tensor(pts, device=device, dtype=torch.float32)
    mk = torch.as_tensor(mask, device=device, dtype=torch.float32)
    N = tq.shape[0]
    lam = torch.empty((N, s * s), device=device, dtype=torch.float32)
    for i0 in range(0, N, 1024):
        i1 = min(N, i0 + 1024)
        M = torch.as_tensor(quat_matrices(tq[i0:i1]), device=device, dtype=torch.float32)
        rc = torch.einsum("nij,pj->npi", M, P) + (s / 2 - 0.5)
        g = (rc + 0.5) / s * 2 - 1  # grid_sample, align_corners=False: voxel i at (2i+1)/s - 1
        out = torch.nn.functional.grid_sample(m.expand(1, 1, s, s, s), g[None, :, :, None, :],
                                              mode="bilinear", padding_mode="zeros",
                                              align_corners=False)
        lam[i0:i1] = out[0, 0, :, :, 0] * mk
    lam *= float(cfg.photons / lam.sum(1, dtype=torch.float64).mean().item())
    lam *= torch.as_tensor(scales, device=device, dtype=torch.float32)[:, None]
    gen = torch.Generator(device=device)
    gen.manual_seed(cfg.seed + 12345 + seed_offset)
    # one Poisson draw per chunk of fewer than 2^31 elements: a single draw over
    # the 256^3 workload's 6.6e9 elements left part of its output unwritten
    step = max(1, (2 ** 31 - 1) // (s * s))
    out = np.empty((N, s * s), np.float32)
    for i0 in range(0, N, step):
        i1 = min(N, i0 + step)
        out[i0:i1] = torch.poisson(lam[i0:i1], generator=gen).cpu().numpy()
    return out
