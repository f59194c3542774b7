"""Seeded synthetic scalar fields for the compression workloads.

The reference measures on HDF5 simulation snapshots (demo.h5, a 512^3
cavitation pressure field) that are not available offline; these fields have
the same shapes and value structure: smooth Gaussian blobs, band-limited
noise with a k^-5/3 energy spectrum and random phases, and sharp spherical
tanh interfaces, offset to a chosen mean (1.0 for density/pressure-like
fields) or scaled to zero mean and unit rms (velocity-like fields).

Fields are float32, x fastest: shape (nz, ny, nx). Generation is plain numpy
and deterministic for a given seed on every host.
"""
import numpy as np


def _noise(shape, rng, rms):
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.rfftfreq(nx) * nx
    k = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    kmax = min(nx, ny, nz) / 2.0
    amp = np.zeros_like(k)
    band = (k >= 1.0) & (k <= kmax)
    # shell energy E(k) ~ k^-5/3 with ~k^2 modes per shell: amplitude k^(-11/6)
    amp[band] = k[band] ** (-11.0 / 6.0)
    phase = rng.uniform(0.0, 2.0 * np.pi, size=k.shape)
    spec = amp * np.exp(1j * phase)
    f = np.fft.irfftn(spec, s=shape, axes=(0, 1, 2))
    s = f.std()
    return f * (rms / s) if s > 0 else f


def _box(c, r, n):
    return max(0, int(np.floor(c - r))), min(n, int(np.ceil(c + r)) + 1)


def generate(shape, seed=0, blobs=20, interfaces=3, noise_rms=0.05, mean=1.0, velocity=False):
    """One field of the given (nz, ny, nx) shape.

    blobs: Gaussian blobs with amplitude U[0.5,2] and sigma U[4,16] cells,
    evaluated within 8 sigma of their centre (beyond it they are below
    1e-13 of their amplitude);
    interfaces: tanh spheres of width 2 cells and jump 1.0, evaluated within
    a box reaching 40 cells beyond the sphere (farther out the profile is
    below 1e-17);
    velocity=True: random signs on the blob amplitudes, then zero mean and
    unit rms; otherwise the field is offset to `mean`.
    """
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    f = np.zeros(shape, np.float64)
    for _ in range(blobs):
        a = rng.uniform(0.5, 2.0) * (rng.choice([-1.0, 1.0]) if velocity else 1.0)
        sig = rng.uniform(4.0, 16.0)
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        (z0, z1), (y0, y1), (x0, x1) = _box(cz, 8 * sig, nz), _box(cy, 8 * sig, ny), _box(cx, 8 * sig, nx)
        gz = np.exp(-((np.arange(z0, z1) - cz) ** 2) / (2 * sig * sig))[:, None, None]
        gy = np.exp(-((np.arange(y0, y1) - cy) ** 2) / (2 * sig * sig))[None, :, None]
        gx = np.exp(-((np.arange(x0, x1) - cx) ** 2) / (2 * sig * sig))[None, None, :]
        f[z0:z1, y0:y1, x0:x1] += a * (gz * gy) * gx
    f += _noise(shape, rng, noise_rms)
    lo = min(nx, ny, nz)
    for _ in range(interfaces):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        r0 = rng.uniform(0.1, 0.3) * lo
        (z0, z1), (y0, y1), (x0, x1) = _box(cz, r0 + 40, nz), _box(cy, r0 + 40, ny), _box(cx, r0 + 40, nx)
        r = np.sqrt((np.arange(z0, z1)[:, None, None] - cz) ** 2 + (np.arange(y0, y1)[None, :, None] - cy) ** 2 +
                    (np.arange(x0, x1)[None, None, :] - cx) ** 2)
        f[z0:z1, y0:y1, x0:x1] += 0.5 * (1.0 - np.tanh((r - r0) / 2.0))
    if velocity:
        f -= f.mean()
        s = f.std()
        if s > 0:
            f /= s
    else:
        f += mean - f.mean()
    return np.ascontiguousarray(f, dtype=np.float32)


def config_field(name, seed=0):
    """The workloads' fields by name: 'small' 128^3 (20 blobs, 3 interfaces),
    'large' 512^3 (200 blobs, 12 interfaces), 'refit' 256^3 (60 blobs,
    6 interfaces)."""
    if name == "small":
        return generate((128, 128, 128), seed, blobs=20, interfaces=3)
    if name == "large":
        return generate((512, 512, 512), seed, blobs=200, interfaces=12)
    if name == "refit":
        return generate((256, 256, 256), seed, blobs=60, interfaces=6)
    raise KeyError(name)


def batch_shapes(n=96, seed=0):
    """Uneven batch: edges drawn uniformly from {64, 96, ..., 384} per axis and
    per-field thresholds log-uniform in [1e-5, 1e-2]."""
    rng = np.random.default_rng(seed)
    edges = np.arange(64, 385, 32)
    shapes = [tuple(int(e) for e in rng.choice(edges, size=3)) for _ in range(n)]
    thr = 10.0 ** rng.uniform(-5.0, -2.0, size=n)
    return shapes, thr


def generate_torch(shape, seed=0, blobs=20, interfaces=3, noise_rms=0.05, mean=1.0, velocity=False, device="cuda"):
    """The generator of `generate` evaluated with torch on `device` in
    float32: same parameter draws (numpy, seeded), noise phases from a
    seeded torch generator. Statistically the same fields, not the same
    bits; for workloads too large to build on the host."""
    import torch
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    f = torch.zeros(shape, dtype=torch.float32, device=device)

    def ar(a, b):
        return torch.arange(a, b, device=device, dtype=torch.float32)

    for _ in range(blobs):
        a = rng.uniform(0.5, 2.0) * (rng.choice([-1.0, 1.0]) if velocity else 1.0)
        sig = rng.uniform(4.0, 16.0)
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        (z0, z1), (y0, y1), (x0, x1) = _box(cz, 8 * sig, nz), _box(cy, 8 * sig, ny), _box(cx, 8 * sig, nx)
        gz = torch.exp(-((ar(z0, z1) - cz) ** 2) / (2 * sig * sig))[:, None, None]
        gy = torch.exp(-((ar(y0, y1) - cy) ** 2) / (2 * sig * sig))[None, :, None]
        gx = torch.exp(-((ar(x0, x1) - cx) ** 2) / (2 * sig * sig))[None, None, :]
        f[z0:z1, y0:y1, x0:x1] += a * (gz * gy) * gx
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    kz = torch.fft.fftfreq(nz, device=device) * nz
    ky = torch.fft.fftfreq(ny, device=device) * ny
    kx = torch.fft.rfftfreq(nx, device=device) * nx
    k = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    kmax = min(nx, ny, nz) / 2.0
    amp = torch.where((k >= 1.0) & (k <= kmax), k.clamp(min=1.0) ** (-11.0 / 6.0), torch.zeros_like(k))
    phase = torch.rand(k.shape, generator=g, device=device) * (2 * np.pi)
    noise = torch.fft.irfftn(torch.polar(amp, phase), s=shape, dim=(0, 1, 2))
    s = noise.std()
    f += noise * (noise_rms / s) if s > 0 else noise
    lo = min(nx, ny, nz)
    for _ in range(interfaces):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        r0 = rng.uniform(0.1, 0.3) * lo
        (z0, z1), (y0, y1), (x0, x1) = _box(cz, r0 + 40, nz), _box(cy, r0 + 40, ny), _box(cx, r0 + 40, nx)
        r = torch.sqrt((ar(z0, z1)[:, None, None] - cz) ** 2 + (ar(y0, y1)[None, :, None] - cy) ** 2 +
                       (ar(x0, x1)[None, None, :] - cx) ** 2)
        f[z0:z1, y0:y1, x0:x1] += 0.5 * (1.0 - torch.tanh((r - r0) / 2.0))
    if velocity:
        f -= f.mean()
        s = f.std()
        if s > 0:
            f /= s
    else:
        f += mean - f.mean()
    return f.contiguous()
