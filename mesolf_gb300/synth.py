"""Seeded synthetic light-field workloads (PSFs, volumes, measured images).

The reference's real PSF (a 3.3 GB MATLAB file) and its demo recordings are not
available, so every workload is synthetic, generated from a seed:

* PSF ``H(K0, K0, N, N, Z)``: for each (u, v, z) a normalised Gaussian disc of radius
  ``2 + 0.6|z_idx|`` px (Gaussian profile with sigma = radius / 2), centred on the array
  and shifted laterally by ``(u - (N+1)/2, v - (N+1)/2) * z_idx * 0.15`` px (1-based u,
  v), optionally confined to a centred per-plane window, times a uniform[0.9, 1.1]
  jitter.  ``Ht`` is the 180-degree rotation of each (u, v, z) slice.
* Volume: Gaussian blobs (lateral sigma in px, axial sigma in planes) at uniform random
  positions plus a constant background.
* Measured image: a forward projection of the volume scaled to a photon peak and
  Poisson-sampled.

Array index order follows MATLAB (``H[x, y, a, b, z]``, ``vol[r, c, z]``); arrays are
returned Fortran-ordered so their memory layout is MATLAB's column-major layout.
"""
from __future__ import annotations

import dataclasses

import numpy as np

__all__ = ["make_psf", "make_volume", "forward_project_full", "poisson_image",
           "Workload", "config1", "config2", "small_config", "fortran32",
           "carpet_geometry", "SomaStream", "uneven_batch_geometry"]


def fortran32(a):
    """float32, column-major (MATLAB) memory layout."""
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


def make_psf(K0, N, z_idx, seed=0, plane_sides=None, shift_per_z=0.15,
             jitter=(0.9, 1.1), dtype=np.float32):
    """Synthetic LFM PSF pair (H, Ht), each (K0, K0, N, N, Z) column-major.

    ``z_idx`` lists the depth index of each plane; ``plane_sides`` (optional) gives a
    per-plane odd window side outside of which the PSF is zero.
    """
    z_idx = np.asarray(z_idx, dtype=np.float64)
    Z = z_idx.size
    rng = np.random.default_rng(seed)
    jit = rng.uniform(jitter[0], jitter[1], size=(N, N, Z))
    H = np.zeros((K0, K0, N, N, Z), dtype=dtype, order="F")
    x = np.arange(K0, dtype=np.float64)
    ctr = (K0 - 1) / 2.0
    uu = np.arange(1, N + 1, dtype=np.float64) - (N + 1) / 2.0
    for k in range(Z):
        zi = z_idx[k]
        radius = 2.0 + 0.6 * abs(zi)
        sigma = radius / 2.0
        cu = ctr + uu * zi * shift_per_z                        # (N,) centres per source index
        d2x = (x[:, None] - cu[None, :]) ** 2                   # (K0, N)
        win = np.ones(K0, dtype=bool)
        if plane_sides is not None:
            win = np.abs(x - ctr) <= (int(plane_sides[k]) - 1) / 2.0
        # hard-edged disc of the given radius, Gaussian profile inside (zero outside)
        lo = max(0, int(np.floor(cu.min() - radius)) - 1)
        hi = min(K0, int(np.ceil(cu.max() + radius)) + 2)
        sub = slice(lo, hi)
        d2 = d2x[sub, None, :, None] + d2x[None, sub, None, :]  # (n, n, N, N)
        g = np.exp(-d2 / (2 * sigma ** 2)) * (d2 <= radius * radius)
        g = g * (win[sub, None] & win[None, sub])[:, :, None, None]
        g = g / g.sum(axis=(0, 1), keepdims=True)
        H[sub, sub, :, :, k] = (g * jit[None, None, :, :, k]).astype(dtype)
    Ht = np.asfortranarray(H[::-1, ::-1, :, :, :])
    return H, Ht


def make_volume(Xr, Xc, Z, n_obj, sigma, peaks, background, seed=0, sigma_z=1.0):
    """Gaussian blobs at uniform random positions plus a background, (Xr, Xc, Z)."""
    rng = np.random.default_rng(seed + 1)
    pos = np.column_stack([rng.uniform(0, Xr, n_obj), rng.uniform(0, Xc, n_obj),
                           rng.uniform(0, Z, n_obj)])
    if peaks == "uniform":
        amp = rng.uniform(0.5, 1.0, n_obj)
    elif peaks == "lognormal":
        amp = rng.lognormal(0.0, 0.5, n_obj)
    else:
        raise ValueError(peaks)
    vol = np.full((Xr, Xc, Z), background, dtype=np.float64)
    rw = int(np.ceil(4 * sigma))
    zw = int(np.ceil(4 * sigma_z))
    for (pr, pc, pz), a in zip(pos, amp):
        r0, r1 = max(0, int(pr) - rw), min(Xr, int(pr) + rw + 1)
        c0, c1 = max(0, int(pc) - rw), min(Xc, int(pc) + rw + 1)
        z0, z1 = max(0, int(pz) - zw), min(Z, int(pz) + zw + 1)
        gr = np.exp(-((np.arange(r0, r1) - pr) ** 2) / (2 * sigma ** 2))
        gc = np.exp(-((np.arange(c0, c1) - pc) ** 2) / (2 * sigma ** 2))
        gz = np.exp(-((np.arange(z0, z1) - pz) ** 2) / (2 * sigma_z ** 2))
        vol[r0:r1, c0:c1, z0:z1] += a * gr[:, None, None] * gc[None, :, None] * gz[None, None, :]
    return np.asfortranarray(vol.astype(np.float32))


def forward_project_full(H, vol, device="cpu", dtype=None):
    """Full LFM forward projection ``sum_{a,b,z} conv2(vol_z .* phase(a,b), H(:,:,a,b,z),
    'same')`` evaluated with FFTs in torch (CPU or CUDA).  Data generation only."""
    import torch
    if dtype is None:
        dtype = torch.float64 if device == "cpu" else torch.float32
    Hn = torch.as_tensor(np.ascontiguousarray(H), device=device).to(dtype)
    v = torch.as_tensor(np.ascontiguousarray(vol), device=device).to(dtype)
    K0, N, Z = Hn.shape[0], Hn.shape[2], Hn.shape[4]
    Xr, Xc = v.shape[0], v.shape[1]
    m = K0 // 2
    E = (Xr + K0 - 1, Xc + K0 - 1)
    out = torch.zeros((Xr, Xc), dtype=dtype, device=device)
    for z in range(Z):
        ts = torch.zeros((N, N, Xr, Xc), dtype=dtype, device=device)
        for a in range(N):
            for b in range(N):
                ts[a, b, a::N, b::N] = v[a::N, b::N, z]
        Fv = torch.fft.rfft2(ts, s=E)
        Fh = torch.fft.rfft2(Hn[:, :, :, :, z].permute(2, 3, 0, 1), s=E)
        full = torch.fft.irfft2((Fv * Fh).sum(dim=(0, 1)), s=E)
        out += full[m:m + Xr, m:m + Xc]
    return out.cpu().numpy().astype(np.float64)


def poisson_image(clean, peak_photons, seed=0):
    """Scale so the maximum is ``peak_photons`` and Poisson-sample (float32 counts)."""
    rng = np.random.default_rng(seed + 2)
    lam = np.clip(clean, 0, None) * (peak_photons / clean.max())
    return np.asfortranarray(rng.poisson(lam).astype(np.float32))


@dataclasses.dataclass
class Workload:
    name: str
    N: int
    lenslets: tuple
    K0: int
    z_idx: np.ndarray
    plane_sides: object
    n_obj: int
    sigma: float
    peaks: str
    background: float
    photons: float
    iters: int
    seed: int = 0

    @property
    def image_shape(self):
        return (self.lenslets[0] * self.N, self.lenslets[1] * self.N)

    @property
    def Z(self):
        return len(self.z_idx)

    @property
    def voxels(self):
        r, c = self.image_shape
        return r * c * self.Z

    def psf(self):
        return make_psf(self.K0, self.N, self.z_idx, seed=self.seed, plane_sides=self.plane_sides)

    def volume(self):
        r, c = self.image_shape
        return make_volume(r, c, self.Z, self.n_obj, self.sigma, self.peaks,
                           self.background, seed=self.seed)

    def measured(self, H, vol, device="cpu"):
        clean = forward_project_full(H, vol, device=device)
        return poisson_image(clean, self.photons, seed=self.seed)


def config1(seed=0):
    """Nnum 15, 11x11 lenslets, 21 planes (-40..40 um), K0 61, 40 spheres, 8 iterations."""
    return Workload("lf165x165x21_k61_it8", 15, (11, 11), 61, np.arange(-10, 11), None,
                    40, 3.0, "uniform", 0.01, 1000.0, 8, seed)


def config2(seed=0):
    """Nnum 15, 67x67 lenslets, 51 planes (0..200 um), plane k window 31+4k (K0 231),
    2000 somas (sigma 4 px, lognormal peaks), 3 iterations."""
    k = np.arange(51)
    sides = np.minimum(31 + 4 * k, 255)
    return Workload("lf1005x1005x51_k231_it3", 15, (67, 67), int(sides.max()), k, sides,
                    2000, 4.0, "lognormal", 0.02, 2000.0, 3, seed)


def small_config(lenslets=(9, 8), K0=61, Z=7, iters=2, seed=0, n_obj=12, name=None):
    """Small uneven workload for parity tests."""
    z = np.arange(Z) - Z // 2
    return Workload(name or f"small{lenslets[0]}x{lenslets[1]}x{Z}_k{K0}", 15, tuple(lenslets),
                    K0, z, None, n_obj, 3.0, "uniform", 0.01, 1000.0, iters, seed)


# ----------------------------------------------------------------------------- streams
def carpet_geometry(n_side=6, lenslets=(45, 71), N=15, seed=5):
    """Image shapes of an n_side x n_side patch carpet, lenslets per side uniform in the
    closed range ``lenslets`` (seeded)."""
    rng = np.random.default_rng(seed)
    L = rng.integers(lenslets[0], lenslets[1] + 1, size=(n_side * n_side, 2))
    return [(int(a) * N, int(b) * N) for a, b in L]


def uneven_batch_geometry(n=64, lenslets=(31, 71), planes=(26, 101), Z=101, N=15, seed=4):
    """Shapes and plane ranges of n independent patches: lenslets per side uniform in
    ``lenslets``, plane count uniform in ``planes``, each range placed at a uniform offset
    inside the PSF's Z planes (seeded)."""
    rng = np.random.default_rng(seed)
    L = rng.integers(lenslets[0], lenslets[1] + 1, size=(n, 2))
    nz = rng.integers(planes[0], planes[1] + 1, size=n)
    z0 = [int(rng.integers(0, Z - k + 1)) for k in nz]
    return [(int(a) * N, int(b) * N) for a, b in L], [(z, int(k)) for z, k in zip(z0, nz)]


class SomaStream:
    """Soma field of one patch whose intensities follow a slow AR(1) random walk across
    frames (x_f = rho x_{f-1} + sqrt(1 - rho^2) e_f, intensity = base * exp(0.25 x_f)),
    rendered on the GPU: impulses at integer soma centres blurred by separable Gaussians
    (lateral sigma in px, axial sigma in planes), plus a constant background.  Volumes are
    (Xr, Xc, Z) float32 torch tensors in column-major layout."""

    def __init__(self, shape, Z, n_obj, sigma=4.0, sigma_z=1.0, background=0.02, rho=0.95,
                 seed=0, device="cuda"):
        import torch
        self.torch = torch
        self.shape = (int(shape[0]), int(shape[1]), int(Z))
        rng = np.random.default_rng(seed)
        Xr, Xc, Z = self.shape
        self.idx = torch.as_tensor(rng.integers(0, Xr, n_obj) + Xr * (rng.integers(0, Xc, n_obj) +
                                   Xc * rng.integers(0, Z, n_obj)), device=device)
        self.base = torch.as_tensor(rng.lognormal(0.0, 0.5, n_obj), dtype=torch.float32, device=device)
        self.x = torch.zeros(n_obj, dtype=torch.float32, device=device)
        self.rho = rho
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(int(seed) + 17)
        self.background = background
        self.device = device

        def g(s):
            r = int(np.ceil(4 * s))
            k = np.exp(-np.arange(-r, r + 1) ** 2 / (2 * s * s))
            return torch.as_tensor(k, dtype=torch.float32, device=device).view(1, 1, -1), r

        self.gl, self.rl = g(sigma)
        self.gz, self.rz = g(sigma_z)

    def _blur_last(self, v, k, r):
        F = self.torch.nn.functional
        sh = v.shape
        return F.conv1d(v.reshape(-1, 1, sh[-1]), k, padding=r).reshape(sh)

    def step(self):
        torch = self.torch
        e = torch.randn(self.x.shape, generator=self.gen, device=self.device)
        self.x = self.rho * self.x + float(np.sqrt(1 - self.rho ** 2)) * e
        amp = self.base * torch.exp(0.25 * self.x)
        Xr, Xc, Z = self.shape
        v = torch.zeros(Xr * Xc * Z, dtype=torch.float32, device=self.device)
        v.index_add_(0, self.idx, amp)
        v = v.view(Z, Xc, Xr)                                   # column-major (Xr, Xc, Z)
        v = self._blur_last(v, self.gl, self.rl)                # along Xr
        v = self._blur_last(v.transpose(1, 2).contiguous(), self.gl, self.rl).transpose(1, 2)   # Xc
        v = self._blur_last(v.permute(1, 2, 0).contiguous(), self.gz, self.rz).permute(2, 0, 1)  # Z
        v = v.contiguous() + self.background
        return v.permute(2, 1, 0)


def sensor_movie(P, T, seed=0, device=None, n_spike=0.004, tau=8.0):
    """Synthetic sensor movie, (P pixels, T frames) float32 column-major (frame-contiguous):
    per-pixel baseline (100..600) with a slow bleaching trend, calcium-like transients
    (events with probability ``n_spike`` per frame, exponential decay ``tau`` frames, amplitude
    up to 300) and Gaussian noise (sigma 8).  numpy on the host when ``device`` is None, else
    a torch tensor built on that device (same distribution, torch's generator)."""
    if device is None:
        rng = np.random.default_rng(seed)
        base = (100 + 500 * rng.random(P)).astype(np.float32)
        trend = (1 - 0.2 * np.arange(T) / max(T, 1)).astype(np.float32)
        Y = np.empty((P, T), np.float32, order="F")
        c = np.zeros(P, np.float32)
        decay = np.float32(np.exp(-1.0 / tau))
        for j in range(T):
            ev = rng.random(P) < n_spike
            c = c * decay + ev * (300 * rng.random(P)).astype(np.float32)
            Y[:, j] = base * trend[j] + c + rng.normal(0, 8, P).astype(np.float32)
        return Y
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    base = 100 + 500 * torch.rand(P, generator=g, device=device)
    Yt = torch.empty((T, P), dtype=torch.float32, device=device)  # row j = frame j
    c = torch.zeros(P, device=device)
    decay = float(np.exp(-1.0 / tau))
    for j in range(T):
        ev = torch.rand(P, generator=g, device=device) < n_spike
        c = c * decay + ev * 300 * torch.rand(P, generator=g, device=device)
        Yt[j] = base * (1 - 0.2 * j / max(T, 1)) + c + 8 * torch.randn(P, generator=g, device=device)
    return Yt.T  # (P, T), column-major
