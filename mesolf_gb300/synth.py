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
           "Workload", "config1", "config2", "small_config", "fortran32"]


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
