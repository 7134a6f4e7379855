"""CPU oracle for the MesoLF light-field projector and phase-space Richardson-Lucy solve.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``mesolf_gb300``) imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference legs use it, and only as the checker.

It is an FP64 numpy restatement of the reference's own formulation, written against
the MATLAB sources (paths relative to the reference project root):

* ``src/recon/recon_theory_phase_space_LFM_with_filter.m`` (the RL solve, view
  weights, NIP filter bank, spiral order, projectors, update, ``sample_filter``),
* ``src/recon/gen_phasespace_PSF_theory.m`` (phase-space PSF realignment),
* ``src/recon/conv2FFT.m`` (FFT 'same' convolution),
* ``src/recon/forwardProjectACC.m`` / ``forwardProjectGPU.m`` (full LFM forward),
* ``src/cuda/mex_lfm_convolution_vec.cu`` (MEX projector, semantics only).

Everything is computed in the reference's formulation (full-resolution ``conv2 'same'``
followed by lenslet sampling, sparse up-sampling followed by ``conv2 'same'``), NOT in
the polyphase form that the CUDA kernels use, so the kernels' index algebra is checked
independently.

PARITY: the MEX projector's semantics (``lfm_conv_vec``) are pinned to the reference's own
kernel: ``oracle/refbuild.py`` compiles ``src/cuda/mex_lfm_convolution_vec.cu`` unchanged
(texture fetches stood in for by plain loads) and ``tests/test_gpu_ref_mex.py`` runs it on
the reference's own input fixture.  The RL loop and the other MATLAB functions are
PARITY UNPINNED: the reference ships no golden vectors or known-answer tests for them, and
MATLAB/Octave cannot run here.  They are pinned by self-consistency checks (FFT path ==
direct path, literal MATLAB-semantics transcription == closed form, adjointness, flux
conservation) and by committed golden vectors generated from this oracle.

Arrays use MATLAB index order: ``LFIMG[r, c]``, ``X[r, c, z]``, ``H[x, y, a, b, z]``.
All indices in this file are 0-based unless a comment says "1-based".
"""
from __future__ import annotations

import math

import numpy as np
from numpy.lib.stride_tricks import sliding_window_view

__all__ = [
    "matlab_round", "normalize_psf", "im_shift3", "gen_phasespace_psf_literal",
    "gen_phasespace_psf", "phase_space_size", "view_weights", "nip_omegas",
    "nip_filter_bank", "nip_axis_filters", "ex_size", "gen_spiral", "conv2_same_direct",
    "conv2fft", "forward_ps", "backward_ps", "rl_update", "freq_filter",
    "sample_filter", "recon_phase_space", "rl_view_step", "lfm_conv_vec",
    "lfm_conv_vec_points", "forward_project_full", "sample_filter_plane_index",
]


# ----------------------------------------------------------------------------- helpers
def matlab_round(x):
    """MATLAB ``round``: half away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


# ----------------------------------------------------------------------------- a2
def normalize_psf(H, Ht):
    """Per-depth normalisation, ``recon_theory_phase_space_LFM_with_filter.m:13-16``.

    ``H(:,:,:,:,i) = H(:,:,:,:,i) / sum(H(:,:,:,:,i),'all')`` and the same for Ht.
    """
    H = np.asarray(H, dtype=np.float64)
    Ht = np.asarray(Ht, dtype=np.float64)
    sH = H.sum(axis=(0, 1, 2, 3))
    sHt = Ht.sum(axis=(0, 1, 2, 3))
    return H / sH, Ht / sHt


# ----------------------------------------------------------------------------- a3
def phase_space_size(K0, N):
    """``IMGsize`` and the 0-based crop start, ``gen_phasespace_PSF_theory.m:6-8``."""
    S = K0 - ((K0 - N) % (2 * N))
    i1 = int(matlab_round(K0 / 2) - math.trunc(S / 2)) - 1  # 1-based -> 0-based
    return S, i1


def im_shift3(img, SHIFTX, SHIFTY):
    """Literal transcription of ``gen_phasespace_PSF_theory.m:34-57`` (zero-fill shift)."""
    eqtol = 1e-10
    if abs(math.fmod(SHIFTX, 1)) > eqtol or abs(math.fmod(SHIFTY, 1)) > eqtol:
        raise ValueError("SHIFTX and SHIFTY should be integer numbers")
    SX = int(matlab_round(SHIFTX))
    SY = int(matlab_round(SHIFTY))
    xl, yl = img.shape[0], img.shape[1]
    new = np.zeros_like(img)
    if SX >= 0 and SY >= 0:
        new[SX:, SY:] = img[:xl - SX, :yl - SY]
    elif SX >= 0 and SY < 0:
        new[SX:, :yl + SY] = img[:xl - SX, -SY:]
    elif SX < 0 and SY >= 0:
        new[:xl + SX, SY:] = img[-SX:, :yl - SY]
    else:
        new[:xl + SX, :yl + SY] = img[-SX:, -SY:]
    return new


def gen_phasespace_psf_literal(H, Ht):
    """Line-by-line transcription of ``gen_phasespace_PSF_theory.m:1-31``.

    MATLAB's column-major ``reshape`` is reproduced with ``order='F'``; ``permute`` with
    ``transpose``; ``end:-1:1`` with ``[::-1]``.  Slow (python loops) -- small PSFs only.
    """
    H = np.asarray(H, dtype=np.float64)
    Ht = np.asarray(Ht, dtype=np.float64)
    K0, N, Z = H.shape[0], H.shape[2], H.shape[4]
    S = K0 - ((K0 - N) % (2 * N))                                   # :6
    index1 = int(matlab_round(K0 / 2) - math.trunc(S / 2))          # :7 (1-based)
    index2 = int(matlab_round(K0 / 2) + math.trunc(S / 2))          # :8 (1-based)
    Hd = np.zeros((S, S, N, N, Z))
    for z in range(Z):                                              # :10
        LFtmp = np.zeros((S, S, N, N))
        for ii in range(1, N + 1):                                  # :13 (1-based)
            for jj in range(1, N + 1):
                LFtmp[:, :, ii - 1, jj - 1] = im_shift3(
                    H[index1 - 1:index2, index1 - 1:index2, ii - 1, jj - 1, z],
                    ii - (N + 1) / 2, jj - (N + 1) / 2)
        Hd[:, :, :, :, z] = LFtmp
    sz = Hd.shape
    Hd = Hd.reshape((N, sz[0] // N, N, sz[0] // N, N, N, sz[4]), order="F")   # :23
    Hd = Hd.transpose((0, 2, 1, 3, 4, 5, 6))                                  # :24
    Hd = Hd[:, :, :, :, ::-1, ::-1, :]                                        # :25
    Hd = Hd.transpose((0, 1, 4, 2, 5, 3, 6))                                  # :26
    Hd = Hd.reshape((N, N, sz[0], sz[0], sz[4]), order="F").transpose((2, 3, 0, 1, 4))  # :27
    Htc = Ht[index1 - 1:index2, index1 - 1:index2, :, :, :]                   # :31
    return np.ascontiguousarray(Hd), np.ascontiguousarray(Htc)


def gen_phasespace_psf(H, Ht):
    """Closed form of ``gen_phasespace_PSF_theory.m:1-31`` (vectorised).

    ``Hps[p, q, u, v, z] = H[i1+p+u-h, i1+q+v-h, N-1-(p mod N), N-1-(q mod N), z]`` when
    ``0 <= p+u-h < S`` and ``0 <= q+v-h < S`` (zero otherwise), with ``h=(N-1)/2`` and
    ``i1`` the 0-based crop start; ``Htc = Ht[i1:i1+S, i1:i1+S]``.  Equal to the literal
    transcription (checked in the tests).
    """
    H = np.asarray(H, dtype=np.float64)
    Ht = np.asarray(Ht, dtype=np.float64)
    K0, N, Z = H.shape[0], H.shape[2], H.shape[4]
    S, i1 = phase_space_size(K0, N)
    h = (N - 1) // 2
    p = np.arange(S)
    Hps = np.zeros((S, S, N, N, Z))
    src_ab = N - 1 - (p % N)
    for u in range(N):
        rp = p + u - h
        vr = (rp >= 0) & (rp < S)
        rr = np.clip(rp, 0, S - 1) + i1
        for v in range(N):
            rq = p + v - h
            vq = (rq >= 0) & (rq < S)
            cc = np.clip(rq, 0, S - 1) + i1
            vals = H[rr[:, None], cc[None, :], src_ab[:, None], src_ab[None, :], :]
            vals = vals * (vr[:, None] & vq[None, :])[:, :, None]
            Hps[:, :, u, v, :] = vals
    Htc = Ht[i1:i1 + S, i1:i1 + S, :, :, :].copy()
    return Hps, Htc


def phasespace_view(H, Ht, u, v):
    """``Hps(:,:,u,v,:)`` and ``Htc(:,:,u,v,:)`` of the normalised PSF pair for one view
    (0-based), without materialising the full 5-D arrays (same closed form as
    :func:`gen_phasespace_psf`, per-depth sums as :func:`normalize_psf`)."""
    K0, N, Z = H.shape[0], H.shape[2], H.shape[4]
    S, i1 = phase_space_size(K0, N)
    h = (N - 1) // 2
    sH = np.array([np.asarray(H[:, :, :, :, z], np.float64).sum() for z in range(Z)])
    sHt = np.array([np.asarray(Ht[:, :, :, :, z], np.float64).sum() for z in range(Z)])
    p = np.arange(S)
    src_ab = N - 1 - (p % N)
    rp, rq = p + u - h, p + v - h
    vr, vq = (rp >= 0) & (rp < S), (rq >= 0) & (rq < S)
    rr, cc = np.clip(rp, 0, S - 1) + i1, np.clip(rq, 0, S - 1) + i1
    hv = np.asarray(H[rr[:, None], cc[None, :], src_ab[:, None], src_ab[None, :], :], np.float64)
    hv = hv * (vr[:, None] & vq[None, :])[:, :, None] / sH
    tv = np.asarray(Ht[i1:i1 + S, i1:i1 + S, u, v, :], np.float64) / sHt
    return hv, tv


# ----------------------------------------------------------------------------- a4
def view_weights(Hps):
    """View weights, ``recon_theory_phase_space_LFM_with_filter.m:20,30-38``."""
    return view_weights_from_sums(Hps.sum(axis=(0, 1, 4)))        # :30 sum over x, y, z


def view_sums(H):
    """Per-view sums of ``Hps`` over x, y and z (the input of ``:31-38``) for the per-depth
    normalised ``H`` of ``:13-16``, computed from the raw ``H`` without building ``Hps``: the
    closed form of :func:`gen_phasespace_psf` puts ``H[r, c, a, b, z]`` at view ``(u, v)``
    exactly when ``r = i1 + p + u - h`` for a ``p`` in ``[0, S)`` with ``p mod N = N-1-a``
    and ``p + u - h`` in ``[0, S)`` (likewise ``c``), so each sum is a masked sum of the raw
    planes divided by the plane's total.  Equals ``Hps.sum(axis=(0, 1, 4))``."""
    K0, N, Z = H.shape[0], H.shape[2], H.shape[4]
    S, i1 = phase_space_size(K0, N)
    h = (N - 1) // 2
    mask = np.zeros((N, K0, N))                  # mask[u, r, a]
    for u in range(N):
        for p in range(S):
            if 0 <= p + u - h < S:
                mask[u, i1 + p + u - h, N - 1 - (p % N)] = 1.0
    out = np.zeros((N, N))
    for z in range(Z):
        Hz = np.asarray(H[:, :, :, :, z], dtype=np.float64)                 # (r, c, a, b)
        tot = Hz.sum()
        rows = np.einsum("ura,rcab->ucb", mask, Hz, optimize=True)         # (u, c, b)
        out += np.einsum("ucb,vcb->uv", rows, mask, optimize=True) / tot
    return out


def view_weights_from_sums(sums):
    """``:31-38`` applied to the per-view sums of ``Hps`` over x, y and z."""
    weight_cut = 0.2
    with np.errstate(invalid="ignore", divide="ignore"):
        w = np.array(sums, dtype=np.float64)
        w[np.isnan(w)] = 0                               # :31
        w = w / w.sum()                                  # :32
        w = w - w.min()                                  # :33
        w = w / w.max()                                  # :36
        w[w < weight_cut] = 0                            # :37 (NaN < 0.2 is false)
        w = w * 0.3                                      # :38
    return w


# ----------------------------------------------------------------------------- a5
def nip_omegas(Z, N, variant="base"):
    """``omega_NIP_array`` of ``recon_theory_phase_space_LFM_with_filter.m:21-26,54-56``.

    ``variant="peeling"``: ``…_with_filter_simple_peeling.m:55-58`` takes ``floor(Z/3)``
    rounded DOWN to even instead of ``ceil(Z/3)`` rounded up."""
    omega_NIP = N - 7
    if variant == "peeling":
        R = Z // 3
        if R % 2 == 1:
            R -= 1
    else:
        R = int(math.ceil(Z / 3))
        if R % 2 == 1:
            R += 1
    nb = 3 * R
    axis = np.arange(1, nb + 1, dtype=np.float64) - nb / 2
    om = omega_NIP * np.exp(-(axis / 100.0 * 2 * np.sqrt(np.log(2))) ** 2)
    om[om < 0.2] = 0.2
    return om


def nip_filter_bank(size_h, size_w, Z, N, variant="base"):
    """Literal filter bank, ``recon_theory_phase_space_LFM_with_filter.m:44-61``.

    ``F_i = |fftshift(fft2(exp(-((xx/w_i)^2+(yy/w_i)^2))))| / max`` on the grid
    ``x=(1:size_h)-size_h/2``, ``y=(1:size_w)-size_w/2``.  Returns (size_h, size_w, 3R).
    """
    om = nip_omegas(Z, N, variant)
    x = np.arange(1, size_h + 1, dtype=np.float64) - size_h / 2
    y = np.arange(1, size_w + 1, dtype=np.float64) - size_w / 2
    yy, xx = np.meshgrid(y, x)
    F = np.zeros((size_h, size_w, om.size))
    for i, w in enumerate(om):
        g = np.exp(-((xx / w) ** 2 + (yy / w) ** 2))
        buf = np.abs(np.fft.fftshift(np.fft.fft2(g)))
        F[:, :, i] = buf / buf.max()
    return F


def nip_axis_filters(size_h, size_w, Z, N):
    """Separable factors of the filter bank: ``F_i = fftshift(ax_i[:,None] * ay_i[None,:])``.

    The Gaussian is separable, so ``|fft2(g)| = |fft(gx)| (x) |fft(gy)|`` and the max is the
    product of the 1-D maxima.  Returned UNSHIFTED (frequency 0 first), each normalised
    to max 1.  Used to cross-check the literal bank.
    """
    om = nip_omegas(Z, N)
    x = np.arange(1, size_h + 1, dtype=np.float64) - size_h / 2
    y = np.arange(1, size_w + 1, dtype=np.float64) - size_w / 2
    ax = np.zeros((om.size, size_h))
    ay = np.zeros((om.size, size_w))
    for i, w in enumerate(om):
        a = np.abs(np.fft.fft(np.exp(-(x / w) ** 2)))
        b = np.abs(np.fft.fft(np.exp(-(y / w) ** 2)))
        ax[i] = a / a.max()
        ay[i] = b / b.max()
    return ax, ay


def sample_filter_plane_index(Z, nb):
    """For each plane (0-based) the 0-based filter-bank index, or -1 if the plane is
    passed through; ``recon_theory_phase_space_LFM_with_filter.m:224-231``."""
    half_z = int(matlab_round(Z / 2))
    idx = np.full(Z, -1, dtype=np.int64)
    for z1 in range(1, Z + 1):                           # 1-based plane index
        if z1 >= half_z - nb / 2 + 1 and z1 <= half_z + nb / 2:
            idx[z1 - 1] = int(z1 - half_z + nb / 2) - 1
    return idx


# ----------------------------------------------------------------------------- a7
def ex_size(xsize, S):
    """FFT grid, ``recon_theory_phase_space_LFM_with_filter.m:78-82``."""
    mmid = S // 2
    out = []
    for n in xsize:
        e = n + mmid
        out.append(int(min(2 ** math.ceil(math.log2(e)), 128 * math.ceil(e / 128))))
    return tuple(out)


# ----------------------------------------------------------------------------- a8
def gen_spiral(Nnum):
    """Literal transcription of ``gen_spiral``, ``…_with_filter.m:156-188``.

    Returns 1-based (i_index, j_index) as MATLAB does.  ``mode(Nnum)`` of a scalar is the
    scalar itself, so the ``== 0`` branch never fires for Nnum > 0.
    """
    if Nnum == 0:
        loop_n = Nnum / 2
    else:
        loop_n = (Nnum + 1) / 2
    loop_n = int(loop_n) if float(loop_n).is_integer() else int(math.floor(loop_n))
    i_index = np.zeros(Nnum * Nnum, dtype=np.int64)
    j_index = np.zeros(Nnum * Nnum, dtype=np.int64)
    start = 1
    for k in range(1, loop_n + 1):
        cs = Nnum - 2 * (k - 1)
        bias = k - 1
        if cs > 1:
            i_new = np.concatenate([np.arange(1, cs + 1), cs * np.ones(cs - 1, dtype=np.int64),
                                    np.arange(cs - 1, 0, -1), np.ones(cs - 2, dtype=np.int64)])
            j_new = np.concatenate([np.ones(cs, dtype=np.int64), np.arange(2, cs + 1),
                                    cs * np.ones(cs - 1, dtype=np.int64), np.arange(cs - 1, 1, -1)])
            n = 4 * (cs - 1)
            i_index[start - 1:start - 1 + n] = i_new + bias
            j_index[start - 1:start - 1 + n] = j_new + bias
            start += n
        else:
            i_index[start - 1] = 1 + bias
            j_index[start - 1] = 1 + bias
    return i_index, j_index


# ----------------------------------------------------------------------------- a10
def conv2_same_direct(x, m):
    """MATLAB ``conv2(x, m, 'same')`` for odd-sized m, by direct summation (FP64)."""
    x = np.asarray(x, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    Sx, Sy = m.shape
    mx, my = Sx // 2, Sy // 2
    xp = np.zeros((x.shape[0] + Sx - 1, x.shape[1] + Sy - 1))
    xp[mx:mx + x.shape[0], my:my + x.shape[1]] = x
    win = sliding_window_view(xp, (Sx, Sy))
    return np.einsum("ijpq,pq->ij", win, m[::-1, ::-1], optimize=True)


def conv2fft(x, m, exsize):
    """Transcription of ``conv2FFT.m:1-22`` with ``exindex(...,'circular')`` and
    ``zeroPad`` (``:246-280``): pad both to ``exsize``, circularly re-centre the kernel
    so its ``floor(size/2)`` element sits at the origin, multiply spectra, crop."""
    x = np.asarray(x, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    E = tuple(int(e) for e in exsize)
    xs = x.shape
    mmid = (m.shape[0] // 2, m.shape[1] // 2)
    xp = np.zeros(E)
    xp[:xs[0], :xs[1]] = x
    mp = np.zeros(E)
    mp[:m.shape[0], :m.shape[1]] = m
    r_idx = (np.arange(mmid[0] + 1, mmid[0] + E[0] + 1) - 1) % E[0]   # exindex circular
    c_idx = (np.arange(mmid[1] + 1, mmid[1] + E[1] + 1) - 1) % E[1]
    m1 = mp[np.ix_(r_idx, c_idx)]
    y = np.real(np.fft.ifft2(np.fft.fft2(xp) * np.fft.fft2(m1)))
    return y[:xs[0], :xs[1]]


# ----------------------------------------------------------------------------- a9
def forward_ps(h_uv, X, N):
    """``forwardProjectGPU_phasespace_theory`` (``…_with_filter.m:243-249``; CPU twin
    ``:191-198``): ``P = sum_z conv2(X_z, h_z, 'same')``, sampled at ``(N+1)/2:N:end``.

    Only the sampled outputs are evaluated, each by a direct FP64 dot product.
    """
    X = np.asarray(X, dtype=np.float64)
    h_uv = np.asarray(h_uv, dtype=np.float64)
    Xr, Xc, Z = X.shape
    S = h_uv.shape[0]
    m = S // 2
    c0 = (N + 1) // 2 - 1
    hf = h_uv[::-1, ::-1, :]
    out = np.zeros(((Xr - c0 + N - 1) // N, (Xc - c0 + N - 1) // N))
    Xp = np.zeros((Xr + 2 * m, Xc + 2 * m))
    for z in range(Z):
        Xp[m:m + Xr, m:m + Xc] = X[:, :, z]
        win = sliding_window_view(Xp, (S, S))[c0::N, c0::N]                # (Li, Lj, S, S)
        out += np.einsum("ijpq,pq->ij", win, hf[:, :, z])
    return out


# ----------------------------------------------------------------------------- a12/a13
def backward_ps(t_uv, R, u, v, N):
    """``backwardProjectGPU_phasespace_theory`` (``…_with_filter.m:211-220``; CPU twin
    ``:201-208``): ``B = 0; B(u:N:end, v:N:end) = R; C_z = conv2(B, t_z, 'same')``.

    ``u, v`` are 0-based.  B is non-zero only on the lattice, so ``conv2`` is evaluated as
    a scatter of shifted kernel copies -- exact FP64.
    """
    t_uv = np.asarray(t_uv, dtype=np.float64)
    R = np.asarray(R, dtype=np.float64)
    Li, Lj = R.shape
    S, Z = t_uv.shape[0], t_uv.shape[2]
    m = S // 2
    Xr, Xc = Li * N, Lj * N
    Cp = np.zeros((Xr + S - 1, Xc + S - 1, Z))
    for i in range(Li):
        r0 = u + N * i
        for j in range(Lj):
            val = R[i, j]
            if val != 0.0:
                c0 = v + N * j
                Cp[r0:r0 + S, c0:c0 + S, :] += val * t_uv
    return Cp[m:m + Xr, m:m + Xc, :]


# ----------------------------------------------------------------------------- a14
def rl_update(X, C, D, w, d_eps=0.0):
    """Multiplicative update, ``…_with_filter.m:130-137``.  ``d_eps=1e-10`` is the peeling
    variant's ``Xguess .* XguessCor ./ (buf + 1e-10)`` (``…_simple_peeling.m:149``)."""
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        Xc = X * C / (D + d_eps)
    Xc[np.isnan(Xc)] = 0
    Xc[np.isinf(Xc)] = 0
    Xc[Xc < 0] = 0
    Xn = Xc * w + (1 - w) * X
    Xn[Xn < 0] = 0
    return Xn


# ----------------------------------------------------------------------------- a15
def freq_filter(image, filt):
    """``freq_filter``, ``…_with_filter.m:251-254``."""
    image_f = np.fft.fftshift(np.fft.fft2(image))
    return np.real(np.fft.ifft2(np.fft.ifftshift(image_f * filt)))


def sample_filter(X, F):
    """``sample_filter``, ``…_with_filter.m:222-240`` (flux-preserving low-pass)."""
    X = np.asarray(X, dtype=np.float64)
    Z = X.shape[2]
    nb = F.shape[2]
    idx = sample_filter_plane_index(Z, nb)
    out = X.copy()
    for z in range(Z):
        if idx[z] >= 0:
            img = X[:, :, z]
            s0 = img.sum()
            buf = freq_filter(img, F[:, :, idx[z]])
            sb = buf.sum()
            # :233 divides by sum(buf); for an all-zero plane that is 0/0 = NaN in MATLAB.
            # Kept as zero here (and in the CUDA filter): planes underflow to exact zero in
            # FP32 long before FP64, and a NaN plane would poison every later iteration.
            out[:, :, z] = s0 * buf / sb if sb != 0 else 0.0
    return out


# ----------------------------------------------------------------------------- a1
def _ratio(LF_sub, HX):
    with np.errstate(invalid="ignore", divide="ignore"):
        R = LF_sub / HX
    R[~np.isfinite(R)] = 0
    return R


def rl_view_step(X, LFIMG, Hps, Htc, u, v, w, N, d_eps=0.0):
    """One view of the inner loop (``…_with_filter.m:109-137``), 0-based (u, v)."""
    HX = forward_ps(Hps[:, :, u, v, :], X, N)
    R = _ratio(LFIMG[u::N, v::N], HX)
    C = backward_ps(Htc[:, :, u, v, :], R, u, v, N)
    D = backward_ps(Htc[:, :, u, v, :], np.ones_like(R), u, v, N)
    return rl_update(X, C, D, w, d_eps)


def recon_phase_space(LFIMG, H, Ht, maxIter, X0=None, callback=None, view_step=None, variant="base"):
    """``recon_theory_phase_space_LFM_with_filter`` (``…_with_filter.m:10-151``), FP64.

    ``X0`` (optional) replaces the flat initial guess of ``:72-73`` (warm start).
    ``callback(it, X)`` is called after each iteration's ``sample_filter``.
    ``view_step(h_uv, t_uv, LFIMG, X, u, v, w, N)`` (optional) replaces ``rl_view_step``
    with an equivalent implementation (the C/OpenMP port in ``oracle/mlf_oracle.c``), so
    that large fixtures can be generated in reasonable time.
    """
    LFIMG = np.asarray(LFIMG, dtype=np.float64)
    Hn, Htn = normalize_psf(H, Ht)                                   # :13-16
    Hps, Htc = gen_phasespace_psf(Hn, Htn)                           # :17
    N = Hps.shape[2]
    w = view_weights(Hps)                                            # :20-40
    F = nip_filter_bank(LFIMG.shape[0], LFIMG.shape[1], Hps.shape[4], N, variant)   # :44-61
    d_eps = 1e-10 if variant == "peeling" else 0.0
    Z = Hps.shape[4]
    if X0 is None:
        X = np.ones((LFIMG.shape[0], LFIMG.shape[1], Z))
        X = X / X.sum() * LFIMG.sum()                                # :72-73
    else:
        X = np.asarray(X0, dtype=np.float64).copy()
    i_idx, j_idx = gen_spiral(N)                                     # :95
    for it in range(maxIter):                                        # :98
        for u2 in range(1, N + 1):
            for v2 in range(1, N + 1):
                u = i_idx[(u2 - 1) * N + v2 - 1] - 1
                v = j_idx[(u2 - 1) * N + v2 - 1] - 1
                if w[u, v] == 0:
                    continue
                if view_step is None:
                    X = rl_view_step(X, LFIMG, Hps, Htc, u, v, w[u, v], N, d_eps)
                else:
                    X = view_step(Hps[:, :, u, v, :], Htc[:, :, u, v, :], LFIMG, X, u, v, w[u, v], N)
        X = sample_filter(X, F)                                      # :142
        if callback is not None:
            callback(it, X)
    return X


# ----------------------------------------------------------------------------- a16
PEEL_MASK_RATIO = 0.1     # …_simple_peeling.m:32
PEEL_REDUCE_RATIO = 0.9   # …_simple_peeling.m:33


def recon_phase_space_peeling(LFIMG, H, Ht, maxIter):
    """``recon_theory_phase_space_LFM_with_filter_simple_peeling`` (``…_simple_peeling.m:13-266``),
    FP64.  Returns ``(Xguess, LFIMG_peeled, proj_sensor)``.

    As written the reference normalises ``size(H, 5)`` planes before ``H`` exists (:22) and
    cuts weights at an undefined ``weight_cut`` (:44); this restatement normalises every
    plane of ``H_origin`` / ``Ht_origin`` and uses the base solver's cut, 0.2
    (``…_with_filter.m:20``).  The two RL runs differ from the base solver by the
    ``floor``-rounded filter bank (:55-58) and ``D + 1e-10`` (:149).  Peeling (:183-205): the
    top plane of the first run and its >10 %-of-max mask are forward-projected with the
    normalised H (``forwardProjectGPU``, :330-348); the projection is scaled so that its
    mask-weighted sum matches the image's, 0.9 of it is subtracted from the image (clamped
    at 0), the second run starts again from the flat guess, and its top plane is replaced by
    the first run's (:262).
    """
    LFIMG = np.asarray(LFIMG, dtype=np.float64)
    Hn, _ = normalize_psf(H, Ht)
    X1 = recon_phase_space(LFIMG, H, Ht, maxIter, variant="peeling")
    top = X1[:, :, 0].copy()
    dummy = np.zeros_like(X1)
    dummy[:, :, 0] = top
    mask = np.zeros_like(X1)
    mask[:, :, 0] = top > top.max() * PEEL_MASK_RATIO
    proj = forward_project_full(Hn, dummy)
    projm = forward_project_full(Hn, mask)
    projm = projm / projm.sum()
    proj = proj * (projm * LFIMG).sum() / (projm * proj).sum()
    LF2 = LFIMG - proj * PEEL_REDUCE_RATIO
    LF2[LF2 < 0] = 0
    X2 = recon_phase_space(LF2, H, Ht, maxIter, variant="peeling")
    X2[:, :, 0] = top
    return X2, LF2, proj


# ----------------------------------------------------------------------------- a18
def _conv_vec_padded(bitmap, kw):
    """Zero-pad a (W, H, n) bitmap by kw//2 so that reference edge clipping
    (``mex_lfm_convolution_vec.cu:55-78``) becomes plain zero padding.

    For even kw the reference's ``kernel_end`` clip never reaches the last input column /
    row (``bitmap_endx = x + kw/2 + 1``), so those are zeroed to keep its semantics."""
    W, Hh, n = bitmap.shape
    hk = kw // 2
    b = np.asarray(bitmap, dtype=np.float64).copy()
    if kw % 2 == 0:
        b[W - 1, :, :] = 0
        b[:, Hh - 1, :] = 0
    P = np.zeros((W + kw, Hh + kw, n))
    P[hk:hk + W, hk:hk + Hh, :] = b
    return P


def lfm_conv_vec(bitmap, kernels):
    """Semantics of ``mex_lfm_convolution_vec`` (``src/cuda/mex_lfm_convolution_vec.cu``
    ``:43-266`` kernel, ``:276-421`` host), FP64.

    ``out(x, y, i) = sum_{kx,ky} in(x+kx-kw/2, y+ky-kw/2, i) * K(kx, ky, x mod 15, y mod 15)``
    (0-based; ``kw/2`` integer division), zero outside the bitmap.  ``bitmap`` is (W, H)
    or (W, H, n); ``kernels`` is (kw, kw, 15, 15).  Small shapes only.
    """
    bm = np.asarray(bitmap, dtype=np.float64)
    squeeze = bm.ndim == 2
    if squeeze:
        bm = bm[:, :, None]
    K = np.asarray(kernels, dtype=np.float64)
    kw = K.shape[0]
    nk = K.shape[2]
    W, Hh, n = bm.shape
    P = _conv_vec_padded(bm, kw)
    out = np.zeros((W, Hh, n))
    win = sliding_window_view(P, (kw, kw), axis=(0, 1))              # (W+1, H+1, n, kw, kw)
    for px in range(nk):
        for py in range(nk):
            xs = np.arange(px, W, nk)
            ys = np.arange(py, Hh, nk)
            if xs.size == 0 or ys.size == 0:
                continue
            sub = win[px:W:nk, py:Hh:nk]                              # (|xs|, |ys|, n, kw, kw)
            out[np.ix_(xs, ys)] = np.einsum("xyipq,pq->xyi", sub, K[:, :, px, py], optimize=True)
    return out[:, :, 0] if squeeze else out


def mex_slot_overlap_kernels(kernels):
    """The kernel set the reference MEX kernel computes with when, on every kernel row, its
    out-of-range fill group wins the shared-memory race (``src/cuda/mex_lfm_convolution_vec.cu``
    ``:114-117,130,139-141,161-182``).

    Each row the 1024 threads copy one row of all 15 kernels of the output row's phase into
    15 shared slots of ``kw`` floats; thread group ``g = t // 15`` copies elements
    ``[kw*g//68, kw*(g+1)//68)`` of slot ``t % 15``.  Group 68 (threads 1020-1023, slots 0-3)
    gets ``[kw, kw + kw//68)``: it writes the first ``kw//68`` elements of the NEXT slot with
    the next row's first elements of its own kernel, while group 0 writes the same cells of
    slots 1-4 with their proper values, with no barrier between the two.  So for
    ``a = x mod 15`` in 1..4 and ``kx < kw//68`` the tap used is either ``K(kx, ky, a, b)``
    or, if group 68 stored last, flat element ``kw*kw*(a-1 + 15 b) + kw*(ky+1) + kx`` of the
    kernel array (``K(kx, ky+1, a-1, b)``; for the last row the next kernel's first row).
    This returns the kernel set of the second outcome for every row; ``lfm_conv_vec`` with
    it gives that outcome's output.  For ``kw < 68`` nothing overlaps and the set is
    ``kernels`` itself."""
    K = np.asarray(kernels)
    kw = K.shape[0]
    nover = kw // 68
    out = K.copy()
    if nover == 0:
        return out
    flat = np.asfortranarray(K).reshape(-1, order="F")
    for b in range(K.shape[3]):
        for a in range(1, 5):
            base = kw * kw * (a - 1 + K.shape[2] * b)
            for ky in range(kw):
                for kx in range(nover):
                    out[kx, ky, a, b] = flat[base + kw * (ky + 1) + kx]
    return out


def lfm_conv_vec_points(bitmap, kernels, pts):
    """``lfm_conv_vec`` evaluated only at the (x, y, i) triples ``pts`` -- for large
    shapes where the full FP64 evaluation is too slow."""
    bm = np.asarray(bitmap, dtype=np.float64)
    if bm.ndim == 2:
        bm = bm[:, :, None]
    K = np.asarray(kernels, dtype=np.float64)
    kw = K.shape[0]
    nk = K.shape[2]
    P = _conv_vec_padded(bm, kw)
    out = np.empty(len(pts))
    for t, (x, y, i) in enumerate(pts):
        out[t] = np.sum(P[x:x + kw, y:y + kw, i] * K[:, :, x % nk, y % nk])
    return out


# ----------------------------------------------------------------------------- a17
def forward_project_full(H, vol, CAindex=None):
    """Full LFM forward projector, ``forwardProjectACC.m:1-18`` / ``forwardProjectGPU.m``:
    ``out = sum_{a,b,z} conv2(vol_z .* 1[(a,b) phase], H(:,:,a,b,z), 'same')``.

    ``CAindex`` (Z x 2, 1-based inclusive, as in ``forwardProjectACC``) crops the PSF per
    plane; None uses the whole PSF (``forwardProjectGPU``).  FFT evaluation in FP64.
    """
    H = np.asarray(H, dtype=np.float64)
    vol = np.asarray(vol, dtype=np.float64)
    N = H.shape[2]
    Xr, Xc, Z = vol.shape
    out = np.zeros((Xr, Xc))
    for z in range(Z):
        if CAindex is not None:
            lo, hi = int(CAindex[z][0]) - 1, int(CAindex[z][1])
            Hz = H[lo:hi, lo:hi, :, :, z]
        else:
            Hz = H[:, :, :, :, z]
        S = Hz.shape[0]
        m = S // 2
        E = (Xr + S - 1, Xc + S - 1)
        acc = np.zeros((E[0], E[1] // 2 + 1), dtype=np.complex128)
        for a in range(N):
            for b in range(N):
                ts = np.zeros((Xr, Xc))
                ts[a::N, b::N] = vol[a::N, b::N, z]
                if not ts.any():
                    continue
                acc += np.fft.rfft2(ts, E) * np.fft.rfft2(Hz[:, :, a, b], E)
        full = np.fft.irfft2(acc, E)
        out += full[m:m + Xr, m:m + Xc]
    return out


def forward_project_discrete(H, vol, unique_array, max_PSF_size):
    """``forwardProjectGPU_discrete.m:1-20``: plane cc projected with PSF plane
    ``unique_array(cc)`` (1-based), cropped to ``ceil(end/2) -/+ floor(max_PSF_size/2)``."""
    H = np.asarray(H, dtype=np.float64)
    K0 = H.shape[0]
    half = int(max_PSF_size) // 2
    c = int(math.ceil(K0 / 2))                      # 1-based centre
    lo, hi = c - half - 1, c + half                 # 0-based [lo, hi)
    out = 0.0
    for cc, u in enumerate(np.ravel(unique_array)):
        Hz = H[lo:hi, lo:hi, :, :, int(u) - 1:int(u)]
        out = out + forward_project_full(Hz, np.asarray(vol, dtype=np.float64)[:, :, cc:cc + 1])
    return out


def forward_project_skip_2d(H, img, step, cc):
    """``forwardProjectGPU_skip_2D.m:1-16``: 2-D image, PSF plane ``cc`` (1-based), phases
    ``aa, bb = 1:step:Nnum`` only."""
    H = np.asarray(H, dtype=np.float64)
    N = H.shape[2]
    img = np.asarray(img, dtype=np.float64)
    Xr, Xc = img.shape
    S = H.shape[0]
    m = S // 2
    E = (Xr + S - 1, Xc + S - 1)
    acc = np.zeros((E[0], E[1] // 2 + 1), dtype=np.complex128)
    for a in range(0, N, int(step)):
        for b in range(0, N, int(step)):
            ts = np.zeros((Xr, Xc))
            ts[a::N, b::N] = img[a::N, b::N]
            acc += np.fft.rfft2(ts, E) * np.fft.rfft2(H[:, :, a, b, int(cc) - 1], E)
    return np.fft.irfft2(acc, E)[m:m + Xr, m:m + Xc]


# ----------------------------------------------------------------------------- f3 summary image
def movmean(x, k, axis=-1):
    """MATLAB ``movmean`` / ``smoothdata(..., 'movmean', k)`` with shrinking end windows:
    the window of element i spans ``i - floor(k/2)`` .. ``i + k - 1 - floor(k/2)`` (for even k
    it is centred on the current and previous elements).  Each window is summed directly
    (left to right), with no running-sum cancellation."""
    x = np.moveaxis(np.asarray(x, dtype=np.float64), axis, -1)
    n = x.shape[-1]
    before = min(int(k) // 2, n - 1)
    after = min(int(k) - 1 - int(k) // 2, n - 1)
    s = np.zeros_like(x)
    cnt = np.zeros(n)
    for d in range(-before, after + 1):
        lo, hi = max(0, -d), min(n, n - d)
        s[..., lo:hi] += x[..., lo + d:hi + d]
        cnt[lo:hi] += 1
    return np.moveaxis(s / cnt, -1, axis)


def rank_1_factorization(Y, maxIter=1, divisor=1.0):
    """``rank_1_factorization.m:32-45``: Y ~ bg_spatial * bg_temporal (pixels x frames)."""
    Y = np.asarray(Y, dtype=np.float64)
    s = np.ones(Y.shape[0]) / np.sqrt(Y.shape[0])
    t = None
    for it in range(1, maxIter + 1):
        t = (s @ Y) / divisor
        t = t / np.linalg.norm(t)
        s = (Y @ t) / divisor
        if it < maxIter:
            s = s / np.linalg.norm(s)
    return s, t


def compute_std_image(Y, y1=None, y2=None):
    """``compute_std_image.m:22-26`` as written:
    ``sqrt((A - y1.^2)/length(y2) - B.^2 + 2*B.*y1*C - y1.^2*C^2)`` with A = sum(Y.^2, 2),
    B = mean(Y, 2), C = mean(y2).  A negative radicand (possible through the expansion) gives
    a complex value in MATLAB; it is clamped to 0 here."""
    Y = np.asarray(Y, dtype=np.float64)
    if y1 is None:
        y1 = np.zeros(Y.shape[0])
        y2 = np.zeros(Y.shape[1])
    A = (Y ** 2).sum(axis=1)
    B = Y.mean(axis=1)
    C = np.mean(y2)
    v = (A - y1 ** 2) / len(y2) - B ** 2 + 2 * B * y1 * C - y1 ** 2 * C ** 2
    return np.sqrt(np.maximum(v, 0.0))


def summary_image(movie, mode="pixelwise", bg_iter=5, window_1=100, window_2=20, poly_index=3):
    """``summary_image_generation_module.m:43-133`` on a (pixels x frames) movie: returns
    ``(summary_image / max(summary_image), bg_spatial, bg_temporal)``.  Defaults are
    ``mesolf_set_params.m:120-132``.  'global' (``:43-61``): Y = movie / max, rank-1 (s, t)
    with divisor 1, compute_std_image(Y, s, t).  'pixelwise' (``:62-97``): rank-1 of the raw
    movie with the max as divisor; per pixel y = movie / max, y - movmean(y, window_1),
    movmean(., window_2), .^poly_index, compute_std_image with zero backgrounds.  The global
    mode's Savitzky-Golay baseline (``:46-50``) only feeds a plot and is not computed."""
    Y = np.asarray(movie, dtype=np.float64)
    M = Y.max()
    if mode == "global":
        Yn = Y / M
        s, t = rank_1_factorization(Yn, bg_iter)
        img = compute_std_image(Yn, s, t)
    elif mode == "pixelwise":
        s, t = rank_1_factorization(Y, bg_iter, M)
        y = Y / M
        z = y - movmean(y, window_1, axis=1)
        z = movmean(z, window_2, axis=1) ** poly_index
        img = compute_std_image(z)
    else:
        raise ValueError('Invalid value for param "detrend_mode"')
    return img / img.max(), s, t


# ----------------------------------------------------------------------------- f4 rectification
def matlab_round(x):
    """MATLAB ``round``: half away from zero."""
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def matlab_colon(a, d, b):
    """MATLAB ``a:d:b`` for a non-zero double step: a + k*d for k = 0 .. floor((b-a)/d), with a
    relative tolerance of 1e-10 on the count (MATLAB's colon also tolerates rounding at the end
    point; its exact rule is not published, so end points within that tolerance are unpinned)."""
    q = (b - a) / d
    if q < -1e-10 * max(1.0, abs(q)):
        return np.zeros(0)
    n = int(np.floor(q + 1e-10 * max(1.0, abs(q)))) + 1
    return a + d * np.arange(n, dtype=np.float64)


def rectify_axis(center, lo, hi, M, dx):
    """One axis of the rectification grid (``image_load_module_aug.m:130-143`` with
    lo = -dx/M, hi = size + 0.9; ``determine_patch_info_aug.m:50-68`` with lo = 1, hi = size):
    ``R = [fliplr(center:-dx/M:lo), center+dx/M:dx/M:hi]``, the 1-based index of ``center`` in
    R, the left cut ``qinit = mod(idx - floor(M/2), M)`` and the kept query vector
    ``R(qinit+1:end)``.  Returns ``(R, idx, qinit, Rq)``."""
    s = dx / M
    left = matlab_colon(center, -s, lo)[::-1]
    right = matlab_colon(center + s, s, hi)
    R = np.concatenate([left, right])
    idx = len(left)                       # find(R == center), 1-based
    c0 = idx - M // 2
    qinit = c0 - M * int(np.floor(c0 / M))
    return R, idx, qinit, R[qinit:]


def interp2_linear(img, yq, xq):
    """``griddedInterpolant({1:H, 1:W}, img)`` evaluated on the grid (yq, xq): bilinear with
    linear extrapolation (the interpolant's default method and extrapolation), 1-based
    coordinates.  Every query uses the cell [i, i+1] x [j, j+1] with i = floor(y) clamped to
    [1, H-1] (and j likewise), so that outside the samples the boundary cell extends linearly."""
    img = np.asarray(img, dtype=np.float64)
    H, W = img.shape
    if H < 2 or W < 2:
        raise ValueError("griddedInterpolant needs at least 2 samples per dimension")
    yq = np.asarray(yq, np.float64)
    xq = np.asarray(xq, np.float64)
    i = np.clip(np.floor(yq), 1, H - 1).astype(np.int64)
    j = np.clip(np.floor(xq), 1, W - 1).astype(np.int64)
    fy = (yq - i)[:, None]
    fx = (xq - j)[None, :]
    v00 = img[i - 1][:, j - 1]
    v10 = img[i][:, j - 1]
    v01 = img[i - 1][:, j]
    v11 = img[i][:, j]
    return (1 - fy) * ((1 - fx) * v00 + fx * v01) + fy * ((1 - fx) * v10 + fx * v11)


def img_rectify_mod(img, x_center, y_center, M, dx):
    """``image_load_module_aug.m:126-164``: resample a raw patch onto the lenslet-aligned grid
    of pitch dx/M (query grids from ``rectify_axis`` with lo = -dx/M, hi = size + 0.9), then cut
    the right / bottom to whole lenslets."""
    H, W = np.shape(img)
    _, _, _, xq = rectify_axis(x_center, -dx / M, W + 0.9, M, dx)
    _, _, _, yq = rectify_axis(y_center, -dx / M, H + 0.9, M, dx)
    out = interp2_linear(img, yq, xq)
    return out[:M * (out.shape[0] // M), :M * (out.shape[1] // M)]


def image_load(frames, patch_info, SI):
    """``image_load_module_aug.m:19-123`` on frames already in memory (``frames`` H x W x n,
    MATLAB order, the files in ``dir`` order; the TIFF reading is out of scope): frame
    selection ``frames_start:frames_step:min(n, frames_end)``, mean of ``frames_step``
    consecutive frames when ``frames_average`` (the last group may be shorter), cut to
    ``raw_cut``, rectification, and division by the movie max.  Returns (pixels, frames)."""
    frames = np.asarray(frames)
    n_files = frames.shape[2]
    start, step = int(SI.get("frames_start", 1)), int(SI.get("frames_step", 1))
    end = SI.get("frames_end", np.inf)
    last = int(min(n_files, end))
    if SI.get("frames_average", True):
        navg = step
        idx = np.arange(start, last + 1)
    else:
        navg = 1
        idx = np.arange(start, last + 1, step)
    n_final = len(np.arange(start, last + 1, step))
    (ys, ye), (xs, xe) = np.asarray(patch_info["raw_cut"], dtype=np.int64)
    h, w = (int(v) for v in patch_info["size"])
    M = int(SI["Nnum"])
    out = np.empty((h * w, n_final), dtype=np.float64)
    for i in range(n_final):
        sel = idx[i * navg:min((i + 1) * navg, len(idx))]
        patch = frames[ys - 1:ye, xs - 1:xe, sel - 1].astype(np.float64).mean(axis=2)
        r = img_rectify_mod(patch, patch_info["raw_cut_xCenter"], patch_info["raw_cut_yCenter"], M,
                            float(SI["frames_dx"]))
        if r.shape != (h, w):
            raise ValueError("After raw patch read and rectification, the shape is different from what was expected.")
        out[:, i] = r.reshape(-1, order="F")
    return out / out.max()


def determine_patch_info(SI, frame_shape):
    """``determine_patch_info_aug.m:12-290`` (no plotting): the rectified full-frame size from
    the grids (lo = 1, hi = size), the lenslet-border crop, the patches ('carpet' or 'roi'),
    and for each patch its raw cut and the lenslet centre inside the cut.  ``frame_shape`` is
    the (rows, cols) of the first frame.  Returns a list of dicts with keys location (2x2,
    1-based [top, left; bottom, right]), size, raw_cut (2x2: [y0, y1; x0, x1]),
    raw_cut_xCenter, raw_cut_yCenter."""
    Hf, Wf = (int(v) for v in frame_shape)
    M = int(SI["Nnum"])
    dx = float(SI["frames_dx"])
    xC, yC = float(SI["frames_x_offset"]), float(SI["frames_y_offset"])
    cut = list(SI.get("frames_crop_border_microlenses", [0, 0, 0, 0]))
    XcutLeft, XcutRight, YcutUp, YcutDown = cut[0], cut[1], cut[2], cut[3]
    Xr, pre_cx, XqInit, Xq = rectify_axis(xC, 1.0, float(Wf), M, dx)
    Yr, pre_cy, YqInit, Yq = rectify_axis(yC, 1.0, float(Hf), M, dx)
    size_y, size_x = M * (len(Yq) // M), M * (len(Xq) // M)
    XsizeML, YsizeML = size_x // M, size_y // M
    if XcutLeft + XcutRight >= XsizeML:
        raise ValueError("X-cut range is larger than the x-size of image")
    if YcutUp + YcutDown >= YsizeML:
        raise ValueError("Y-cut range is larger than the y-size of image")
    Xrange = np.arange(1 + XcutLeft, XsizeML - XcutRight + 1)
    Yrange = np.arange(1 + YcutUp, YsizeML - YcutDown + 1)
    gh, gw = len(Yrange) * M, len(Xrange) * M
    patches = []
    mode = SI.get("patch_mode", "carpet")

    def add(top_left, bottom_right):
        ph = bottom_right[0] - top_left[0] + 1
        pw = bottom_right[1] - top_left[1] + 1
        ph -= ph % M
        pw -= pw % M
        if ph < 50 or pw < 50:
            return
        patches.append({"location": np.array([[top_left[0], top_left[1]],
                                              [top_left[0] + ph - 1, top_left[1] + pw - 1]]),
                        "size": (int(ph), int(pw))})

    if mode == "carpet":
        n = SI.get("n_patches", 1)
        n = [n, n] if np.isscalar(n) else list(n)
        psh = int(np.ceil((gh // n[0]) / M)) * M
        psw = int(np.ceil((gw // n[1]) / M)) * M
        for k in range(n[0] * n[1]):
            ci, cj = k % n[0] + 1, k // n[0] + 1          # ind2sub, column-major
            tl = [(ci - 1) * psh + 1, (cj - 1) * psw + 1]
            br = [min(ci * psh, gh), min(cj * psw, gw)]
            add(tl, br)
    elif mode == "roi":
        rps = int(SI["ROI_patch_size"])
        rps -= rps % M
        for roi in np.atleast_2d(np.asarray(SI["ROI_list"])):
            tl0, br0 = [int(roi[0]), int(roi[1])], [int(roi[2]), int(roi[3])]
            rs = [br0[0] - tl0[0] + 1, br0[1] - tl0[1] + 1]
            nh, nw = int(np.ceil(rs[0] / rps)), int(np.ceil(rs[1] / rps))
            sh_, sw_ = rps, rps
            if rs[0] < rps:
                sh_, nh = rs[0], 1
            if rs[1] < rps:
                sw_, nw = rs[1], 1
            for k in range(nh * nw):
                ci, cj = k % nh + 1, k // nh + 1
                tl = [(ci - 1) * sh_ + tl0[0], (cj - 1) * sw_ + tl0[1]]
                br = [min(ci * sh_, rs[0]) + tl0[0] - 1, min(cj * sw_, rs[1]) + tl0[1] - 1]
                add(tl, br)
    else:
        raise ValueError("patch_mode should be either 'carpet' or 'roi'")
    Y_after_top = (Yrange[0] - 1) * M + 1
    X_after_left = (Xrange[0] - 1) * M + 1
    margin = int(np.ceil(M / 2)) - 2
    for p in patches:
        (top, left), (bottom, right) = p["location"]
        pt = top + Y_after_top - 1 + YqInit - 1 - margin
        pl = left + X_after_left - 1 + XqInit - 1 - margin
        pb = bottom + Y_after_top - 1 + YqInit - 1 + margin - 1
        pr = right + X_after_left - 1 + XqInit - 1 + margin - 1
        for v, R in ((pt, Yr), (pb, Yr), (pl, Xr), (pr, Xr)):
            if v < 1 or v > len(R):
                raise IndexError("Index exceeds the number of array elements")
        y0 = max(int(np.floor(Yr[pt - 1])), 1)
        y1 = min(int(np.ceil(Yr[pb - 1])), Hf)
        x0 = max(int(np.floor(Xr[pl - 1])), 1)
        x1 = min(int(np.ceil(Xr[pr - 1])), Wf)
        cy = int(matlab_round((pt + pb) / 2))
        cx = int(matlab_round((pl + pr) / 2))
        my = (pre_cy - cy) % M
        mx = (pre_cx - cx) % M
        yc = Yr[cy - (M - my) - 1] if my >= int(np.ceil(M / 2)) else Yr[cy + my - 1]
        xc = Xr[cx - (M - mx) - 1] if mx >= int(np.ceil(M / 2)) else Xr[cx + mx - 1]
        p["raw_cut"] = np.array([[y0, y1], [x0, x1]])
        p["raw_cut_yCenter"] = float(yc - Yr[pt - 1])
        p["raw_cut_xCenter"] = float(xc - Xr[pl - 1])
    return patches
