"""Pins of the CPU oracle (no GPU).

The reference ships no golden vectors for this path and cannot run here (no MATLAB; its
MEX uses removed texture references), so the oracle is pinned by self-consistency:
literal MATLAB-semantics transcriptions against closed forms, FFT path against direct
sums, adjointness, flux conservation.
"""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth


@pytest.mark.parametrize("K0,Z", [(61, 2), (45, 2), (75, 1), (91, 1)])
def test_phasespace_closed_form_matches_literal(K0, Z):
    z = np.arange(Z) - Z // 2
    H, Ht = synth.make_psf(K0, 15, z, seed=3)
    Hn, Htn = R.normalize_psf(H, Ht)
    A, At = R.gen_phasespace_psf_literal(Hn, Htn)
    B, Bt = R.gen_phasespace_psf(Hn, Htn)
    assert A.shape == B.shape
    np.testing.assert_array_equal(A, B)
    np.testing.assert_array_equal(At, Bt)


def test_phase_space_size():
    # gen_phasespace_PSF_theory.m:6-8 for the workloads' PSF sides
    assert R.phase_space_size(61, 15) == (45, 8)
    assert R.phase_space_size(231, 15) == (225, 3)
    assert R.phase_space_size(255, 15) == (255, 0)
    assert R.phase_space_size(241, 15)[0] == 225


def test_normalize_sums_to_one():
    H, Ht = synth.make_psf(61, 15, [-2, 0, 3], seed=1)
    Hn, Htn = R.normalize_psf(H, Ht)
    np.testing.assert_allclose(Hn.sum(axis=(0, 1, 2, 3)), 1.0, rtol=1e-13)
    np.testing.assert_allclose(Htn.sum(axis=(0, 1, 2, 3)), 1.0, rtol=1e-13)


def test_spiral_order():
    i, j = R.gen_spiral(15)
    pairs = list(zip(i.tolist(), j.tolist()))
    assert len(set(pairs)) == 225 and min(i) == 1 and max(i) == 15
    # outer ring: down the first column, along the last row, up the last column, back
    assert pairs[:15] == [(k, 1) for k in range(1, 16)]
    assert pairs[15:29] == [(15, k) for k in range(2, 16)]
    assert pairs[29:43] == [(k, 15) for k in range(14, 0, -1)]
    assert pairs[43:56] == [(1, k) for k in range(14, 1, -1)]
    assert pairs[-1] == (8, 8)
    i3, j3 = R.gen_spiral(3)
    assert list(zip(i3, j3)) == [(1, 1), (2, 1), (3, 1), (3, 2), (3, 3), (2, 3), (1, 3), (1, 2), (2, 2)]


@pytest.mark.parametrize("shape,S", [((60, 45), 45), ((33, 50), 15), ((165, 165), 45)])
def test_conv2fft_equals_direct(shape, S):
    rng = np.random.default_rng(0)
    x = rng.random(shape)
    m = rng.random((S, S))
    d = R.conv2_same_direct(x, m)
    f = R.conv2fft(x, m, R.ex_size(shape, S))
    assert np.abs(d - f).max() <= 1e-12 * np.abs(d).max()


def test_exsize():
    assert R.ex_size((165, 165), 45) == (256, 256)
    assert R.ex_size((1005, 1005), 225) == (1152, 1152)


def test_filter_bank_separable_and_omegas():
    F = R.nip_filter_bank(45, 30, 5, 15)
    ax, ay = R.nip_axis_filters(45, 30, 5, 15)
    for i in range(F.shape[2]):
        np.testing.assert_allclose(F[:, :, i], np.fft.fftshift(np.outer(ax[i], ay[i])), atol=1e-15)
    om = R.nip_omegas(51, 15)
    assert om.size == 54 and om.max() == 8.0 and om.min() > 6.5
    assert R.nip_omegas(21, 15).size == 24


def test_sample_filter_flux_and_plane_map():
    rng = np.random.default_rng(1)
    X = rng.random((45, 30, 7)) + 0.1
    F = R.nip_filter_bank(45, 30, 7, 15)
    Y = R.sample_filter(X, F)
    np.testing.assert_allclose(Y.sum(axis=(0, 1)), X.sum(axis=(0, 1)), rtol=1e-12)
    idx = R.sample_filter_plane_index(7, F.shape[2])
    assert (idx >= 0).all()
    # planes outside the bank's range pass through (a deep stack, a narrow bank)
    idx2 = R.sample_filter_plane_index(40, 6)
    assert (idx2 < 0).sum() == 34 and list(idx2[idx2 >= 0]) == list(range(6))


def test_sample_filter_odd_size_shift_convention():
    """fftshift / ifftshift are not inverses of each other's roles for odd sizes; the
    composition used by freq_filter must equal filtering by ifftshift(F)."""
    rng = np.random.default_rng(2)
    img = rng.random((15, 9))
    F = rng.random((15, 9))
    a = R.freq_filter(img, F)
    b = np.real(np.fft.ifft2(np.fft.fft2(img) * np.fft.ifftshift(F)))
    np.testing.assert_allclose(a, b, atol=1e-13)


def test_forward_backward_adjoint_center_view():
    """With Ht = rot180(Hps) per slice, the backward projector of the centre view is the
    adjoint of the forward projector (which samples at the lenslet centre)."""
    rng = np.random.default_rng(4)
    N, S, Z, L = 15, 45, 3, 4
    h = rng.random((S, S, Z))
    t = h[::-1, ::-1, :]
    X = rng.random((L * N, L * N, Z))
    Rimg = rng.random((L, L))
    c = (N - 1) // 2
    lhs = np.sum(R.forward_ps(h, X, N) * Rimg)
    rhs = np.sum(X * R.backward_ps(t, Rimg, c, c, N))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_forward_ps_matches_fft_formulation():
    rng = np.random.default_rng(5)
    N, S, Z = 15, 45, 2
    h = rng.random((S, S, Z))
    X = rng.random((60, 75, Z))
    E = R.ex_size((60, 75), S)
    P = sum(R.conv2fft(X[:, :, z], h[:, :, z], E) for z in range(Z))
    ref = P[7::N, 7::N]
    np.testing.assert_allclose(R.forward_ps(h, X, N), ref, rtol=1e-11)


def test_backward_ps_matches_fft_formulation():
    rng = np.random.default_rng(6)
    N, S, Z = 15, 45, 2
    t = rng.random((S, S, Z))
    Rimg = rng.random((4, 5))
    u, v = 3, 11
    B = np.zeros((60, 75))
    B[u::N, v::N] = Rimg
    E = R.ex_size((60, 75), S)
    ref = np.stack([R.conv2fft(B, t[:, :, z], E) for z in range(Z)], axis=2)
    np.testing.assert_allclose(R.backward_ps(t, Rimg, u, v, N), ref, rtol=1e-10, atol=1e-13)


def test_rl_update_semantics():
    X = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    C = np.array([1.0, np.nan, 1.0, -1.0, 0.0])
    D = np.array([2.0, 1.0, 0.0, 1.0, 0.0])
    out = R.rl_update(X, C, D, 0.3)
    # 0.5*w + (1-w)*1 ; NaN->0 ; Inf->0 ; negative->0 ; 0/0 -> NaN -> 0
    np.testing.assert_allclose(out, [0.3 * 0.5 + 0.7, 0.7 * 2, 0.7 * 3, 0.7 * 4, 0.7 * 5])


def test_conv_vec_semantics_small():
    """lfm_conv_vec against a literal per-pixel loop of the MEX kernel's clipping logic
    (mex_lfm_convolution_vec.cu:55-78,147-251)."""
    rng = np.random.default_rng(7)
    for W, Hh, n, kw in [(20, 17, 2, 7), (16, 31, 1, 6), (15, 15, 1, 1)]:
        bm = rng.random((W, Hh, n))
        K = rng.random((kw, kw, 15, 15))
        got = R.lfm_conv_vec(bm, K)
        ref = np.zeros_like(bm)
        for i in range(n):
            for y in range(Hh):
                for x in range(W):
                    sx, sy = x - kw // 2, y - kw // 2
                    ksx = -sx if sx < 0 else 0
                    ksy = -sy if sy < 0 else 0
                    kex = kw - max(0, x + kw // 2 + 1 - W)
                    key = kw - max(0, y + kw // 2 + 1 - Hh)
                    acc = 0.0
                    for ky in range(ksy, key):
                        for kx in range(ksx, kex):
                            acc += bm[sx + kx, sy + ky, i] * K[kx, ky, x % 15, y % 15]
                    ref[x, y, i] = acc
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)


def test_rl_view_step_flux_and_positivity():
    w = synth.small_config(lenslets=(4, 3), K0=61, Z=3)
    H, Ht = w.psf()
    vol = w.volume()
    LF = w.measured(H, vol)
    X = R.recon_phase_space(LF, H, Ht, 1)
    assert X.shape == (60, 45, 3)
    assert np.isfinite(X).all() and (X >= 0).all()


def test_c_port_matches_numpy_oracle():
    """The C/OpenMP port used for the CPU baseline agrees with the numpy oracle."""
    from oracle import cbuild
    rng = np.random.default_rng(9)
    N, S, Z = 15, 45, 3
    h = rng.random((S, S, Z))
    t = rng.random((S, S, Z))
    X = rng.random((60, 75, Z))
    LF = rng.random((60, 75)) * 100
    np.testing.assert_allclose(cbuild.forward(h, X, N), R.forward_ps(h, X, N), rtol=1e-12)
    Rimg = rng.random((4, 5))
    np.testing.assert_allclose(cbuild.backward(t, Rimg, 3, 11, N), R.backward_ps(t, Rimg, 3, 11, N),
                               rtol=1e-12, atol=1e-14)
    ref = R.rl_view_step(X, LF, h[:, :, None, None, :].repeat(15, 2).repeat(15, 3),
                         t[:, :, None, None, :].repeat(15, 2).repeat(15, 3), 3, 11, 0.3, N)
    np.testing.assert_allclose(cbuild.view_step(h, t, LF, X, 3, 11, 0.3, N), ref, rtol=1e-11)


def test_full_forward_equals_interleaved_phase_space_views():
    """a17 through the phase-space operator: forwardProjectGPU.m's sum over (a, b, z) of
    conv2(vol_z .* phase(a, b), H(:,:,a,b,z), 'same') equals, pixel (u + N i, v + N j),
    view (u, v)'s phase-space forward projection at lenslet (i, j) with the per-plane
    normalised PSF times the plane sums of H (PSF inside the crop)."""
    w = synth.small_config(lenslets=(3, 2), K0=61, Z=3)
    H, Ht = w.psf()
    vol = np.random.default_rng(1).random((45, 30, 3))
    full = R.forward_project_full(H, vol)
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, _ = R.gen_phasespace_psf(Hn, Htn)
    sums = H.astype(np.float64).sum(axis=(0, 1, 2, 3))
    lf = np.zeros_like(full)
    for u in range(15):
        for v in range(15):
            lf[u::15, v::15] = R.forward_ps(Hps[:, :, u, v, :], vol * sums, 15)
    assert np.abs(lf - full).max() <= 1e-12 * np.abs(full).max()


def test_sample_filter_zero_plane_stays_zero():
    """An all-zero plane is passed as zeros (the reference's 0/0 would be NaN)."""
    F = R.nip_filter_bank(30, 45, 5, 15)
    X = np.random.default_rng(0).random((30, 45, 5))
    X[:, :, 2] = 0.0
    Y = R.sample_filter(X, F)
    assert np.isfinite(Y).all() and not Y[:, :, 2].any()
    assert np.allclose(Y[:, :, 1].sum(), X[:, :, 1].sum())


def test_peeling_filter_bank_rounds_down():
    """…_simple_peeling.m:55-58: floor(Z/3) rounded down to even (base: ceil, up)."""
    assert R.nip_omegas(51, 15).size == 54 and R.nip_omegas(51, 15, "peeling").size == 48
    assert R.nip_omegas(21, 15).size == 24 and R.nip_omegas(21, 15, "peeling").size == 18
    assert R.nip_omegas(7, 15, "peeling").size == 6


def test_phase_space_kept_mask_matches_impulses():
    """The crop-and-shift region of gen_phasespace_PSF_theory.m: a unit PSF pixel inside the
    mask projects identically through the phase-space operator and the full sum; one outside
    is lost."""
    from mesolf_gb300.api import phase_space_kept_mask
    K0, N = 61, 15
    keep = phase_space_kept_mask(K0, N)
    vol = np.random.default_rng(0).random((90, 90, 1))   # every PSF offset lands inside
    for (i, j, a, b) in [(8, 30, 7, 3), (15, 30, 0, 3), (14, 30, 0, 3), (52, 40, 7, 7), (46, 30, 14, 2),
                         (45, 30, 14, 2), (30, 7, 5, 7), (30, 53, 5, 7)]:
        H = np.zeros((K0, K0, N, N, 1))
        H[i, j, a, b, 0] = 1.0
        full = R.forward_project_full(H, vol)
        Hps, _ = R.gen_phasespace_psf(H, H[::-1, ::-1])
        lf = np.zeros_like(full)
        for u in range(N):
            for v in range(N):
                lf[u::N, v::N] = R.forward_ps(Hps[:, :, u, v, :], vol, N)
        same = np.abs(lf - full).max() <= 1e-9 * max(1.0, np.abs(full).max())
        assert same == bool(keep[i, j, a, b]), (i, j, a, b)


@pytest.mark.parametrize("W,H,kw", [(31, 46, 16), (40, 33, 7), (47, 52, 21)])
def test_mex_correlation_equals_forward_projection_of_reindexed_kernels(W, H, kw):
    """The identity behind the tensor-core route of the MEX projector: the correlation with
    the kernel slot taken from the output pixel's phase (mex_lfm_convolution_vec.cu:43-266)
    equals the full forward projection (forwardProjectGPU.m, PSF slice from the source
    pixel's phase) of H'[d][psi] = K[c-d+hk][(psi-(c-d)) mod 15], embedded in K0 = 15 + 30m
    >= kw + 14, on the bitmap zero-padded to multiples of 15 (last row / column zeroed for
    even kw) -- and so equals the interleaved phase-space views of H'."""
    rng = np.random.default_rng(kw)
    bm = rng.random((W, H))
    K = rng.random((kw, kw, 15, 15))
    ref = R.lfm_conv_vec(bm, K)
    K0 = 15
    while K0 < kw + 14:
        K0 += 30
    c, hk = (K0 - 1) // 2, kw // 2
    Hp = np.zeros((K0, K0, 15, 15, 1))
    for dx in range(K0):
        kx = c - dx + hk
        if not 0 <= kx < kw:
            continue
        for dy in range(K0):
            ky = c - dy + hk
            if not 0 <= ky < kw:
                continue
            ps = (np.arange(15) - (c - dx)) % 15
            qs = (np.arange(15) - (c - dy)) % 15
            Hp[dx, dy, :, :, 0] = K[kx, ky][np.ix_(ps, qs)]
    b = bm.copy()
    if kw % 2 == 0:
        b[W - 1, :] = 0
        b[:, H - 1] = 0
    Wp, Hq = -(-W // 15) * 15, -(-H // 15) * 15
    bp = np.zeros((Wp, Hq, 1))
    bp[:W, :H, 0] = b
    out = R.forward_project_full(Hp, bp)[:W, :H]
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_movmean_matches_matlab_window_rule():
    x = np.arange(10, dtype=float)
    # k = 4 (even): window of element i is [i-2, i+1], shrunk at the ends
    assert np.allclose(R.movmean(x, 4), [np.mean(x[max(0, i - 2):i + 2]) for i in range(10)])
    # k = 3 (odd): [i-1, i+1]
    assert np.allclose(R.movmean(x, 3), [np.mean(x[max(0, i - 1):i + 2]) for i in range(10)])


def test_summary_image_std_and_rank1():
    rng = np.random.default_rng(0)
    mov = rng.random((50, 300)) + np.linspace(0, 1, 300)[None, :]
    img, s, t = R.summary_image(mov, "pixelwise", bg_iter=2, window_1=40, window_2=5, poly_index=2)
    assert img.shape == (50,) and np.isclose(img.max(), 1.0) and (img >= 0).all()
    assert np.isclose(np.linalg.norm(t), 1.0)
    # rank-1 fit of an exact rank-1 matrix recovers its factors' directions
    a, b = rng.random(30), rng.random(80)
    s1, t1 = R.rank_1_factorization(np.outer(a, b), 3)
    assert np.allclose(np.abs(s1 / np.linalg.norm(s1)), a / np.linalg.norm(a))
    assert np.allclose(np.abs(t1), b / np.linalg.norm(b))


def test_summary_image_known_answers():
    # pixels with a linear ramp: the moving mean of a ramp equals the ramp away from the ends
    # (odd window), so the detrended series is zero there; a constant pixel has zero std
    T = 200
    ramp = np.arange(T, dtype=float)
    mov = np.stack([1 + 0 * ramp, 5 + 0.01 * ramp, 3 + np.sin(ramp / 7)])
    img, _, _ = R.summary_image(mov, "pixelwise", bg_iter=1, window_1=11, window_2=1, poly_index=1)
    assert img[0] < 1e-12 and img[2] == 1.0 and 0 < img[1] < 0.1
    # compute_std_image as written (not the residual std of Y - s t)
    Y = np.outer(np.arange(1, 5.0), np.ones(7))
    s, t = R.rank_1_factorization(Y, 1)
    A, B, C = (Y ** 2).sum(1), Y.mean(1), t.mean()
    v = (A - s ** 2) / 7 - B ** 2 + 2 * B * s * C - s ** 2 * C ** 2
    assert (v < 0).any()  # the expansion can go negative: MATLAB gives a complex value, 0 here
    assert np.allclose(R.compute_std_image(Y, s, t), np.sqrt(np.maximum(v, 0)))
